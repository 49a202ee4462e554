// Instantiations and dispatch of the register-resident small-class kernel
// (all (la, lb, lc, ld) with la + lb + lc + ld <= 2).
#include "gx_small.cuh"

namespace gx {

namespace {
template <int A, int B, int C, int D>
cudaError_t go(const EriDev& d, const QuartetClass& qc, cudaStream_t s) {
    // one warp per task group, four warps per block
    small::small_kernel<A, B, C, D><<<(qc.ngroup + 3) / 4, 128, 0, s>>>(d, qc);
    return cudaGetLastError();
}
}  // namespace

bool small_class(int la, int lb, int lc, int ld) { return la + lb + lc + ld <= 2; }

cudaError_t launch_lane32_a(int la, int lb, int lc, int ld, const EriDev& d, const QuartetClass& qc, cudaStream_t s,
                            bool* found);
cudaError_t launch_lane32_b(int la, int lb, int lc, int ld, const EriDev& d, const QuartetClass& qc, cudaStream_t s,
                            bool* found);
cudaError_t launch_lane32_c(int la, int lb, int lc, int ld, const EriDev& d, const QuartetClass& qc, cudaStream_t s,
                            bool* found);

// (L = 5 classes were measured too: at 235-255 registers with spills the
// lane kernel lost to the generic kernel on every one of them)
bool lane32_class(int la, int lb, int lc, int ld) {
    const int L = la + lb + lc + ld;
    return L >= 3 && L <= 4 && la <= 2 && lb <= 2 && lc <= 2 && ld <= 2;
}

cudaError_t launch_lane32(int la, int lb, int lc, int ld, const EriDev& d, const QuartetClass& qc, cudaStream_t s) {
    if (qc.ntask <= 0 || qc.ngroup <= 0) return cudaSuccess;
    bool found = false;
    cudaError_t e = launch_lane32_a(la, lb, lc, ld, d, qc, s, &found);
    if (!found) e = launch_lane32_b(la, lb, lc, ld, d, qc, s, &found);
    if (!found) e = launch_lane32_c(la, lb, lc, ld, d, qc, s, &found);
    return found ? e : cudaErrorInvalidValue;
}

cudaError_t launch_small(int la, int lb, int lc, int ld, const EriDev& d, const QuartetClass& qc, cudaStream_t s) {
    if (qc.ntask <= 0 || qc.ngroup <= 0) return cudaSuccess;
    const int key = ((la * 3 + lb) * 3 + lc) * 3 + ld;
    switch (key) {
#define GX_CASE(A, B, C, D) \
    case ((A * 3 + B) * 3 + C) * 3 + D: return go<A, B, C, D>(d, qc, s);
        GX_CASE(0, 0, 0, 0)
        GX_CASE(1, 0, 0, 0)
        GX_CASE(0, 1, 0, 0)
        GX_CASE(0, 0, 1, 0)
        GX_CASE(0, 0, 0, 1)
        GX_CASE(2, 0, 0, 0)
        GX_CASE(0, 2, 0, 0)
        GX_CASE(0, 0, 2, 0)
        GX_CASE(0, 0, 0, 2)
        GX_CASE(1, 1, 0, 0)
        GX_CASE(1, 0, 1, 0)
        GX_CASE(1, 0, 0, 1)
        GX_CASE(0, 1, 1, 0)
        GX_CASE(0, 1, 0, 1)
        GX_CASE(0, 0, 1, 1)
#undef GX_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

}  // namespace gx
