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
