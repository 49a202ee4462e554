// Instantiations of the FP32 lane kernel (gx_lane.cuh), part c: classes
// (11|20), (12|01), (12|10), (20|02), (20|11), (20|20), (21|01), (21|10), (22|00).
#include "gx_lane.cuh"

namespace gx {

cudaError_t launch_lane32_c(int la, int lb, int lc, int ld, const EriDev& d, const QuartetClass& qc,
                               cudaStream_t s, bool* found) {
    *found = true;
    const int key = ((la * 3 + lb) * 3 + lc) * 3 + ld;
    switch (key) {
#define GX_CASE(A, B, C, D)                                                                     \
    case ((A * 3 + B) * 3 + C) * 3 + D:                                                         \
        lane::lane32_kernel<A, B, C, D><<<(qc.ngroup + 3) / 4, 128, 0, s>>>(d, qc);             \
        return cudaGetLastError();
        GX_CASE(1, 1, 2, 0)
        GX_CASE(1, 2, 0, 1)
        GX_CASE(1, 2, 1, 0)
        GX_CASE(2, 0, 0, 2)
        GX_CASE(2, 0, 1, 1)
        GX_CASE(2, 0, 2, 0)
        GX_CASE(2, 1, 0, 1)
        GX_CASE(2, 1, 1, 0)
        GX_CASE(2, 2, 0, 0)
#undef GX_CASE
        default:
            *found = false;
            return cudaSuccess;
    }
}

}  // namespace gx
