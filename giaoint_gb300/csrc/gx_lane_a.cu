// Instantiations of the FP32 lane kernel (gx_lane.cuh), part a: classes
// (00|12), (00|21), (01|02), (01|11), (01|20), (02|01), (02|10), (10|02), (10|11), (10|20), (11|01), (11|10), (12|00), (20|01), (20|10), (21|00).
#include "gx_lane.cuh"

namespace gx {

cudaError_t launch_lane32_a(int la, int lb, int lc, int ld, const EriDev& d, const QuartetClass& qc,
                               cudaStream_t s, bool* found) {
    *found = true;
    const int key = ((la * 3 + lb) * 3 + lc) * 3 + ld;
    switch (key) {
#define GX_CASE(A, B, C, D)                                                                     \
    case ((A * 3 + B) * 3 + C) * 3 + D:                                                         \
        lane::lane32_kernel<A, B, C, D><<<(qc.ngroup + 3) / 4, 128, 0, s>>>(d, qc);             \
        return cudaGetLastError();
        GX_CASE(0, 0, 1, 2)
        GX_CASE(0, 0, 2, 1)
        GX_CASE(0, 1, 0, 2)
        GX_CASE(0, 1, 1, 1)
        GX_CASE(0, 1, 2, 0)
        GX_CASE(0, 2, 0, 1)
        GX_CASE(0, 2, 1, 0)
        GX_CASE(1, 0, 0, 2)
        GX_CASE(1, 0, 1, 1)
        GX_CASE(1, 0, 2, 0)
        GX_CASE(1, 1, 0, 1)
        GX_CASE(1, 1, 1, 0)
        GX_CASE(1, 2, 0, 0)
        GX_CASE(2, 0, 0, 1)
        GX_CASE(2, 0, 1, 0)
        GX_CASE(2, 1, 0, 0)
#undef GX_CASE
        default:
            *found = false;
            return cudaSuccess;
    }
}

}  // namespace gx
