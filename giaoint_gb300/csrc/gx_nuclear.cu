// GIAO nuclear-attraction matrix V[mu][nu] = sum_C -Z_C <mu| 1/|r - C| |nu>
// (src/nuclear.cpp:27-170, 207-330 of the reference).
//
// Same formulation as the electron-repulsion kernels: the London phase lives
// in the complex Hermite expansion E~ of the primitive pair (K1 records), so
// per (primitive pair, nucleus)
//   V = -Z (2 pi / p) K_ab sum_K E~_K R^_K(X' = P' - C),
// with R^ the three-index MD table of the complex separation seeded by
// (-2p)^n F_n(p X'.X').  With the pair prefactor F = sqrt(2 pi^{5/2}) K_ab / p
// of the K1 record this is -Z F (2 pi / sqrt(2 pi^{5/2})) sum_K E~_K R^_K.
//
// One warp per ordered segmented shell pair: for every (primitive pair,
// nucleus) lane 0 forms the Boys values and seeds, the warp builds R^ level
// by level (nuclear_rec), and lane l contracts the component pairs ab = l, l+32,
// ... into per-warp accumulators; the block is written once at the end.
#include "gx_internal.h"

namespace gx {

namespace {

// Level-parallel recurrence between columns 0 and 1 (stride 2) of R, level
// 0 ending in column 0.
__device__ void nuclear_rec(int L, const double2* seed, const double2* X, double2* R, const uint32_t* herm_xyz,
                            int lane) {
    int cur = (L % 2 == 0) ? 0 : 1;
    if (lane == 0) R[cur] = seed[L];
    __syncwarp();
    for (int n = L - 1; n >= 0; --n) {
        const int nxt = cur ^ 1;
        const int cnt = herm_count(L - n);
        for (int e = lane; e < cnt; e += 32) {
            double2 v;
            if (e == 0) {
                v = seed[n];
            } else {
                const uint32_t kx = __ldg(&herm_xyz[e]);
                const int k = kx & 255, l = (kx >> 8) & 255, m = (kx >> 16) & 255;
                int axis, pw, i1, i2;
                if (k > 0) {
                    axis = 0, pw = k, i1 = herm_index(k - 1, l, m), i2 = k > 1 ? herm_index(k - 2, l, m) : 0;
                } else if (l > 0) {
                    axis = 1, pw = l, i1 = herm_index(0, l - 1, m), i2 = l > 1 ? herm_index(0, l - 2, m) : 0;
                } else {
                    axis = 2, pw = m, i1 = herm_index(0, 0, m - 1), i2 = m > 1 ? herm_index(0, 0, m - 2) : 0;
                }
                v = cmul(X[axis], R[2 * i1 + cur]);
                if (pw > 1) v = cmacr(v, (double)(pw - 1), R[2 * i2 + cur]);
            }
            R[2 * e + nxt] = v;
        }
        __syncwarp();
        cur = nxt;
    }
}

__global__ void __launch_bounds__(32) nuclear_kernel(BasisDev bs, PairData pp, BoysTable boys, const GLRules* gl,
                                                     const uint32_t* herm_xyz, const PairClassDev* classes,
                                                     const int* pp_class, int nnuc, const double* charge,
                                                     const double* center, const long long* seg_ao, long long n,
                                                     double2* out, DevStatus* status) {
    extern __shared__ double2 nsm[];
    const int lane = threadIdx.x;
    const int ns = bs.ns;
    const int sa = blockIdx.x / ns, sb = blockIdx.x - (blockIdx.x / ns) * ns;
    const int la = bs.l[sa], lb = bs.l[sb];
    const int L = la + lb;
    const int nab = ncart(la) * ncart(lb);
    const int NL = herm_count(L);
    double2* R = nsm;                 // 2 columns x NL
    double2* seed = R + 2 * NL;       // L + 1 seeds, then X'[3]
    double2* acc = seed + L + 4;      // nab accumulators
    for (int i = lane; i < nab; i += 32) acc[i] = c2(0.0, 0.0);
    const int p0 = bs.sp_off[sa * ns + sb];
    const int kab = bs.nprim[sa] * bs.nprim[sb];
    const PairClassDev pc = classes[pp_class[p0]];
    const double scale = 6.283185307179586 / 5.914967172795613;  // 2 pi / sqrt(2 pi^{5/2})
    for (int it = 0; it < kab * nnuc; ++it) {
        const int ip = p0 + it / nnuc, c = it - (it / nnuc) * nnuc;
        const double p = pp.p[ip];
        if (lane == 0) {
            double2 X[3];
            for (int x = 0; x < 3; ++x) X[x] = c2(pp.Pr[3 * ip + x] - center[3 * c + x], pp.Pi[3 * ip + x]);
            const double tre = p * (X[0].x * X[0].x + X[1].x * X[1].x + X[2].x * X[2].x -
                                    (X[0].y * X[0].y + X[1].y * X[1].y + X[2].y * X[2].y));
            const double tim = 2.0 * p * (X[0].x * X[0].y + X[1].x * X[1].y + X[2].x * X[2].y);
            double2 Sh[BOYS_MAX_ORDER + 1], e0;
            if (const int rc = boys_eval(tre, tim, L, boys, gl, Sh, e0)) {
                report(status, rc, blockIdx.x, L, tre, tim);
                e0 = c2(0.0, 0.0);
            }
            double2 s = e0;
            for (int k = 0; k <= L; ++k) {
                seed[k] = cmul(s, Sh[k]);
                s = cscale(s, -2.0 * p);
            }
            for (int x = 0; x < 3; ++x) seed[L + 1 + x] = X[x];
        }
        __syncwarp();
        nuclear_rec(L, seed, seed + L + 1, R, herm_xyz, lane);
        const double2 pref = cscale(pp.F[ip], -charge[c] * scale);
        const double2* E = pp.Epool + pp.Eoff[ip];
        for (int ab = lane; ab < nab; ab += 32) {
            const int bo = pc.boxoff[ab];
            const int bd = pc.boxdim[ab];
            const int nbox = (bd & 255) * ((bd >> 8) & 255) * ((bd >> 16) & 255);
            double2 v = c2(0.0, 0.0);
            for (int e = 0; e < nbox; ++e) {
                const uint32_t ke = pc.ent[bo + e];
                v = cmac(v, E[bo + e], R[2 * herm_index(ke & 255, (ke >> 8) & 255, (ke >> 16) & 255)]);
            }
            acc[ab] = cmac(acc[ab], pref, v);
        }
        __syncwarp();  // R and seed are rewritten by the next entry
    }
    const int ncb = ncart(lb);
    for (int ab = lane; ab < nab; ab += 32) {
        const int ca = ab / ncb, cb = ab - ca * ncb;
        out[(seg_ao[sa] + ca) * n + seg_ao[sb] + cb] = acc[ab];
    }
}

}  // namespace

cudaError_t launch_nuclear(const BasisDev& bs, const PairData& pp, const BoysTable& boys, const GLRules* gl,
                           const uint32_t* herm_xyz, const PairClassDev* classes, const int* pp_class, int nnuc,
                           const double* charge, const double* center, const long long* seg_ao, long long n,
                           int max_pair_L, int max_nab, double2* out, DevStatus* status, cudaStream_t s) {
    const long long blocks = (long long)bs.ns * bs.ns;
    if (blocks == 0) return cudaSuccess;
    const size_t smem = (size_t)(2 * herm_count(max_pair_L) + max_pair_L + 4 + max_nab) * sizeof(double2);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(nuclear_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    nuclear_kernel<<<(unsigned)blocks, 32, smem, s>>>(bs, pp, boys, gl, herm_xyz, classes, pp_class, nnuc, charge,
                                                      center, seg_ao, n, out, status);
    return cudaGetLastError();
}

}  // namespace gx
