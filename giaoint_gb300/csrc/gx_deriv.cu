// ERI centre derivatives d/dR_{slot,axis} (ab|cd) and magnetic derivatives
// d/dB_b (ab|cd) of London-orbital shell quartets
// (compute_eri_center_derivatives / compute_eri_magnetic_derivatives and
// EriResponses::centers / magnetic, src/derivatives.cpp:53-106, 215-245,
// 268-280, 556-640, 954-966 of the reference).
//
// For a Cartesian primitive with normalisation N(alpha, l) = g(alpha, l) h(l),
//   g(alpha, l) = (2 alpha / pi)^{3/4} (4 alpha)^{|l|/2},
//   h(l)        = prod_x ((2 l_x - 1)!!)^{-1/2},
// the derivative of slot k along axis x is
//   h(l_k) [ Z_k(l_k + 1_x) - l_x D_k(l_k - 1_x)
//            + i phi_k sum_c (B x e_x)_c U_k(l_k + 1_c) ]
//   + i phi_k sum_c (B x e_x)_c R_{k,c} (ab|cd),
// and the field derivative along b is the sum over the four slots of
//   i phi_k sum_c (e_b x (R_k - O))_c [h(l_k) U_k(l_k + 1_c) + R_{k,c} (ab|cd)],
// phi_k = +1/2 on the bra side of a pair (slots 0, 2), -1/2 on the ket side,
// where Z_k, U_k and D_k are contracted integrals with slot k replaced by a
// raw-primitive shell of angular momentum l + 1, l + 1 and l - 1 and
// contraction coefficients w g(alpha, l) 2 alpha, w g(alpha, l) and
// w g(alpha, l).  Those blocks are ordinary ERIs of an extended basis and run
// through the electron-repulsion class kernels; this kernel gathers them into
// the (4, 3, na, nb, nc, nd) blocks of the reference layout.
#include <algorithm>

#include "gx_internal.h"

namespace gx {

namespace {

__device__ __forceinline__ int comp_index(int l, int lx, int lz) {
    const int m = l - lx;
    return m * (m + 1) / 2 + lz;
}

// Component c of a shell of angular momentum l in the reference order
// (x descending, then y descending).
__device__ __forceinline__ void comp_of(int l, int c, int& lx, int& ly, int& lz) {
    int m = 0;
    while ((m + 1) * (m + 2) / 2 <= c) ++m;
    lz = c - m * (m + 1) / 2;
    lx = l - m;
    ly = m - lz;
}

__global__ void __launch_bounds__(256) deriv_combine_kernel(DerivCombineArgs a) {
    const long long total = a.offsets[a.nq];
    const bool centre = a.mode == 0;
    const bool has_u = !centre || a.field;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        // quartet of element e: last i with offsets[i] <= e
        int lo = 0, hi = a.nq - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(&a.offsets[mid]) <= e) lo = mid;
            else hi = mid - 1;
        }
        const int qi = lo;
        int sh[4], l[4], nc[4], dim[4];
        long long size = 1;
        for (int k = 0; k < 4; ++k) {
            sh[k] = (int)__ldg(&a.quartets[4 * qi + k]);
            l[k] = __ldg(&a.shell_l[sh[k]]);
            nc[k] = __ldg(&a.shell_ncontr[sh[k]]);
            dim[k] = nc[k] * ncart(l[k]);
            size *= dim[k];
        }
        const long long rel = e - __ldg(&a.offsets[qi]);
        const int d = (int)(rel / size);
        const long long r0 = rel - (long long)d * size;
        long long r = r0;
        int idx[4];
        for (int j = 3; j >= 0; --j) {
            idx[j] = (int)(r % dim[j]);
            r /= dim[j];
        }
        // this quartet's derived blocks: per slot [Z, D if l > 0] (centre), [U]; then [plain]
        long long off = __ldg(&a.derived_offsets[qi]);
        long long zoff[4], doff[4], uoff[4], boff = -1;
        double uscale[4];  // U = Z / (2 alpha) for a single-primitive shell in centre mode
        for (int j = 0; j < 4; ++j) {
            const long long up = size / dim[j] * (nc[j] * ncart(l[j] + 1));
            zoff[j] = doff[j] = uoff[j] = -1;
            uscale[j] = 1.0;
            if (centre) {
                zoff[j] = off;
                off += up;
                if (l[j] > 0) {
                    doff[j] = off;
                    off += size / dim[j] * (nc[j] * ncart(l[j] - 1));
                }
            }
            const double inv2a = centre ? __ldg(&a.shell_inv2a[sh[j]]) : 0.0;
            if (has_u && inv2a != 0.0) {
                uoff[j] = zoff[j];
                uscale[j] = inv2a;
            } else if (has_u) {
                uoff[j] = off;
                off += up;
            }
        }
        if (has_u) boff = off;
        // linear index of the derived block whose slot k has angular momentum
        // lp and component (px, py, pz), contraction xk
        auto derived = [&](int k, int xk, int lp, int px, int pz) {
            long long li = 0;
            for (int j = 0; j < 4; ++j) {
                const int dj = j == k ? nc[j] * ncart(lp) : dim[j];
                const int ij = j == k ? xk * ncart(lp) + comp_index(lp, px, pz) : idx[j];
                li = li * dj + ij;
            }
            return li;
        };
        double2 res = c2(0.0, 0.0);
        const double2 base = has_u ? __ldg(&a.derived[boff + r0]) : c2(0.0, 0.0);
        // slots contributing: one (centre mode) or all four (magnetic mode)
        const int k0 = centre ? d / 3 : 0, k1 = centre ? d / 3 + 1 : 4;
        for (int k = k0; k < k1; ++k) {
            const int lk = l[k], nck = ncart(lk);
            const int xk = idx[k] / nck, ck = idx[k] - xk * nck;
            int ang[3];
            comp_of(lk, ck, ang[0], ang[1], ang[2]);
            const double hk = __ldg(&a.shell_raw[sh[k]])
                                  ? 1.0
                                  : a.inv_sqrt_df[ang[0]] * a.inv_sqrt_df[ang[1]] * a.inv_sqrt_df[ang[2]];
            const double phi = (k % 2 == 0) ? 0.5 : -0.5;
            double w[3];  // phase derivative: B x e_x (centre) or e_b x (R_k - O) (magnetic)
            if (centre) {
                const int x = d - 3 * k;
                int up[3] = {ang[0], ang[1], ang[2]};
                ++up[x];
                double2 v = __ldg(&a.derived[zoff[k] + derived(k, xk, lk + 1, up[0], up[2])]);
                if (ang[x] > 0) {
                    int dn[3] = {ang[0], ang[1], ang[2]};
                    --dn[x];
                    const double2 t = __ldg(&a.derived[doff[k] + derived(k, xk, lk - 1, dn[0], dn[2])]);
                    v.x -= ang[x] * t.x;
                    v.y -= ang[x] * t.y;
                }
                res = c2(hk * v.x, hk * v.y);
                if (!a.field) break;
                w[0] = x == 2 ? a.B[1] : (x == 1 ? -a.B[2] : 0.0);
                w[1] = x == 0 ? a.B[2] : (x == 2 ? -a.B[0] : 0.0);
                w[2] = x == 1 ? a.B[0] : (x == 0 ? -a.B[1] : 0.0);
            } else {
                const int b = d;
                double D[3];
                for (int c = 0; c < 3; ++c) D[c] = __ldg(&a.shell_center[3 * sh[k] + c]) - a.O[c];
                w[0] = b == 1 ? D[2] : (b == 2 ? -D[1] : 0.0);
                w[1] = b == 2 ? D[0] : (b == 0 ? -D[2] : 0.0);
                w[2] = b == 0 ? D[1] : (b == 1 ? -D[0] : 0.0);
            }
            double2 t = c2(0.0, 0.0);
            for (int c = 0; c < 3; ++c) {
                const double coef = phi * w[c];
                if (coef == 0.0) continue;
                int uc[3] = {ang[0], ang[1], ang[2]};
                ++uc[c];
                const double2 u = __ldg(&a.derived[uoff[k] + derived(k, xk, lk + 1, uc[0], uc[2])]);
                const double R = __ldg(&a.shell_center[3 * sh[k] + c]);
                const double hu = hk * uscale[k];
                // coef * (h U + R base)
                t.x += coef * (hu * u.x + R * base.x);
                t.y += coef * (hu * u.y + R * base.y);
            }
            // + i t
            res.x -= t.y;
            res.y += t.x;
        }
        a.out[e] = res;
    }
}

// d2/dR_{k,r} dB_b (ab|cd) at fixed gauge origin, index (k 3 + r) 3 + b:
//   M0 D0[k,r] + sum_j sum_c i phi_j (e_b x (R_j - O))_c
//                  [h_j Dj[k,r](l_j + 1_c) + delta_jk delta_rc E0]
//   + sum_c i phi_k (e_b x e_r)_c [h_k Ek(l_k + 1_c) + R_{k,c} E0],
// M0 = sum_j sum_c i phi_j (e_b x (R_j - O))_c R_{j,c}; Dj / Ej are the
// centre derivatives / plain blocks of the quartet with slot j replaced by its
// U shell (raw primitives, coefficients w g(alpha, l)), D0 / E0 those of the
// quartet itself.  This is the reference's centre response applied to the
// field response plus the cross term (src/derivatives.cpp:160-181, 232-245),
// regrouped by linearity.
__global__ void __launch_bounds__(256) deriv_mixed_kernel(DerivMixedArgs a) {
    const long long total = a.offsets[a.nq];
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = a.nq - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(&a.offsets[mid]) <= e) lo = mid;
            else hi = mid - 1;
        }
        const int qi = lo;
        int sh[4], l[4], nc[4], dim[4];
        long long size = 1;
        for (int k = 0; k < 4; ++k) {
            sh[k] = (int)__ldg(&a.quartets[4 * qi + k]);
            l[k] = __ldg(&a.shell_l[sh[k]]);
            nc[k] = __ldg(&a.shell_ncontr[sh[k]]);
            dim[k] = nc[k] * ncart(l[k]);
            size *= dim[k];
        }
        const long long rel = e - __ldg(&a.offsets[qi]);
        const int d = (int)(rel / size);
        const long long r0 = rel - (long long)d * size;
        const int k = d / 9, r = (d / 3) % 3, b = d % 3;
        int idx[4], xs[4], ang[4][3];
        double h[4];
        {
            long long t = r0;
            for (int j = 3; j >= 0; --j) {
                idx[j] = (int)(t % dim[j]);
                t /= dim[j];
            }
            for (int j = 0; j < 4; ++j) {
                const int nck = ncart(l[j]);
                xs[j] = idx[j] / nck;
                comp_of(l[j], idx[j] - xs[j] * nck, ang[j][0], ang[j][1], ang[j][2]);
                h[j] = __ldg(&a.shell_raw[sh[j]])
                           ? 1.0
                           : a.inv_sqrt_df[ang[j][0]] * a.inv_sqrt_df[ang[j][1]] * a.inv_sqrt_df[ang[j][2]];
            }
        }
        // linear index of element idx with slot j at component (px, py, pz) of l_j + 1
        auto up_index = [&](int j, int px, int pz) {
            long long li = 0;
            for (int t = 0; t < 4; ++t) {
                const int dt = t == j ? nc[t] * ncart(l[t] + 1) : dim[t];
                const int it = t == j ? xs[t] * ncart(l[t] + 1) + comp_index(l[t] + 1, px, pz) : idx[t];
                li = li * dt + it;
            }
            return li;
        };
        const double2 e0 = __ldg(&a.E[__ldg(&a.eoff[qi]) + r0]);
        const double2 d0 = __ldg(&a.D[0][__ldg(&a.doff[qi]) + (long long)(k * 3 + r) * size + r0]);
        double2 acc = c2(0.0, 0.0);
        double m0 = 0.0;  // M0 = i m0
        for (int j = 0; j < 4; ++j) {
            const double phi = (j % 2 == 0) ? 0.5 : -0.5;
            double D[3], R[3], w[3];
            for (int c = 0; c < 3; ++c) {
                R[c] = __ldg(&a.shell_center[3 * sh[j] + c]);
                D[c] = R[c] - a.O[c];
            }
            w[0] = b == 1 ? D[2] : (b == 2 ? -D[1] : 0.0);
            w[1] = b == 2 ? D[0] : (b == 0 ? -D[2] : 0.0);
            w[2] = b == 0 ? D[1] : (b == 1 ? -D[0] : 0.0);
            const long long sizej = size / dim[j] * (nc[j] * ncart(l[j] + 1));
            const double2* Dj = a.D[1 + j] + __ldg(&a.doff[(long long)(1 + j) * a.nq + qi]) +
                                (long long)(k * 3 + r) * sizej;
            for (int c = 0; c < 3; ++c) {
                const double coef = phi * w[c];
                if (coef == 0.0) continue;
                m0 += coef * R[c];
                int up[3] = {ang[j][0], ang[j][1], ang[j][2]};
                ++up[c];
                const double2 v = __ldg(&Dj[up_index(j, up[0], up[2])]);
                double tx = h[j] * v.x, ty = h[j] * v.y;
                if (j == k && r == c) {
                    tx += e0.x;
                    ty += e0.y;
                }
                // += i coef (tx, ty)
                acc.x -= coef * ty;
                acc.y += coef * tx;
            }
        }
        // + i m0 d0
        acc.x -= m0 * d0.y;
        acc.y += m0 * d0.x;
        {
            // cross term: (e_b x e_r)_c
            const double phi = (k % 2 == 0) ? 0.5 : -0.5;
            double cr[3] = {0.0, 0.0, 0.0};
            if (b != r) {
                const int c = 3 - b - r;  // the remaining axis; sign of the permutation (b, r, c)
                cr[c] = ((b + 1) % 3 == r) ? 1.0 : -1.0;
            }
            const double2* Ek = a.E + __ldg(&a.eoff[(long long)(1 + k) * a.nq + qi]);
            for (int c = 0; c < 3; ++c) {
                const double coef = phi * cr[c];
                if (coef == 0.0) continue;
                int up[3] = {ang[k][0], ang[k][1], ang[k][2]};
                ++up[c];
                const double2 u = __ldg(&Ek[up_index(k, up[0], up[2])]);
                const double Rc = __ldg(&a.shell_center[3 * sh[k] + c]);
                const double tx = h[k] * u.x + Rc * e0.x, ty = h[k] * u.y + Rc * e0.y;
                acc.x -= coef * ty;
                acc.y += coef * tx;
            }
        }
        a.out[e] = acc;
    }
}

// Per-atom contraction of centre derivatives (src/assembly.cpp:87-158), one
// warp per canonical quartet: for every local element and every distinct
// orbit image (identity, pair exchange, conjugate reversal, conjugate
// exchanged reversal) the weight
//   sum P[nu,mu] Q[sig,lam] (Coulomb) + sum P[nu,lam] Q[sig,mu] (exchange)
//   + gamma[mu,nu,lam,sig]
// at the image's AO indices multiplies the derivative (conjugated for the
// last two images); lanes stride over the elements and a fixed shuffle tree
// sums the twelve partial sums, so the result does not depend on scheduling.
__global__ void __launch_bounds__(128) deriv_contract_kernel(DerivContractArgs a) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int perm[4][4] = {{0, 1, 2, 3}, {2, 3, 0, 1}, {1, 0, 3, 2}, {3, 2, 1, 0}};
    const long long n = a.n;
    for (int qi = warp; qi < a.nq; qi += nwarps) {
        int sh[4], dim[4];
        long long st[4], size = 1;
        for (int k = 0; k < 4; ++k) {
            sh[k] = (int)__ldg(&a.quartets[4 * qi + k]);
            dim[k] = __ldg(&a.shell_ncontr[sh[k]]) * ncart(__ldg(&a.shell_l[sh[k]]));
            st[k] = __ldg(&a.ao_start[sh[k]]);
            size *= dim[k];
        }
        bool active[4] = {true, true, true, true};
        for (int o = 1; o < 4; ++o)
            for (int p = 0; p < o && active[o]; ++p) {
                bool same = true;
                for (int k = 0; k < 4; ++k) same = same && sh[perm[o][k]] == sh[perm[p][k]];
                if (same) active[o] = false;
            }
        const double2* blk = a.D + __ldg(&a.offsets[qi]);
        double2 acc[12];
#pragma unroll
        for (int t = 0; t < 12; ++t) acc[t] = c2(0.0, 0.0);
        for (long long loc = lane; loc < size; loc += 32) {
            long long ao[4];
            long long rest = loc;
            for (int k = 3; k >= 0; --k) {
                ao[k] = st[k] + rest % dim[k];
                rest /= dim[k];
            }
            double2 wd = c2(0.0, 0.0), wc = c2(0.0, 0.0);  // direct / conjugated images
            for (int o = 0; o < 4; ++o) {
                if (!active[o]) continue;
                const long long mu = ao[perm[o][0]], nu = ao[perm[o][1]], la = ao[perm[o][2]], si = ao[perm[o][3]];
                double2 w = c2(0.0, 0.0);
                for (int p = 0; p < a.npc; ++p) {
                    const double2* P = a.coulomb + (2 * p) * n * n;
                    const double2* Q = P + n * n;
                    w = cmac(w, __ldg(&P[nu * n + mu]), __ldg(&Q[si * n + la]));
                }
                for (int p = 0; p < a.npx; ++p) {
                    const double2* P = a.exchange + (2 * p) * n * n;
                    const double2* Q = P + n * n;
                    w = cmac(w, __ldg(&P[nu * n + la]), __ldg(&Q[si * n + mu]));
                }
                const long long gi = ((mu * n + nu) * n + la) * n + si;
                if (a.gamma) w = cadd(w, __ldg(&a.gamma[gi]));
                if (a.gamma_real) w.x += __ldg(&a.gamma_real[gi]);
                if (o < 2)
                    wd = cadd(wd, w);
                else
                    wc = cadd(wc, w);
            }
#pragma unroll
            for (int t = 0; t < 12; ++t) {
                const double2 dv = __ldg(&blk[(long long)t * size + loc]);
                // d wd + conj(d) wc
                acc[t].x += dv.x * wd.x - dv.y * wd.y + dv.x * wc.x + dv.y * wc.y;
                acc[t].y += dv.x * wd.y + dv.y * wd.x + dv.x * wc.y - dv.y * wc.x;
            }
        }
#pragma unroll
        for (int t = 0; t < 12; ++t)
            for (int off = 16; off > 0; off >>= 1) {
                acc[t].x += __shfl_xor_sync(0xffffffffu, acc[t].x, off);
                acc[t].y += __shfl_xor_sync(0xffffffffu, acc[t].y, off);
            }
        if (lane == 0)
            for (int t = 0; t < 12; ++t) a.partials[(long long)qi * 12 + t] = acc[t];
    }
}

__global__ void __launch_bounds__(256) gather_abs_kernel(const double2* __restrict__ src,
                                                         const long long* __restrict__ idx, double* __restrict__ dst,
                                                         long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double2 v = src[__ldg(&idx[i])];
        dst[i] = hypot(v.x, v.y);
    }
}

}  // namespace

cudaError_t launch_gather_abs(const double2* src, const long long* idx, double* dst, long long n, int sms,
                              cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const long long want = (n + 255) / 256;
    const unsigned blocks = (unsigned)std::max<long long>(1, std::min(want, (long long)sms * 8));
    gather_abs_kernel<<<blocks, 256, 0, s>>>(src, idx, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_deriv_contract(const DerivContractArgs& args, int sms, cudaStream_t s) {
    if (args.nq == 0) return cudaSuccess;
    const long long want = ((long long)args.nq + 3) / 4;  // 4 warps per block
    const unsigned blocks = (unsigned)std::max<long long>(1, std::min(want, (long long)sms * 16));
    deriv_contract_kernel<<<blocks, 128, 0, s>>>(args);
    return cudaGetLastError();
}

cudaError_t launch_deriv_mixed(const DerivMixedArgs& args, long long total, int sms, cudaStream_t s) {
    if (total == 0) return cudaSuccess;
    const long long want = (total + 255) / 256;
    const unsigned blocks = (unsigned)std::max<long long>(1, std::min(want, (long long)sms * 8));
    deriv_mixed_kernel<<<blocks, 256, 0, s>>>(args);
    return cudaGetLastError();
}

cudaError_t launch_deriv_combine(const DerivCombineArgs& args, long long total, int sms, cudaStream_t s) {
    if (total == 0) return cudaSuccess;
    const long long want = (total + 255) / 256;
    const long long cap = (long long)sms * 8;
    const unsigned blocks = (unsigned)std::max<long long>(1, std::min(want, cap));
    deriv_combine_kernel<<<blocks, 256, 0, s>>>(args);
    return cudaGetLastError();
}

}  // namespace gx
