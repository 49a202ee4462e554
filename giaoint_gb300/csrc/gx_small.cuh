// Register-resident kernel for the small quartet classes (L = la+lb+lc+ld <= 2).
//
// One lane evaluates one primitive quartet completely: Boys values, Hermite
// table Rh, ket transform W[K][cd] and bra transform into its contribution
// v[ab][cd], all in registers.  A warp walks the primitive quartets of a
// group of shell quartets with equal primitive counts as one stream and
// compacts the ones that survive screening (and belong to the current
// precision pass) into full batches of 32 with a ballot, so screening removes
// issue slots instead of idling lanes.  Lanes of a batch that belong to the
// same shell quartet are summed by a segmented warp reduction and the first
// lane of each segment adds the sum to the output block.  Every loop is
// expanded at compile time from constexpr plans (index-sequence folds), so
// all register indices are constants.
#pragma once

#include <utility>

#include "gx_internal.h"

namespace gx {
namespace small {

__host__ __device__ constexpr int nc(int l) { return (l + 1) * (l + 2) / 2; }
__host__ __device__ constexpr int hc(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }
__host__ __device__ constexpr int hi(int k, int l, int m) {
    const int s = k + l + m;
    return s * (s + 1) * (s + 2) / 6 + (s - k) * (s - k + 1) / 2 + m;
}
struct I3 {
    int x, y, z;
};
__host__ __device__ constexpr I3 comp(int l, int idx) {  // x-major Cartesian component
    int k = 0;
    for (int x = l; x >= 0; --x)
        for (int y = l - x; y >= 0; --y) {
            if (k == idx) return I3{x, y, l - x - y};
            ++k;
        }
    return I3{0, 0, 0};
}
__host__ __device__ constexpr I3 herm(int idx) {  // Hermite multi-index of enumeration position idx
    for (int s = 0;; ++s)
        for (int k = s; k >= 0; --k)
            for (int l = s - k; l >= 0; --l)
                if (hi(k, l, s - k - l) == idx) return I3{k, l, s - k - l};
}
// box of component pair ab of pair class (la, lb)
__host__ __device__ constexpr I3 boxdim(int la, int lb, int ab) {
    const I3 a = comp(la, ab / nc(lb)), b = comp(lb, ab % nc(lb));
    return I3{a.x + b.x + 1, a.y + b.y + 1, a.z + b.z + 1};
}
__host__ __device__ constexpr int boxsize(int la, int lb, int ab) {
    const I3 d = boxdim(la, lb, ab);
    return d.x * d.y * d.z;
}
__host__ __device__ constexpr int boxoff(int la, int lb, int ab) {
    int o = 0;
    for (int i = 0; i < ab; ++i) o += boxsize(la, lb, i);
    return o;
}
__host__ __device__ constexpr I3 boxent(int la, int lb, int ab, int e) {
    const I3 d = boxdim(la, lb, ab);
    return I3{e / (d.y * d.z), (e / d.z) % d.y, e % d.z};
}
__host__ __device__ constexpr int etot(int la, int lb) { return boxoff(la, lb, nc(la) * nc(lb)); }

// Rh recurrence plan: step s of the in-place descending scheme.
struct RStep {
    int kind;  // 0 = recurrence entry, 1 = seed of level n
    int dst, s1, s2, axis, coef, n;
};
__host__ __device__ constexpr int rsteps(int L) {
    int c = 0;
    for (int n = L - 1; n >= 0; --n) {
        for (int d = L - n; d >= 1; --d) c += (d + 1) * (d + 2) / 2;
        ++c;
    }
    return c;
}
__host__ __device__ constexpr RStep rstep(int L, int idx) {
    int c = 0;
    for (int n = L - 1; n >= 0; --n) {
        for (int d = L - n; d >= 1; --d)
            for (int k = d; k >= 0; --k)
                for (int l = d - k; l >= 0; --l) {
                    const int m = d - k - l;
                    if (c++ == idx) {
                        if (k > 0) return RStep{0, hi(k, l, m), hi(k - 1, l, m), k > 1 ? hi(k - 2, l, m) : 0, 0, k - 1, n};
                        if (l > 0) return RStep{0, hi(0, l, m), hi(0, l - 1, m), l > 1 ? hi(0, l - 2, m) : 0, 1, l - 1, n};
                        return RStep{0, hi(0, 0, m), hi(0, 0, m - 1), m > 1 ? hi(0, 0, m - 2) : 0, 2, m - 1, n};
                    }
                }
        if (c++ == idx) return RStep{1, 0, 0, 0, 0, 0, n};
    }
    return RStep{1, 0, 0, 0, 0, 0, 0};
}

// ket-transform MAC t over (cd, e, K): W[K][cd] += s(e) Ecd[off(cd)+e] Rh[K + ent(e)]
struct KMac {
    int w, eoff, r, neg;
};
template <int LA, int LB, int LC, int LD>
__host__ __device__ constexpr int kmacs() {
    int c = 0;
    for (int cd = 0; cd < nc(LC) * nc(LD); ++cd) c += boxsize(LC, LD, cd) * hc(LA + LB);
    return c;
}
template <int LA, int LB, int LC, int LD>
__host__ __device__ constexpr KMac kmac(int idx) {
    constexpr int NH = hc(LA + LB), NCD = nc(LC) * nc(LD);
    int c = 0;
    for (int cd = 0; cd < NCD; ++cd)
        for (int e = 0; e < boxsize(LC, LD, cd); ++e)
            for (int K = 0; K < NH; ++K)
                if (c++ == idx) {
                    const I3 h = herm(K), t = boxent(LC, LD, cd, e);
                    return KMac{K * NCD + cd, boxoff(LC, LD, cd) + e, hi(h.x + t.x, h.y + t.y, h.z + t.z),
                                (t.x + t.y + t.z) & 1};
                }
    return KMac{0, 0, 0, 0};
}
// bra-transform MAC t over (ab, e, cd): out[ab][cd] += Eab[off(ab)+e] W[ent(e)][cd]
struct BMac {
    int o, eoff, w;
};
template <int LA, int LB, int LC, int LD>
__host__ __device__ constexpr int bmacs() {
    int c = 0;
    for (int ab = 0; ab < nc(LA) * nc(LB); ++ab) c += boxsize(LA, LB, ab) * nc(LC) * nc(LD);
    return c;
}
template <int LA, int LB, int LC, int LD>
__host__ __device__ constexpr BMac bmac(int idx) {
    constexpr int NCD = nc(LC) * nc(LD);
    int c = 0;
    for (int ab = 0; ab < nc(LA) * nc(LB); ++ab)
        for (int e = 0; e < boxsize(LA, LB, ab); ++e)
            for (int cd = 0; cd < NCD; ++cd)
                if (c++ == idx) {
                    const I3 t = boxent(LA, LB, ab, e);
                    return BMac{ab * NCD + cd, boxoff(LA, LB, ab) + e, hi(t.x, t.y, t.z) * NCD + cd};
                }
    return BMac{0, 0, 0};
}

__device__ __forceinline__ float2 fmul2(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 fmac2(float2 c, float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}

template <int L, int... S>
__device__ __forceinline__ void run_rec32(float2* R, const float2* seed, const float2* X,
                                          std::integer_sequence<int, S...>) {
    (
        [&] {
            constexpr RStep st = rstep(L, S);
            if constexpr (st.kind == 1) {
                R[0] = seed[st.n];
            } else {
                float2 v = fmul2(X[st.axis], R[st.s1]);
                if constexpr (st.coef > 0) {
                    v.x = fmaf((float)st.coef, R[st.s2].x, v.x);
                    v.y = fmaf((float)st.coef, R[st.s2].y, v.y);
                }
                R[st.dst] = v;
            }
        }(),
        ...);
}

template <int LA, int LB, int LC, int LD, int... S>
__device__ __forceinline__ void run_k32(float2* W, const float2* R, const float2* __restrict__ Ecd,
                                        std::integer_sequence<int, S...>) {
    (
        [&] {
            constexpr KMac m = kmac<LA, LB, LC, LD>(S);
            float2 e = __ldg(&Ecd[m.eoff]);
            if constexpr (m.neg) e = make_float2(-e.x, -e.y);
            W[m.w] = fmac2(W[m.w], e, R[m.r]);
        }(),
        ...);
}

template <int LA, int LB, int LC, int LD, int... S>
__device__ __forceinline__ void run_b32(float2* out, const float2* W, const float2* __restrict__ Eab,
                                        std::integer_sequence<int, S...>) {
    (
        [&] {
            constexpr BMac m = bmac<LA, LB, LC, LD>(S);
            out[m.o] = fmac2(out[m.o], __ldg(&Eab[m.eoff]), W[m.w]);
        }(),
        ...);
}

template <int L, int... S>
__device__ __forceinline__ void run_rec(double2* R, const double2* seed, const double2* X,
                                        std::integer_sequence<int, S...>) {
    (
        [&] {
            constexpr RStep st = rstep(L, S);
            if constexpr (st.kind == 1) {
                R[0] = seed[st.n];
            } else {
                double2 v = cmul(X[st.axis], R[st.s1]);
                if constexpr (st.coef > 0) v = cmacr(v, (double)st.coef, R[st.s2]);
                R[st.dst] = v;
            }
        }(),
        ...);
}

template <int LA, int LB, int LC, int LD, int... S>
__device__ __forceinline__ void run_k(double2* W, const double2* R, const double2* __restrict__ Ecd,
                                      std::integer_sequence<int, S...>) {
    (
        [&] {
            constexpr KMac m = kmac<LA, LB, LC, LD>(S);
            double2 e = __ldg(&Ecd[m.eoff]);
            if constexpr (m.neg) e = c2(-e.x, -e.y);
            W[m.w] = cmac(W[m.w], e, R[m.r]);
        }(),
        ...);
}

template <int LA, int LB, int LC, int LD, int... S>
__device__ __forceinline__ void run_b(double2* out, const double2* W, const double2* __restrict__ Eab,
                                      std::integer_sequence<int, S...>) {
    (
        [&] {
            constexpr BMac m = bmac<LA, LB, LC, LD>(S);
            out[m.o] = cmac(out[m.o], __ldg(&Eab[m.eoff]), W[m.w]);
        }(),
        ...);
}

// Seeds C (-2 rho)^n F_n for one primitive quartet; zero seeds on a Boys
// failure, which is reported through the status word.
template <int L>
__device__ __forceinline__ void quartet_seeds(const EriDev& d, long long item, double2 C, double rho, double tre,
                                              double tim, double2* Sh) {
    double2 e0;
    if (const int rc = boys_eval(tre, tim, L, d.boys, d.gl, Sh, e0)) {
        report(d.status, rc, item, L, tre, tim);
        C = c2(0.0, 0.0);
        e0 = c2(0.0, 0.0);
    }
    C = cmul(C, e0);
    const double m2r = -2.0 * rho;
#pragma unroll
    for (int n = 0; n <= L; ++n) {
        Sh[n] = cmul(C, Sh[n]);
        C = cscale(C, m2r);
    }
}

// Segmented sum over lanes with equal key (keys non-decreasing along the
// warp): afterwards the first lane of each run holds the run's total.
template <int N>
__device__ __forceinline__ void seg_sum(double2* v, int key, int lane) {
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int ko = __shfl_down_sync(0xffffffffu, key, off);
        const bool take = lane + off < 32 && ko == key;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            const double ox = __shfl_down_sync(0xffffffffu, v[i].x, off);
            const double oy = __shfl_down_sync(0xffffffffu, v[i].y, off);
            if (take) v[i] = c2(v[i].x + ox, v[i].y + oy);
        }
    }
}
template <int N>
__device__ __forceinline__ void seg_sum(float2* v, int key, int lane) {
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int ko = __shfl_down_sync(0xffffffffu, key, off);
        const bool take = lane + off < 32 && ko == key;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            const float ox = __shfl_down_sync(0xffffffffu, v[i].x, off);
            const float oy = __shfl_down_sync(0xffffffffu, v[i].y, off);
            if (take) v[i] = make_float2(v[i].x + ox, v[i].y + oy);
        }
    }
}

template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(128) small_kernel(EriDev d, QuartetClass qc) {
    constexpr int L = LA + LB + LC + LD;
    constexpr int NL = hc(L), NH = hc(LA + LB);
    constexpr int NAB = nc(LA) * nc(LB), NCD = nc(LC) * nc(LD), NOUT = NAB * NCD;
    constexpr int NCB = nc(LB), NCDD = nc(LD);
    __shared__ int s_queue[4][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    int* queue = s_queue[wib];
    const int nwarp = gridDim.x * (blockDim.x >> 5);
    const PairData& pp = d.pairs;
    const float skip = d.skip_cut, cut32 = d.fp32_cut;
    const float cut64 = fmaxf(cut32, skip);
    // Mixed precision: pass 0 evaluates the FP64 quartets, pass 1 the FP32
    // quartets whose Boys argument lies in the asymptotic sector (FP32 Boys),
    // pass 2 the other FP32 quartets (FP64 Boys, FP32 recurrence), so that
    // every batch follows one Boys path.
    const int npass = cut32 > 0.0f ? 3 : 1;
    unsigned n64 = 0, n32 = 0;
    auto out_ptr = [&](const Task& t, int o) {
        const int ab = o / NCD, cd = o - ab * NCD;
        const int ca = ab / NCB, cb = ab - ca * NCB, cc = cd / NCDD, cdd = cd - cc * NCDD;
        return d.out + t.out_off + (long long)ca * t.st[0] + (long long)cb * t.st[1] + (long long)cc * t.st[2] +
               (long long)cdd * t.st[3];
    };
    for (int grp = blockIdx.x * (blockDim.x >> 5) + wib; grp < qc.ngroup; grp += nwarp) {
        const int2 gi = qc.groups[grp];
        const Task t0 = qc.tasks[gi.x];
        const int Kab = d.basis.nprim[t0.sa] * d.basis.nprim[t0.sb];
        const int Kcd = d.basis.nprim[t0.sc] * d.basis.nprim[t0.sd];
        const int KK = Kab * Kcd;
        const int S = gi.y * KK;
        for (int it = lane; it < gi.y * NOUT; it += 32) {
            const int g = it / NOUT;
            *out_ptr(qc.tasks[gi.x + g], it - g * NOUT) = c2(0.0, 0.0);
        }
        __syncwarp();
        for (int pass = 0; pass < npass; ++pass) {
            int cursor = 0;
            while (cursor < S) {
                // compact up to 32 surviving entries of this pass
                int nb = 0;
                while (nb < 32 && cursor < S) {
                    const int idx = cursor + lane;
                    bool valid = false;
                    if (idx < S) {
                        const int g = idx / KK, r = idx - g * KK;
                        const int P = r / Kcd, Q = r - P * Kcd;
                        const Task tg = qc.tasks[gi.x + g];
                        const int op = tg.pab + P;
                        const int oq = tg.pcd + Q;
                        const float b = pp.sbound[op] * pp.sbound[oq];
                        valid = pass == 0 ? b >= cut64 : (b >= skip && b < cut32);
                        if (valid && pass > 0)
                            valid = (pass == 1) == boys_asymptotic32(pp, pp.order[op], pp.order[oq], L);
                    }
                    const unsigned mask = __ballot_sync(0xffffffffu, valid);
                    const int cnt = __popc(mask);
                    const int take = min(cnt, 32 - nb);
                    const int rank = __popc(mask & ((1u << lane) - 1u));
                    if (valid && rank < take) queue[nb + rank] = idx;
                    if (take < cnt) {
                        const unsigned m2 = __ballot_sync(0xffffffffu, valid && rank == take);
                        cursor += __ffs(m2) - 1;
                    } else {
                        cursor += 32;
                    }
                    nb += take;
                }
                __syncwarp();
                if (nb == 0) break;
                const bool active = lane < nb;
                int key = -1 - lane;  // idle lanes never match another lane
                double2 v[NOUT];
                float2 v32[NOUT];
#pragma unroll
                for (int i = 0; i < NOUT; ++i) {
                    v[i] = c2(0.0, 0.0);
                    v32[i] = make_float2(0.0f, 0.0f);
                }
                bool used64 = false;
                if (active) {
                    const int idx = queue[lane];
                    const int g = idx / KK, r = idx - g * KK;
                    const int P = r / Kcd, Q = r - P * Kcd;
                    key = g;
                    const Task tg = qc.tasks[gi.x + g];
                    const int ip = pp.order[tg.pab + P];
                    const int iq = pp.order[tg.pcd + Q];
                    const double p = pp.p[ip], q = pp.p[iq];
                    const double2 X[3] = {c2(pp.Pr[3 * ip] - pp.Pr[3 * iq], pp.Pi[3 * ip] - pp.Pi[3 * iq]),
                                          c2(pp.Pr[3 * ip + 1] - pp.Pr[3 * iq + 1], pp.Pi[3 * ip + 1] - pp.Pi[3 * iq + 1]),
                                          c2(pp.Pr[3 * ip + 2] - pp.Pr[3 * iq + 2], pp.Pi[3 * ip + 2] - pp.Pi[3 * iq + 2])};
                    const double rs = rsqrt(p + q);
                    const double rho = p * q * rs * rs;
                    const double tre = rho * (fma(X[0].x, X[0].x, fma(X[1].x, X[1].x, X[2].x * X[2].x)) -
                                              fma(X[0].y, X[0].y, fma(X[1].y, X[1].y, X[2].y * X[2].y)));
                    const double tim = 2.0 * rho * fma(X[0].x, X[0].y, fma(X[1].x, X[1].y, X[2].x * X[2].y));
                    const double2 C = cscale(cmul(pp.F[ip], pp.F[iq]), rs);
                    double2 Sh[L + 1];
                    bool ok32 = false;
                    if (pass > 0) {
                        float2 S32[L + 1];
                        ok32 = pass == 1 && seeds32(C, rho, tre, tim, L, S32);
                        if (!ok32) {
                            // FP64 Boys; FP32 recurrence when the seeds fit
                            quartet_seeds<L>(d, gi.x + g, C, rho, tre, tim, Sh);
                            ok32 = true;
#pragma unroll
                            for (int n = 0; n <= L; ++n) {
                                ok32 = ok32 && fabs(Sh[n].x) + fabs(Sh[n].y) < 1.0e25;
                                S32[n] = make_float2((float)Sh[n].x, (float)Sh[n].y);
                            }
                        }
                        if (ok32) {
                            const float2 X32[3] = {make_float2((float)X[0].x, (float)X[0].y),
                                                   make_float2((float)X[1].x, (float)X[1].y),
                                                   make_float2((float)X[2].x, (float)X[2].y)};
                            float2 R32[NL];
                            if constexpr (L == 0) {
                                R32[0] = S32[0];
                            } else {
                                R32[0] = S32[L];
                                run_rec32<L>(R32, S32, X32, std::make_integer_sequence<int, rsteps(L)>{});
                            }
                            float2 W32[NH * NCD];
#pragma unroll
                            for (int i = 0; i < NH * NCD; ++i) W32[i] = make_float2(0.0f, 0.0f);
                            run_k32<LA, LB, LC, LD>(W32, R32, pp.Epool32 + pp.Eoff[iq],
                                                    std::make_integer_sequence<int, kmacs<LA, LB, LC, LD>()>{});
                            run_b32<LA, LB, LC, LD>(v32, W32, pp.Epool32 + pp.Eoff[ip],
                                                    std::make_integer_sequence<int, bmacs<LA, LB, LC, LD>()>{});
                            ++n32;
                        }
                    } else {
                        quartet_seeds<L>(d, gi.x + g, C, rho, tre, tim, Sh);
                    }
                    if (!ok32) {
                        double2 R[NL];
                        if constexpr (L == 0) {
                            R[0] = Sh[0];
                        } else {
                            R[0] = Sh[L];
                            run_rec<L>(R, Sh, X, std::make_integer_sequence<int, rsteps(L)>{});
                        }
                        double2 W[NH * NCD];
#pragma unroll
                        for (int i = 0; i < NH * NCD; ++i) W[i] = c2(0.0, 0.0);
                        run_k<LA, LB, LC, LD>(W, R, pp.Epool + pp.Eoff[iq],
                                              std::make_integer_sequence<int, kmacs<LA, LB, LC, LD>()>{});
                        run_b<LA, LB, LC, LD>(v, W, pp.Epool + pp.Eoff[ip],
                                              std::make_integer_sequence<int, bmacs<LA, LB, LC, LD>()>{});
                        used64 = true;
                        ++n64;
                    }
                }
                // FP32 contributions are reduced in FP32, FP64 ones in FP64, and
                // the first lane of each segment adds both in FP64.
                if (pass == 0 || __any_sync(0xffffffffu, used64)) seg_sum<NOUT>(v, key, lane);
                if (pass > 0) {
                    seg_sum<NOUT>(v32, key, lane);
#pragma unroll
                    for (int i = 0; i < NOUT; ++i) v[i] = cadd(v[i], c2((double)v32[i].x, (double)v32[i].y));
                }
                const int kprev = __shfl_up_sync(0xffffffffu, key, 1);
                if (active && (lane == 0 || kprev != key)) {
                    const Task tg = qc.tasks[gi.x + key];
#pragma unroll
                    for (int i = 0; i < NOUT; ++i) {
                        double2* o = out_ptr(tg, i);
                        *o = cadd(*o, v[i]);
                    }
                }
                __syncwarp();
            }
        }
    }
    if (d.counters) {
        const unsigned a64 = __reduce_add_sync(0xffffffffu, n64);
        const unsigned a32 = __reduce_add_sync(0xffffffffu, n32);
        if (lane == 0) {
            atomicAdd(&d.counters[0], (unsigned long long)a64);
            atomicAdd(&d.counters[1], (unsigned long long)a32);
        }
    }
}

}  // namespace small
}  // namespace gx
