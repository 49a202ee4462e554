// Class-specialised FP32 lane kernel for the mixed-precision primitive
// quartets of the classes with 3 <= L <= 4 (each l <= 2).
//
// In mixed precision a primitive quartet whose Schwarz product lies below the
// FP32 cutoff is evaluated in FP32.  The class-generic kernel runs those
// entries through its table-driven warp transforms, where shared-memory index
// chains, not FP32 arithmetic, set the cost, so an FP32 entry cost about as
// much as an FP64 one.  Here the FP32 entries of a class get their own
// kernel, compiled per (la, lb, lc, ld): one lane evaluates one primitive
// quartet completely in registers -- the Hermite table Rh by the constexpr
// recurrence plan, then, ket component by ket component, the ket transform
// W[K] = sum_{K' in box(cd)} (-1)^{|K'|} E~cd[K'] Rh[K + K'] and the bra
// transform v[ab] = sum_{K in box(ab)} E~ab[K] W[K].  Lanes of a batch that
// belong to the same shell quartet are summed by a segmented warp reduction
// per ket component and the first lane of each segment adds the sum (in
// FP64) to the output block.  The class-generic kernel of the same class
// runs first on the same stream, zeroes the blocks and adds the FP64 entries.
//
// FP64 is kept where the precision split asks for it: forming X', T and the
// prefactor, the Boys function outside its asymptotic sector (and its
// downward recursion), the seeds C (-2 rho)^n F_n, and every output sum.  The
// seeds of the lanes of one shell quartet are scaled by one power of two so
// that their largest magnitude is 2^60 before the conversion to FP32 (the
// recurrence and both transforms are linear in the seeds, so the scale is
// undone exactly when the FP32 sum is added in FP64); no FP32 entry has to
// fall back to FP64 for range.
//
// Two passes over a warp's primitive quartets keep each batch on one Boys
// path: pass 0 the entries whose argument the FP32 pair geometry places in
// the asymptotic sector, pass 1 the others (FP64 Boys and seeds).  In pass 0
// T is recomputed in FP32 from the FP64 separation X' (a lane outside the
// sector takes the FP64 path), F_0 = sqrt(pi)/(2 sqrt T) in FP32, and the
// seeds follow in FP32 from the scaled C F_0 by S_{n+1} = -(2n+1) S_n / X'.X'
// (the asymptotic recurrence F_{n+1} = F_n (n + 1/2)/T with T = rho X'.X'):
// only X', the prefactor C and its power-of-two scale stay in FP64.
#pragma once

#include <utility>

#include "gx_small.cuh"

namespace gx {
namespace lane {

using small::boxdim;
using small::boxent;
using small::boxoff;
using small::boxsize;
using small::hc;
using small::herm;
using small::hi;
using small::I3;
using small::nc;

// ket transform of ket component CD, box entry E: W[K] += s E~cd[E] Rh[K + ent(E)]
template <int LA, int LB, int LC, int LD, int CD, int E, int... K>
__device__ __forceinline__ void ket_entry(float2* W, const float2* R, float2 ev, std::integer_sequence<int, K...>) {
    constexpr I3 t = boxent(LC, LD, CD, E);
    (
        [&] {
            constexpr I3 h = herm(K);
            constexpr int r = hi(h.x + t.x, h.y + t.y, h.z + t.z);
            W[K] = small::fmac2(W[K], ev, R[r]);
        }(),
        ...);
}

template <int LA, int LB, int LC, int LD, int CD, int... E>
__device__ __forceinline__ void ket_component(float2* W, const float2* R, const float2* __restrict__ Ecd,
                                              std::integer_sequence<int, E...>) {
    (
        [&] {
            constexpr I3 t = boxent(LC, LD, CD, E);
            float2 ev = __ldg(&Ecd[boxoff(LC, LD, CD) + E]);
            if constexpr ((t.x + t.y + t.z) & 1) ev = make_float2(-ev.x, -ev.y);
            ket_entry<LA, LB, LC, LD, CD, E>(W, R, ev, std::make_integer_sequence<int, hc(LA + LB)>{});
        }(),
        ...);
}

// Read-only load of one FP32 record word.  The volatile form keeps the
// compiler from hoisting the bra record out of the ket-component loop into
// registers (for large bra records that costs more in occupancy and spills
// than the reloads, which hit L1).
template <bool VOLATILE>
__device__ __forceinline__ float2 ld_rec(const float2* p) {
    if constexpr (VOLATILE) {
        float2 v;
        asm volatile("ld.global.nc.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
        return v;
    } else {
        return __ldg(p);
    }
}

// bra transform of bra component AB: v += sum_{K in box(AB)} E~ab[K] W[K]
template <int LA, int LB, int AB, int... E>
__device__ __forceinline__ float2 bra_component(const float2* W, const float2* __restrict__ Eab,
                                                std::integer_sequence<int, E...>) {
    constexpr bool kReload = small::etot(LA, LB) > 24;
    float2 v = make_float2(0.0f, 0.0f);
    (
        [&] {
            constexpr I3 t = boxent(LA, LB, AB, E);
            v = small::fmac2(v, ld_rec<kReload>(&Eab[boxoff(LA, LB, AB) + E]), W[hi(t.x, t.y, t.z)]);
        }(),
        ...);
    return v;
}

template <int LA, int LB, int... AB>
__device__ __forceinline__ void bra_all(float2* v, const float2* W, const float2* __restrict__ Eab,
                                        std::integer_sequence<int, AB...>) {
    ((v[AB] = bra_component<LA, LB, AB>(W, Eab, std::make_integer_sequence<int, boxsize(LA, LB, AB)>{})), ...);
}

// Segmented sum over the lanes of one shell quartet (keys non-decreasing
// along the warp; take bit r: add the value of lane + 2^r): afterwards the
// first lane of each run holds the run's total.
template <int N>
__device__ __forceinline__ void seg_sum_masked(float2* v, unsigned take) {
#pragma unroll
    for (int r = 0; r < 5; ++r) {
        const int off = 1 << r;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            const float ox = __shfl_down_sync(0xffffffffu, v[i].x, off);
            const float oy = __shfl_down_sync(0xffffffffu, v[i].y, off);
            if ((take >> r) & 1u) v[i] = make_float2(v[i].x + ox, v[i].y + oy);
        }
    }
}

// Per-batch state of the output add: the head lane's task block and the
// power of two that undoes its seed scale.
struct OutCtx {
    double2* base;
    int st[4];
    double unscale;
    bool head;
};

template <int LA, int LB, int LC, int LD, int CD>
__device__ __forceinline__ void component(const float2* R, const float2* __restrict__ Ecd,
                                          const float2* __restrict__ Eab, unsigned take, const OutCtx& oc) {
    constexpr int NH = hc(LA + LB), NAB = nc(LA) * nc(LB);
    constexpr int NCB = nc(LB), NCDD = nc(LD);
    float2 W[NH];
#pragma unroll
    for (int k = 0; k < NH; ++k) W[k] = make_float2(0.0f, 0.0f);
    ket_component<LA, LB, LC, LD, CD>(W, R, Ecd, std::make_integer_sequence<int, boxsize(LC, LD, CD)>{});
    float2 v[NAB];
    bra_all<LA, LB>(v, W, Eab, std::make_integer_sequence<int, NAB>{});
    seg_sum_masked<NAB>(v, take);
    if (oc.head) {
        constexpr int cc = CD / NCDD, cdd = CD - (CD / NCDD) * NCDD;
        double2* o = oc.base + (long long)cc * oc.st[2] + (long long)cdd * oc.st[3];
#pragma unroll
        for (int ab = 0; ab < NAB; ++ab) {
            const int ca = ab / NCB, cb = ab - (ab / NCB) * NCB;
            double2* p = o + (long long)ca * oc.st[0] + (long long)cb * oc.st[1];
            *p = cadd(*p, c2((double)v[ab].x * oc.unscale, (double)v[ab].y * oc.unscale));
        }
    }
}

template <int LA, int LB, int LC, int LD, int... CD>
__device__ __forceinline__ void all_components(const float2* R, const float2* __restrict__ Ecd,
                                               const float2* __restrict__ Eab, unsigned take, const OutCtx& oc,
                                               std::integer_sequence<int, CD...>) {
    (component<LA, LB, LC, LD, CD>(R, Ecd, Eab, take, oc), ...);
}

// 2^e as a double (|e| <= 1000)
__device__ __forceinline__ double pow2(int e) { return __hiloint2double((e + 1023) << 20, 0); }

template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(128) lane32_kernel(EriDev d, QuartetClass qc) {
    constexpr int L = LA + LB + LC + LD;
    constexpr int NL = hc(L);
    constexpr int NCD = nc(LC) * nc(LD);
    __shared__ int s_queue[4][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    int* queue = s_queue[wib];
    const int nwarp = gridDim.x * (blockDim.x >> 5);
    const PairData& pp = d.pairs;
    const float skip = d.skip_cut, cut32 = d.fp32_cut;
    unsigned n32 = 0;
    for (int grp = blockIdx.x * (blockDim.x >> 5) + wib; grp < qc.ngroup; grp += nwarp) {
        const int2 gi = qc.groups[grp];
        const Task t0 = qc.tasks[gi.x];
        const int Kab = d.basis.nprim[t0.sa] * d.basis.nprim[t0.sb];
        const int Kcd = d.basis.nprim[t0.sc] * d.basis.nprim[t0.sd];
        const int KK = Kab * Kcd;
        const int S = gi.y * KK;
        for (int pass = 0; pass < 2; ++pass) {
            int cursor = 0;
            while (cursor < S) {
                // compact up to 32 FP32 entries of this pass
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
                        valid = b >= skip && b < cut32 &&
                                (pass == 0) == boys_asymptotic32(pp, pp.order[op], pp.order[oq], L);
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
                int ip = 0, iq = 0;
                double2 Sh[L + 1];
                double2 X[3];
                double2 C = c2(0.0, 0.0);
                float2 F0 = make_float2(0.0f, 0.0f), iXX = make_float2(0.0f, 0.0f);
                int mode = 1;  // 0: FP32 seeds from the asymptotic recurrence; 1: FP64 seeds in Sh
                int e_lane = -1000;
                Task tg{};
                if (active) {
                    const int idx = queue[lane];
                    const int g = idx / KK, r = idx - g * KK;
                    const int P = r / Kcd, Q = r - P * Kcd;
                    key = g;
                    tg = qc.tasks[gi.x + g];
                    ip = pp.order[tg.pab + P];
                    iq = pp.order[tg.pcd + Q];
                    const double p = pp.p[ip], q = pp.p[iq];
#pragma unroll
                    for (int x = 0; x < 3; ++x)
                        X[x] = c2(pp.Pr[3 * ip + x] - pp.Pr[3 * iq + x], pp.Pi[3 * ip + x] - pp.Pi[3 * iq + x]);
                    const double rs = rsqrt(p + q);
                    C = cscale(cmul(pp.F[ip], pp.F[iq]), rs);
                    if (pass == 0) {
                        // T in FP32 from the FP64 separation (the asymptotic
                        // sector is far from T = 0, where FP32 would not do)
                        const float2 x0 = make_float2((float)X[0].x, (float)X[0].y);
                        const float2 x1 = make_float2((float)X[1].x, (float)X[1].y);
                        const float2 x2 = make_float2((float)X[2].x, (float)X[2].y);
                        const float pf = (float)p, qf = (float)q;
                        const float rho32 = __fdividef(pf * qf, pf + qf);
                        const float2 XX = make_float2(fmaf(x0.x, x0.x, fmaf(x1.x, x1.x, x2.x * x2.x)) -
                                                          fmaf(x0.y, x0.y, fmaf(x1.y, x1.y, x2.y * x2.y)),
                                                      2.0f * fmaf(x0.x, x0.y, fmaf(x1.x, x1.y, x2.x * x2.y)));
                        const float tr = rho32 * XX.x, ti = rho32 * XX.y;
                        const float r2 = fmaf(tr, tr, ti * ti);
                        if (tr >= 2.0f * L + 24.0f && fabsf(ti) <= 0.5f * tr &&
                            (r2 <= 160.0f * 160.0f || tr >= 2.0f * L + 60.0f)) {
                            // F_0 = sqrt(pi) / (2 sqrt(T)); seeds later by
                            // S_{n+1} = S_n (-(2n + 1)) / (X'.X'), from
                            // F_{n+1} = F_n (n + 1/2) / T and T = rho X'.X'
                            const float ir = rsqrtf(r2);
                            const float sq = sqrtf(0.5f * (r2 * ir + tr));
                            const float k0 = 0.886226925452758f * ir;
                            F0 = make_float2(k0 * sq, -k0 * (0.5f * ti / sq));
                            const float m2 = fmaf(XX.x, XX.x, XX.y * XX.y);
                            iXX = make_float2(__fdividef(XX.x, m2), -__fdividef(XX.y, m2));
                            const float ixx = rsqrtf(m2);
                            float gm = 1.0f, gmax = 1.0f;
#pragma unroll
                            for (int n = 0; n < L; ++n) {
                                gm *= (2.0f * n + 1.0f) * ixx;
                                gmax = fmaxf(gmax, gm);
                            }
                            // binary exponents from the bits (integer work)
                            const int ec = max((__double2hiint(C.x) >> 20) & 0x7ff, (__double2hiint(C.y) >> 20) & 0x7ff);
                            const int ef = (__float_as_int(fmaxf(fabsf(F0.x), fabsf(F0.y))) >> 23) & 0xff;
                            const int eg = (__float_as_int(gmax) >> 23) & 0xff;
                            if (ec > 0 && ec < 0x7ff && ef > 0 && ef < 0xff && eg < 0xff)
                                e_lane = (ec - 1023) + (ef - 127) + (eg - 127) + 2;
                            mode = 0;
                        }
                    }
                    if (mode == 1) {
                        const double rho = p * q * rs * rs;
                        const double tre = rho * (fma(X[0].x, X[0].x, fma(X[1].x, X[1].x, X[2].x * X[2].x)) -
                                                  fma(X[0].y, X[0].y, fma(X[1].y, X[1].y, X[2].y * X[2].y)));
                        const double tim = 2.0 * rho * fma(X[0].x, X[0].y, fma(X[1].x, X[1].y, X[2].x * X[2].y));
                        small::quartet_seeds<L>(d, gi.x + g, C, rho, tre, tim, Sh);
                        // largest binary exponent of the seeds, read from the bits
#pragma unroll
                        for (int n = 0; n <= L; ++n) {
                            const int ex = (__double2hiint(Sh[n].x) >> 20) & 0x7ff;
                            const int ey = (__double2hiint(Sh[n].y) >> 20) & 0x7ff;
                            const int e = max(ex, ey);
                            if (e > 0 && e < 0x7ff) e_lane = max(e_lane, e - 1023);
                        }
                    }
                }
                // segment structure: heads, the take masks of the reduction and
                // the largest seed exponent of each segment, broadcast to it
                const int kprev = __shfl_up_sync(0xffffffffu, key, 1);
                const bool head = active && (lane == 0 || kprev != key);
                unsigned take = 0;
                int e_seg = e_lane;
#pragma unroll
                for (int r = 0; r < 5; ++r) {
                    const int off = 1 << r;
                    const int ko = __shfl_down_sync(0xffffffffu, key, off);
                    const int eo = __shfl_down_sync(0xffffffffu, e_seg, off);
                    if (lane + off < 32 && ko == key) {
                        take |= 1u << r;
                        e_seg = max(e_seg, eo);
                    }
                }
                const unsigned heads = __ballot_sync(0xffffffffu, head);
                const int my_head = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
                e_seg = __shfl_sync(0xffffffffu, e_seg, active ? my_head : lane);
                const int shift = max(-1000, min(1000, e_seg - 60));
                // Rh in registers (zero on idle lanes, which still take part in
                // the shuffles of every reduction: one code path for all lanes)
                float2 R32[NL];
#pragma unroll
                for (int i = 0; i < NL; ++i) R32[i] = make_float2(0.0f, 0.0f);
                if (active) {
                    const double sc = pow2(-shift);
                    float2 S32[L + 1];
                    if (mode == 0) {
                        S32[0] = small::fmul2(make_float2((float)(C.x * sc), (float)(C.y * sc)), F0);
#pragma unroll
                        for (int n = 0; n < L; ++n) {
                            const float2 t = small::fmul2(S32[n], iXX);
                            S32[n + 1] = make_float2(-(2.0f * n + 1.0f) * t.x, -(2.0f * n + 1.0f) * t.y);
                        }
                    } else {
#pragma unroll
                        for (int n = 0; n <= L; ++n)
                            S32[n] = make_float2((float)(Sh[n].x * sc), (float)(Sh[n].y * sc));
                    }
                    const float2 X32[3] = {make_float2((float)X[0].x, (float)X[0].y),
                                           make_float2((float)X[1].x, (float)X[1].y),
                                           make_float2((float)X[2].x, (float)X[2].y)};
                    R32[0] = S32[L];
                    small::run_rec32<L>(R32, S32, X32, std::make_integer_sequence<int, small::rsteps(L)>{});
                    ++n32;
                }
                OutCtx oc;
                oc.base = d.out + tg.out_off;
                oc.st[0] = tg.st[0];
                oc.st[1] = tg.st[1];
                oc.st[2] = tg.st[2];
                oc.st[3] = tg.st[3];
                oc.unscale = pow2(shift);
                oc.head = head;
                // idle lanes read the first words of the record pool (in bounds; their values are zeroed by R32)
                const long long eq = active ? pp.Eoff[iq] : 0, ep = active ? pp.Eoff[ip] : 0;
                all_components<LA, LB, LC, LD>(R32, pp.Epool32 + eq, pp.Epool32 + ep, take, oc,
                                               std::make_integer_sequence<int, NCD>{});
                __syncwarp();
            }
        }
    }
    if (d.counters) {
        const unsigned a32 = __reduce_add_sync(0xffffffffu, n32);
        if (lane == 0) atomicAdd(&d.counters[1], (unsigned long long)a32);
    }
}

}  // namespace lane
}  // namespace gx
