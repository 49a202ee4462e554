// Register-resident kernel for the small quartet classes (L = la+lb+lc+ld <= 2).
//
// One lane evaluates one whole shell quartet: every primitive quartet's
// Boys values, Hermite table Rh, ket transform W[K][cd] (accumulated over the
// ket primitive pairs) and bra transform into out[ab][cd], all in registers.
// Lanes of a warp run quartets with equal primitive counts (tasks are sorted
// by (Kab, Kcd) within a class), so no lane idles and no FP64 instruction is
// issued for a masked-off lane.  Every loop is expanded at compile time from
// constexpr plans (index-sequence folds), so all register indices are
// constants.
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

template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(128) small_kernel(EriDev d, const Task* tasks, int ntask) {
    constexpr int L = LA + LB + LC + LD;
    constexpr int NL = hc(L), NH = hc(LA + LB);
    constexpr int NAB = nc(LA) * nc(LB), NCD = nc(LC) * nc(LD);
    const int tk = blockIdx.x * blockDim.x + threadIdx.x;
    if (tk >= ntask) return;
    const Task t = tasks[tk];
    const int ns = d.basis.ns;
    const int Kab = d.basis.nprim[t.sa] * d.basis.nprim[t.sb];
    const int Kcd = d.basis.nprim[t.sc] * d.basis.nprim[t.sd];
    const int pab0 = d.basis.sp_off[t.sa * ns + t.sb];
    const int pcd0 = d.basis.sp_off[t.sc * ns + t.sd];
    const PairData& pp = d.pairs;
    double2 out[NAB * NCD];
#pragma unroll
    for (int i = 0; i < NAB * NCD; ++i) out[i] = c2(0.0, 0.0);
    for (int P = 0; P < Kab; ++P) {
        const int ip = pab0 + P;
        const double p = pp.p[ip];
        const double Pr0 = pp.Pr[3 * ip], Pr1 = pp.Pr[3 * ip + 1], Pr2 = pp.Pr[3 * ip + 2];
        const double Pi0 = pp.Pi[3 * ip], Pi1 = pp.Pi[3 * ip + 1], Pi2 = pp.Pi[3 * ip + 2];
        const double2 Fab = pp.F[ip];
        double2 W[NH * NCD];
#pragma unroll
        for (int i = 0; i < NH * NCD; ++i) W[i] = c2(0.0, 0.0);
        for (int Q = 0; Q < Kcd; ++Q) {
            const int iq = pcd0 + Q;
            const double q = pp.p[iq];
            const double2 X[3] = {c2(Pr0 - pp.Pr[3 * iq], Pi0 - pp.Pi[3 * iq]),
                                  c2(Pr1 - pp.Pr[3 * iq + 1], Pi1 - pp.Pi[3 * iq + 1]),
                                  c2(Pr2 - pp.Pr[3 * iq + 2], Pi2 - pp.Pi[3 * iq + 2])};
            const double r = rsqrt(p + q);
            const double rho = p * q * r * r;
            const double tre = rho * (fma(X[0].x, X[0].x, fma(X[1].x, X[1].x, X[2].x * X[2].x)) -
                                      fma(X[0].y, X[0].y, fma(X[1].y, X[1].y, X[2].y * X[2].y)));
            const double tim = 2.0 * rho * fma(X[0].x, X[0].y, fma(X[1].x, X[1].y, X[2].x * X[2].y));
            double2 Sh[L + 1];
            double2 e0;
            double2 C = cscale(cmul(Fab, pp.F[iq]), r);
            if (const int rc = boys_eval(tre, tim, L, d.boys, d.gl, Sh, e0)) {
                report(d.status, rc, tk, L, tre, tim);
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
            double2 R[NL];
            if constexpr (L == 0) {
                R[0] = Sh[0];
            } else {
                R[0] = Sh[L];
                run_rec<L>(R, Sh, X, std::make_integer_sequence<int, rsteps(L)>{});
            }
            run_k<LA, LB, LC, LD>(W, R, pp.Epool + pp.Eoff[iq],
                                  std::make_integer_sequence<int, kmacs<LA, LB, LC, LD>()>{});
        }
        run_b<LA, LB, LC, LD>(out, W, pp.Epool + pp.Eoff[ip],
                              std::make_integer_sequence<int, bmacs<LA, LB, LC, LD>()>{});
    }
    constexpr int NCB = nc(LB), NCDD = nc(LD);
#pragma unroll
    for (int ab = 0; ab < NAB; ++ab)
#pragma unroll
        for (int cd = 0; cd < NCD; ++cd) {
            const int ca = ab / NCB, cb = ab % NCB, cc = cd / NCDD, cdd = cd % NCDD;
            d.out[t.out_off + (long long)ca * t.st[0] + (long long)cb * t.st[1] + (long long)cc * t.st[2] +
                  (long long)cdd * t.st[3]] = out[ab * NCD + cd];
        }
}

}  // namespace small
}  // namespace gx
