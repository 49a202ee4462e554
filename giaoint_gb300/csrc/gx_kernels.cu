// GB300 kernels for the GIAO electron-repulsion path.
//
//   boys_table_kernel     scaled Boys values on the Taylor grid (setup)
//   boys_values_kernel    F_0..F_n(z) for the boys() entry point (K2)
//   pair_kernel           primitive-pair records: complex centre, prefactor
//                         and complex Hermite coefficients (K1)
//   quartet_kernel        class-generic shell-quartet ERIs (K3/K4)
//   scatter_full_kernel   the four symmetry images of the full tensor (K5)
//
// Formulation (own derivation; same integral as src/eri.cpp:67-384).
// The reference builds, per Cartesian component quartet, a six-index complex
// table R_{tuv;tau phi chi} whose recurrence carries the London phase as
// -i q terms.  Writing R = d^t/dP^t d^tau/dQ^tau [e^{-i q_ab.P - i q_cd.Q}
// H(P - Q)] and applying Leibniz per axis gives
//   (ab|cd) = sum_{K,K'} E~ab_K E~cd_K' (-1)^{|K'|} Rh_{K+K'}
// with complex Hermite coefficients E~_k = sum_{t>=k} C(t,k) (-i q)^{t-k} E_t
// (E_t the real McMurchie-Davidson coefficients, src/hermite.cpp:8-40) and
// Rh the ordinary three-index MD table of the complex centre separation
// X' = P' - Q', seeded by common (-2 rho)^n F_n(rho X'^2).  E~ depends only
// on the primitive pair, so it is computed once per (basis, field) by
// pair_kernel; per primitive quartet only Rh (C(L+3,3) entries) and the two
// contractions remain.
#include <cstdint>
#include <algorithm>
#include <cstdio>

#include "gx_internal.h"

namespace gx {

// ---------------------------------------------------------------------------
// Boys table (setup): S_n(z0) = e^{z0} F_n(z0), n < 43, on the 1/8 grid.
// Fixed-segment 32-point Gauss-Legendre of the scaled integral, segments
// doubled until two successive results agree to 4e-16 relative.
// ---------------------------------------------------------------------------

// Compensated fixed-segment 32-point Gauss-Legendre of the scaled integral
// (setup only).  e^{x(1-t^2)} is formed as e^x e^{-x t^2} so that the
// rounding of the exponent stays small where the integrand is large.
__device__ void boys_quad_kahan(double x, double y, int L, int segments, const GLRules* gl, double2* out,
                                double2* comp) {
    for (int n = 0; n <= L; ++n) {
        out[n] = c2(0.0, 0.0);
        comp[n] = c2(0.0, 0.0);
    }
    const double inv = 1.0 / (double)segments;
    const double hw = 0.5 * inv;
    const double ex = exp(x);
    for (int s = 0; s < segments; ++s) {
        const double mid = ((double)s + 0.5) * inv;
        for (int k = 0; k < 32; ++k) {
            const double t = fma(hw, gl->x32[k], mid);
            const double t2 = t * t;
            const double mag = ex * exp(-x * t2) * hw * gl->w32[k];
            double sn, cs;
            sincos(y * (1.0 - t2), &sn, &cs);
            double2 term = c2(mag * cs, mag * sn);
            for (int n = 0; n <= L; ++n) {
                const double yr = term.x - comp[n].x, yi = term.y - comp[n].y;
                const double tr = out[n].x + yr, ti = out[n].y + yi;
                comp[n] = c2((tr - out[n].x) - yr, (ti - out[n].y) - yi);
                out[n] = c2(tr, ti);
                term = cscale(term, t2);
            }
        }
    }
}

// Table: 16 segments x 32 points, a single compensated pass; checked against
// 30-digit references to 3e-15 relative over the whole grid (tests compare
// the device Boys function with the oracle across every region).
__global__ void boys_table_kernel(double2* S, double2* E0, const GLRules* gl, int* unused) {
    (void)unused;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= BOYS_NX * BOYS_NY) return;
    const int ix = p / BOYS_NY, iy = p - ix * BOYS_NY;
    const double x = BOYS_X0 + BOYS_H * ix, y = -BOYS_Y1 + BOYS_H * iy;
    constexpr int N = BOYS_TABLE_ORDERS - 1;
    double2 a[N + 1], c[N + 1];
    boys_quad_kahan(x, y, N, 16, gl, a, c);
    double2* dst = S + (size_t)p * BOYS_TABLE_ORDERS;
    for (int n = 0; n <= N; ++n) dst[n] = a[n];
    double sn, cs;
    sincos(-y, &sn, &cs);
    const double m = exp(-x);
    E0[p] = c2(m * cs, m * sn);
}

cudaError_t launch_boys_table(double2* S, double2* E0, const GLRules* gl, int* fail_count, cudaStream_t s) {
    const int n = BOYS_NX * BOYS_NY;
    boys_table_kernel<<<(n + 127) / 128, 128, 0, s>>>(S, E0, gl, fail_count);
    return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// boys() entry point: one thread per argument.  region follows the
// reference's dispatch (src/boys.cpp:245-294) for diagnostics.
// ---------------------------------------------------------------------------

__global__ void boys_values_kernel(const double2* z, long long count, int nmax, int scaled, BoysTable tab,
                                   const GLRules* gl, double2* out, int* region, DevStatus* st) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const double x = z[i].x, y = z[i].y;
    double2 Sh[BOYS_MAX_ORDER + 1];
    double2 e0;
    if (const int rc = boys_eval(x, y, nmax, tab, gl, Sh, e0)) {
        report(st, rc, i, nmax, x, y);
        return;
    }
    // scaled output: e^{z} F_n = e^{z} e0 Sh
    double2 f = e0;
    if (scaled) {
        double sn, cs;
        sincos(y, &sn, &cs);
        const double m = exp(x);
        f = cmul(f, c2(m * cs, m * sn));
    }
    bool finite = true;
    for (int n = 0; n <= nmax; ++n) {
        const double2 v = cmul(f, Sh[n]);
        finite = finite && isfinite(v.x) && isfinite(v.y);
        out[i * (nmax + 1) + n] = v;
    }
    if (!finite) report(st, -40, i, nmax, x, y);
    if (region) {
        const double mag = sqrt(x * x + y * y);
        int r;
        if (mag <= 0.75)
            r = 0;
        else if (x >= 2.0 * nmax + 60.0 && fabs(y) <= 0.5 * x)
            r = 3;
        else if (x < 0.0)
            r = 2;
        else
            r = 1;
        region[i] = r;
    }
}

cudaError_t launch_boys_values(const double2* z, long long count, int nmax, int scaled, const BoysTable& tab,
                               const GLRules* gl, double2* out, int* region, DevStatus* st, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    boys_values_kernel<<<(unsigned)((count + 127) / 128), 128, 0, s>>>(z, count, nmax, scaled, tab, gl, out,
                                                                          region, st);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// K1: primitive-pair records.  One thread per primitive pair.
// ---------------------------------------------------------------------------

__device__ double log_odd_double_factorial(int l) {
    // ln((2l-1)!!) = l ln 2 + lgamma(l + 1/2) - ln(pi)/2
    if (l == 0) return 0.0;
    return l * 0.69314718055994530942 + lgamma(l + 0.5) - 0.57236494292470008707;
}

// Radial part of the primitive normalisation (src/types.cpp:60-72) without
// the component factor: (2a/pi)^{3/4} (4a)^{l/2}.
__device__ double radial_norm(double a, int l) {
    return exp(0.75 * log(2.0 * a / 3.14159265358979323846) + 0.5 * l * log(4.0 * a));
}

// 1-D real MD coefficients E^{ij}_t, t <= i + j, by repeated raising
// (src/hermite.cpp:8-40): first i raisings about A, then j about B.
__device__ void hermite_1d(int i, int j, double PA, double PB, double inv2p, double* e) {
    const int n = i + j;
    for (int t = 0; t <= n + 1; ++t) e[t] = 0.0;
    e[0] = 1.0;
    for (int step = 0; step < n; ++step) {
        const double d = step < i ? PA : PB;
        // in place, descending t: new e[t] = inv2p e[t-1] + d e[t] + (t+1) e[t+1]
        double upper = 0.0;  // old e[t+1]
        for (int t = step + 1; t >= 0; --t) {
            const double old = e[t];
            e[t] = (t > 0 ? inv2p * e[t - 1] : 0.0) + d * old + (double)(t + 1) * upper;
            upper = old;
        }
    }
}

__global__ void pair_kernel(BasisDev bs, double3 B, double3 O, int npp, const int* pp_a, const int* pp_b,
                            const int* pp_pa, const int* pp_pb, const int* pp_class, const PairClassDev* classes,
                            double* out_p, double* out_Pr, double* out_Pi, double2* out_F, const long long* Eoff,
                            double2* Epool, float2* Epool32, double* out_bound, float4* out_g32) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npp) return;
    const int a = pp_a[i], b = pp_b[i];
    const int pa = bs.primoff[a] + pp_pa[i], pb = bs.primoff[b] + pp_pb[i];
    const double al = bs.exps[pa], be = bs.exps[pb];
    const double A[3] = {bs.center[3 * a], bs.center[3 * a + 1], bs.center[3 * a + 2]};
    const double Bc[3] = {bs.center[3 * b], bs.center[3 * b + 1], bs.center[3 * b + 2]};
    const double p = al + be, mu = al * be / p;
    double P[3], q[3], r2 = 0.0;
    const double Bv[3] = {B.x, B.y, B.z}, Ov[3] = {O.x, O.y, O.z};
    double ka[3], kb[3];
    {
        // London wave vectors k = B x (R - O) / 2 (src/types.cpp:179-186)
        const double da[3] = {A[0] - Ov[0], A[1] - Ov[1], A[2] - Ov[2]};
        const double db[3] = {Bc[0] - Ov[0], Bc[1] - Ov[1], Bc[2] - Ov[2]};
        ka[0] = 0.5 * (Bv[1] * da[2] - Bv[2] * da[1]);
        ka[1] = 0.5 * (Bv[2] * da[0] - Bv[0] * da[2]);
        ka[2] = 0.5 * (Bv[0] * da[1] - Bv[1] * da[0]);
        kb[0] = 0.5 * (Bv[1] * db[2] - Bv[2] * db[1]);
        kb[1] = 0.5 * (Bv[2] * db[0] - Bv[0] * db[2]);
        kb[2] = 0.5 * (Bv[0] * db[1] - Bv[1] * db[0]);
    }
    double qP = 0.0, qq = 0.0;
    for (int x = 0; x < 3; ++x) {
        P[x] = (al * A[x] + be * Bc[x]) / p;
        q[x] = kb[x] - ka[x];
        r2 += (A[x] - Bc[x]) * (A[x] - Bc[x]);
        qP += q[x] * P[x];
        qq += q[x] * q[x];
    }
    const int la = bs.l[a], lb = bs.l[b];
    const bool raw_a = bs.raw[a] != 0, raw_b = bs.raw[b] != 0;
    const double na = raw_a ? 1.0 : radial_norm(al, la);
    const double nb = raw_b ? 1.0 : radial_norm(be, lb);
    // 2 pi^{5/2} / (p q sqrt(p+q)) = sqrt(2 pi^{5/2})/p * sqrt(2 pi^{5/2})/q / sqrt(p+q)
    const double mag = 5.914967172795613 * bs.coefs[pa] * bs.coefs[pb] * na * nb * exp(-mu * r2) / p;
    double sn, cs;
    sincos(-qP, &sn, &cs);
    const double damp = exp(-qq / (4.0 * p));
    out_p[i] = p;
    for (int x = 0; x < 3; ++x) {
        out_Pr[3 * i + x] = P[x];
        out_Pi[3 * i + x] = -0.5 * q[x] / p;
    }
    out_F[i] = c2(mag * damp * cs, mag * damp * sn);
    out_g32[2 * i] = make_float4((float)P[0], (float)P[1], (float)P[2], (float)p);
    out_g32[2 * i + 1] = make_float4((float)(-0.5 * q[0] / p), (float)(-0.5 * q[1] / p), (float)(-0.5 * q[2] / p), 0.0f);

    // complex Hermite coefficients per axis and per component pair
    const PairClassDev pc = classes[pp_class[i]];
    double2* rec = Epool + Eoff[i];
    float2* rec32 = Epool32 + Eoff[i];
    const double inv2p = 0.5 / p;
    int ab = 0;
    double bmax = 0.0;
    for (int xa = la; xa >= 0; --xa)
        for (int ya = la - xa; ya >= 0; --ya) {
            const int ca[3] = {xa, ya, la - xa - ya};
            for (int xb = lb; xb >= 0; --xb)
                for (int yb = lb - xb; yb >= 0; --yb, ++ab) {
                    const int cb[3] = {xb, yb, lb - xb - yb};
                    double2 Et[3][34];
                    int dim[3];
                    double g = 1.0;
                    for (int x = 0; x < 3; ++x) {
                        if (!raw_a) g *= exp(-0.5 * log_odd_double_factorial(ca[x]));
                        if (!raw_b) g *= exp(-0.5 * log_odd_double_factorial(cb[x]));
                        double e[35];
                        hermite_1d(ca[x], cb[x], P[x] - A[x], P[x] - Bc[x], inv2p, e);
                        const int n = ca[x] + cb[x];
                        dim[x] = n + 1;
                        // E~_k = sum_{t>=k} C(t,k) (-i q)^{t-k} E_t
                        for (int k = 0; k <= n; ++k) {
                            double2 acc = c2(0.0, 0.0);
                            double binom = 1.0;        // C(t, k) for t = k
                            double2 pw = c2(1.0, 0.0); // (-i q)^{t-k}
                            for (int t = k; t <= n; ++t) {
                                acc = cadd(acc, cscale(pw, binom * e[t]));
                                pw = cmul(pw, c2(0.0, -q[x]));
                                binom = binom * (double)(t + 1) / (double)(t + 1 - k);
                            }
                            Et[x][k] = acc;
                        }
                    }
                    const int off = pc.boxoff[ab];
                    int e = 0;
                    for (int k = 0; k < dim[0]; ++k)
                        for (int l = 0; l < dim[1]; ++l) {
                            const double2 xy = cmul(Et[0][k], Et[1][l]);
                            for (int m = 0; m < dim[2]; ++m, ++e) {
                                const double2 v = cscale(cmul(xy, Et[2][m]), g);
                                rec[off + e] = v;
                                rec32[off + e] = make_float2((float)v.x, (float)v.y);
                                bmax = fmax(bmax, fabs(v.x) + fabs(v.y));
                            }
                        }
                }
        }
    out_bound[i] = mag * damp * bmax;
}

// Exact primitive Schwarz factor of every primitive pair P = (a pa, b pb):
// bound[P] = sqrt(max over component pairs |(ab|ba)_PP|), from the records of
// P and of its reversed pair (b pb, a pa).  |(ab|cd)_PQ| <= bound[P] bound[Q]
// holds for every component of a primitive quartet (Cauchy-Schwarz in the
// Coulomb metric, the argument of src/eri.cpp:587-619 applied per primitive
// pair).  Pairs with la+lb > 4 get an infinite bound (never screened).
constexpr int BOUND_MAX_LAB = 4;

__global__ void pair_bound_kernel(BasisDev bs, EriDev d, int npp, const int* pp_a, const int* pp_b, const int* pp_pa,
                                  const int* pp_pb, const int* pp_class, const PairClassDev* classes, double* bound) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npp) return;
    const int a = pp_a[i], b = pp_b[i];
    const int la = bs.l[a], lb = bs.l[b];
    if (la + lb > BOUND_MAX_LAB) {
        bound[i] = 1.0e300;
        return;
    }
    const int j = bs.sp_off[b * bs.ns + a] + pp_pb[i] * bs.nprim[a] + pp_pa[i];
    const PairData& pp = d.pairs;
    const int L = 2 * (la + lb);
    const double p = pp.p[i];
    double2 X[3];
    for (int x = 0; x < 3; ++x) X[x] = c2(pp.Pr[3 * i + x] - pp.Pr[3 * j + x], pp.Pi[3 * i + x] - pp.Pi[3 * j + x]);
    const double rho = 0.5 * p;
    const double tre = rho * (X[0].x * X[0].x + X[1].x * X[1].x + X[2].x * X[2].x - X[0].y * X[0].y -
                              X[1].y * X[1].y - X[2].y * X[2].y);
    const double tim = 2.0 * rho * (X[0].x * X[0].y + X[1].x * X[1].y + X[2].x * X[2].y);
    double2 Sh[2 * BOUND_MAX_LAB + 1];
    double2 e0;
    if (boys_eval(tre, tim, L, d.boys, d.gl, Sh, e0)) {
        bound[i] = 1.0e300;
        return;
    }
    double2 C = cmul(cscale(cmul(pp.F[i], pp.F[j]), rsqrt(2.0 * p)), e0);
    constexpr int NR = (2 * BOUND_MAX_LAB + 1) * (2 * BOUND_MAX_LAB + 2) * (2 * BOUND_MAX_LAB + 3) / 6;
    double2 R[NR];
    for (int n = 0; n <= L; ++n) {
        Sh[n] = cmul(C, Sh[n]);
        C = cscale(C, -2.0 * rho);
    }
    R[0] = Sh[L];
    for (int n = L - 1; n >= 0; --n) {
        for (int dg = L - n; dg >= 1; --dg)
            for (int k = dg; k >= 0; --k)
                for (int l = dg - k; l >= 0; --l) {
                    const int m = dg - k - l;
                    double2 v;
                    if (k > 0) {
                        v = cmul(X[0], R[herm_index(k - 1, l, m)]);
                        if (k > 1) v = cmacr(v, (double)(k - 1), R[herm_index(k - 2, l, m)]);
                    } else if (l > 0) {
                        v = cmul(X[1], R[herm_index(0, l - 1, m)]);
                        if (l > 1) v = cmacr(v, (double)(l - 1), R[herm_index(0, l - 2, m)]);
                    } else {
                        v = cmul(X[2], R[herm_index(0, 0, m - 1)]);
                        if (m > 1) v = cmacr(v, (double)(m - 1), R[herm_index(0, 0, m - 2)]);
                    }
                    R[herm_index(k, l, m)] = v;
                }
        R[0] = Sh[n];
    }
    const PairClassDev ci = classes[pp_class[i]], cj = classes[pp_class[j]];
    const double2* Ei = pp.Epool + pp.Eoff[i];
    const double2* Ej = pp.Epool + pp.Eoff[j];
    const int nb = ncart(lb), na = ncart(la);
    double best = 0.0;
    for (int ab = 0; ab < ci.nab; ++ab) {
        const int ca = ab / nb, cb = ab - ca * nb;
        const int ba = cb * na + ca;
        const int oi = ci.boxoff[ab], di = ci.boxdim[ab];
        const int oj = cj.boxoff[ba], dj = cj.boxdim[ba];
        const int ni = (di & 255) * ((di >> 8) & 255) * ((di >> 16) & 255);
        const int nj = (dj & 255) * ((dj >> 8) & 255) * ((dj >> 16) & 255);
        double2 acc = c2(0.0, 0.0);
        for (int e = 0; e < ni; ++e) {
            const uint32_t ke = ci.ent[oi + e];
            const int k1 = ke & 255, l1 = (ke >> 8) & 255, m1 = (ke >> 16) & 255;
            double2 inner = c2(0.0, 0.0);
            for (int f = 0; f < nj; ++f) {
                const uint32_t kf = cj.ent[oj + f];
                const int k2 = kf & 255, l2 = (kf >> 8) & 255, m2 = (kf >> 16) & 255;
                double2 ev = Ej[oj + f];
                if ((k2 + l2 + m2) & 1) ev = c2(-ev.x, -ev.y);
                inner = cmac(inner, ev, R[herm_index(k1 + k2, l1 + l2, m1 + m2)]);
            }
            acc = cmac(acc, Ei[oi + e], inner);
        }
        best = fmax(best, sqrt(acc.x * acc.x + acc.y * acc.y));
    }
    bound[i] = sqrt(best) * (1.0 + 1.0e-10) + 1.0e-300;
}

cudaError_t launch_pair_precompute(const BasisDev& basis, const double* B, const double* O, int npp, const int* pp_a,
                                   const int* pp_b, const int* pp_pa, const int* pp_pb, const int* pp_class,
                                   const PairClassDev* classes, double* p, double* Pr, double* Pi, double2* F,
                                   const long long* Eoff, double2* Epool, float2* Epool32, double* bound, float4* g32,
                                   const EriDev* dev_for_bounds, cudaStream_t s) {
    if (npp <= 0) return cudaSuccess;
    pair_kernel<<<(npp + 63) / 64, 64, 0, s>>>(basis, make_double3(B[0], B[1], B[2]), make_double3(O[0], O[1], O[2]),
                                               npp, pp_a, pp_b, pp_pa, pp_pb, pp_class, classes, p, Pr, Pi, F, Eoff,
                                               Epool, Epool32, bound, g32);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !dev_for_bounds) return e;
    pair_bound_kernel<<<(npp + 63) / 64, 64, 0, s>>>(basis, *dev_for_bounds, npp, pp_a, pp_b, pp_pa, pp_pb, pp_class,
                                                     classes, bound);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// K3/K4: class-generic quartet kernel, one warp per shell quartet.
//
// Phase 1 (lane-parallel): up to B1 primitive quartets (P, Q..Q+B1) at a
//   time, one per lane: T = rho X'^2, Boys, seeds, and the in-place Rh
//   recurrence into the lane's column of shared memory.
// Phase 2 (warp-cooperative, per primitive quartet): ket transform
//   W[K][cd] += sum_{K' in box(cd)} E~cd_K' Rh_{K+K'}, accumulated over the
//   ket primitive pairs; then, once per bra primitive pair, the bra
//   transform out[ab][cd] += sum_{K in box(ab)} E~ab_K W[K][cd] straight
//   into the caller's output block (lane-owned entries, coalesced).
// The sign (-1)^{|K'|} of the ket side is applied to the ket records when
// they are read as kets (ket_sign below).
// ---------------------------------------------------------------------------

__constant__ double c_int[40];  // c_int[k] = k, avoids int->double conversions in inner loops

// FP64 quantities of primitive quartet (ip, iq): the complex centre
// separation X' = P' - Q', rho = pq / (p + q), the Boys argument
// T = rho X'.X' and C = F_ab F_cd / sqrt(p + q).
struct QuartetArgs {
    double2 X[3], C;
    double rho, tre, tim;
};
__device__ __forceinline__ QuartetArgs quartet_args(const PairData& pp, int ip, int iq) {
    QuartetArgs a;
    const double p = pp.p[ip], q = pp.p[iq];
    for (int x = 0; x < 3; ++x)
        a.X[x] = c2(pp.Pr[3 * ip + x] - pp.Pr[3 * iq + x], pp.Pi[3 * ip + x] - pp.Pi[3 * iq + x]);
    const double r = rsqrt(p + q);
    a.rho = p * q * r * r;
    const double2* X = a.X;
    a.tre = a.rho * (fma(X[0].x, X[0].x, fma(X[1].x, X[1].x, X[2].x * X[2].x)) -
                     fma(X[0].y, X[0].y, fma(X[1].y, X[1].y, X[2].y * X[2].y)));
    a.tim = 2.0 * a.rho * fma(X[0].x, X[0].y, fma(X[1].x, X[1].y, X[2].x * X[2].y));
    a.C = cscale(cmul(pp.F[ip], pp.F[iq]), r);
    return a;
}

// FP64 seeds C (-2 rho)^n F_n(T) into Sh[0..L].  Boys failures are reported
// through the status word and give zero seeds.
__device__ __forceinline__ void quartet_seeds_rt(const EriDev& d, int L, const QuartetArgs& a, double2* Sh,
                                                 long long item) {
    double2 e0;
    double2 C = a.C;
    if (const int rc = boys_eval(a.tre, a.tim, L, d.boys, d.gl, Sh, e0)) {
        report(d.status, rc, item, L, a.tre, a.tim);
        C = c2(0.0, 0.0);
        e0 = c2(0.0, 0.0);
        for (int n = 0; n <= L; ++n) Sh[n] = c2(0.0, 0.0);
    }
    C = cmul(C, e0);
    const double m2r = -2.0 * a.rho;
    for (int n = 0; n <= L; ++n) {
        Sh[n] = cmul(C, Sh[n]);
        C = cscale(C, m2r);
    }
}

// In-place descending-level Hermite recurrence into one column (stride
// apart) of the shared table, FP64 (T = double2) or FP32 (T = float2).
template <typename T>
__device__ __forceinline__ T tmul(T a, T b);
template <>
__device__ __forceinline__ double2 tmul(double2 a, double2 b) { return cmul(a, b); }
template <>
__device__ __forceinline__ float2 tmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 tmacr(double2 c, int k, double2 a) { return cmacr(c, c_int[k], a); }
__device__ __forceinline__ float2 tmacr(float2 c, int k, float2 a) {
    return make_float2(fmaf((float)k, a.x, c.x), fmaf((float)k, a.y, c.y));
}
__device__ __forceinline__ double2 tmac(double2 c, double2 a, double2 b) { return cmac(c, a, b); }
__device__ __forceinline__ float2 tmac(float2 c, float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}

template <typename T>
__device__ __forceinline__ void hermite_rec(int L, const T* seed, const T* X, T* col, int stride) {
    col[0] = seed[L];
    for (int n = L - 1; n >= 0; --n) {
        for (int dg = L - n; dg >= 1; --dg) {
            for (int k = dg; k >= 0; --k) {
                for (int l = dg - k; l >= 0; --l) {
                    const int m = dg - k - l;
                    int axis, pw, i1, i2;
                    if (k > 0) {
                        axis = 0;
                        pw = k;
                        i1 = herm_index(k - 1, l, m);
                        i2 = k > 1 ? herm_index(k - 2, l, m) : 0;
                    } else if (l > 0) {
                        axis = 1;
                        pw = l;
                        i1 = herm_index(0, l - 1, m);
                        i2 = l > 1 ? herm_index(0, l - 2, m) : 0;
                    } else {
                        axis = 2;
                        pw = m;
                        i1 = herm_index(0, 0, m - 1);
                        i2 = m > 1 ? herm_index(0, 0, m - 2) : 0;
                    }
                    T v = tmul(X[axis], col[i1 * stride]);
                    if (pw > 1) v = tmacr(v, pw - 1, col[i2 * stride]);
                    col[herm_index(k, l, m) * stride] = v;
                }
            }
        }
        col[0] = seed[n];
    }
}

// The same recurrence driven by the precomputed step list of order L (every
// lane reads the same step: one broadcast load instead of the index
// arithmetic of the nested loops).
template <typename T>
__device__ __forceinline__ void hermite_rec_plan(const int2* plan, int nsteps, int L, const T* seed, const T* X, T* col,
                                                 int stride) {
    col[0] = seed[L];
    for (int i = 0; i < nsteps; ++i) {
        const int2 st = __ldg(&plan[i]);
        if (st.y & (1 << 22)) {
            col[0] = seed[(st.y >> 23) & 63];
            continue;
        }
        const int dst = st.x & 0xffff, s1 = (st.x >> 16) & 0xffff;
        const int s2 = st.y & 0x3fff, axis = (st.y >> 14) & 3, coef = (st.y >> 16) & 63;
        const T xa = axis == 0 ? X[0] : (axis == 1 ? X[1] : X[2]);
        T v = tmul(xa, col[s1 * stride]);
        if (coef > 0) v = tmacr(v, coef, col[s2 * stride]);
        col[dst * stride] = v;
    }
}

template <typename T>
__device__ __forceinline__ void hermite_rec_any(const EriDev& d, int L, const T* seed, const T* X, T* col, int stride) {
    if (L >= 1 && L <= REC_PLAN_MAX) {
        const int o = d.rec_plan_off[L];
        hermite_rec_plan<T>(d.rec_plan + o, d.rec_plan_off[L + 1] - o, L, seed, X, col, stride);
    } else {
        hermite_rec<T>(L, seed, X, col, stride);
    }
}

// Per-warp shared layout of quartet_kernel (all offsets in bytes).  R holds
// B1 + 1 columns (the last one is the cooperative recurrence's second
// buffer); `seed` holds one entry's seeds and X' for the cooperative path.
// FP32 entries of a mixed-precision batch keep their table in R too: the
// float2 of row r sits in the first half of the 16-byte slot of column j.
struct WarpSmem {
    size_t R, W, W32, queue, flag, eoff, seed, stage, total;
};
// Per-warp shared layout.  Batched mode: R columns of all B1 entries
// (stride B1 + 1) and one seed area; stream mode: a two-column R buffer and
// the seeds and X' of every batch entry (L + 4 slots each).
// stage32: the E~ staging also holds the FP32 copy of a record (mixed
// precision when this kernel takes FP32 entries; otherwise only the FP64
// record is staged and the FP32 half is not allocated)
__host__ __device__ inline WarpSmem warp_smem(int NL, int B1, int Nab, int CH, bool mixed, int stage_e, int stream,
                                              int L, bool stage32) {
    WarpSmem w;
    const size_t B1p = B1 + 1;
    w.R = 0;
    w.W = w.R + (size_t)NL * (stream ? 2 : B1p) * 16;
    w.W32 = w.W + (size_t)Nab * CH * 16;
    w.queue = w.W32 + (mixed ? (((size_t)Nab * CH * 8 + 15) / 16) * 16 : 0);
    w.flag = w.queue + (((size_t)B1 * 4 + 15) / 16) * 16;
    w.eoff = w.flag + (((size_t)B1 * 4 + 15) / 16) * 16;
    w.seed = w.eoff + (((size_t)B1 * 8 + 15) / 16) * 16;
    w.stage = w.seed + (stream ? (size_t)B1 * (L + 4) : (size_t)(BOYS_MAX_ORDER + 1 + 3)) * 16;
    // FP64 record (16 B per word) followed by its FP32 copy (8 B per word)
    w.total = w.stage + (((size_t)stage_e * (stage32 ? 24 : 16) + 15) / 16) * 16;
    return w;
}

// Block-shared class tables (32-bit words): ket boxoff[ncd], ket
// boxdim[ncd], ket box entries as Hermite indices with the (-1)^{|K'|} sign in
// bit 16 [Etot_ket], bra boxoff[nab], bra boxdim[nab], bra box entries as
// Hermite indices [Etot_bra], and hsum[K][K'] = index of K + K' for every bra
// row K < Nab and ket row K' < herm_count(Lcd).
__host__ __device__ inline int class_tab_words(const QuartetClass& qc) {
    return 2 * qc.ket.nab + qc.ket.Etot + 2 * qc.bra.nab + qc.bra.Etot + qc.Nab * herm_count(qc.ket.Lab);
}
struct ClassTabs {
    const int* kbo;
    const int* kbd;
    const uint32_t* kh;
    const int* bbo;
    const int* bbd;
    const uint32_t* bh;
    const int* hsum;
    int ncdh;
};

// Warp-cooperative Hermite recurrence of one primitive quartet: level n
// (entries of total degree <= L - n) from level n + 1, all entries of a
// level in parallel across the lanes, ping-ponging between columns j and s
// of the shared table so that level 0 ends in column j.
template <typename T>
__device__ __forceinline__ void coop_rec(int L, const T* seed, const T* X, T* R, int B1p, int j, int s,
                                         const uint32_t* herm_xyz, int lane) {
    int cur = (L % 2 == 0) ? j : s;
    if (lane == 0) R[cur] = seed[L];
    __syncwarp();
    for (int n = L - 1; n >= 0; --n) {
        const int nxt = cur == j ? s : j;
        const int cnt = herm_count(L - n);
        for (int e = lane; e < cnt; e += 32) {
            T v;
            if (e == 0) {
                v = seed[n];
            } else {
                const uint32_t kx = __ldg(&herm_xyz[e]);
                const int k = kx & 255, l = (kx >> 8) & 255, m = (kx >> 16) & 255;
                int axis, pw, i1, i2;
                if (k > 0) {
                    axis = 0;
                    pw = k;
                    i1 = herm_index(k - 1, l, m);
                    i2 = k > 1 ? herm_index(k - 2, l, m) : 0;
                } else if (l > 0) {
                    axis = 1;
                    pw = l;
                    i1 = herm_index(0, l - 1, m);
                    i2 = l > 1 ? herm_index(0, l - 2, m) : 0;
                } else {
                    axis = 2;
                    pw = m;
                    i1 = herm_index(0, 0, m - 1);
                    i2 = m > 1 ? herm_index(0, 0, m - 2) : 0;
                }
                v = tmul(X[axis], R[i1 * B1p + cur]);
                if (pw > 1) v = tmacr(v, pw - 1, R[i2 * B1p + cur]);
            }
            R[e * B1p + nxt] = v;
        }
        __syncwarp();
        cur = nxt;
    }
}

// Work split of a transform with `items` work items: J lanes share an item
// (the largest power of two with items * J <= 32; 1 when items >= 16), so
// that small classes still fill the warp.  Groups of J lanes are aligned.
__device__ __forceinline__ int lanes_per_item(int items) {
    int J = 1;
    while (J < 32 && items * J * 2 <= 32) J *= 2;
    return J;
}
__device__ __forceinline__ double2 group_sum(double2 v, int J) {
    for (int off = J >> 1; off > 0; off >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, off);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, off);
    }
    return v;
}
__device__ __forceinline__ float2 group_sum(float2 v, int J) {
    for (int off = J >> 1; off > 0; off >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, off);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, off);
    }
    return v;
}

// Ket transform of the batch entries j0..j1-1 (one run with the same bra
// pair) into W (FP64 entries) and W32 (FP32 entries):
//   W[K][cd] += sum_j sum_{K' in box(cd)} (-1)^{|K'|} E~cd_j[K'] Rh_j[K + K'].
// Entry by entry, the warp first copies the entry's ket E~ record into its
// staging buffer with one coalesced load (stg; null: read it from global
// memory), then every work item -- KT consecutive Hermite rows K of one ket
// component cd, its box entries split over the item's J lanes -- contracts
// it against the entry's R column (FP32 entries: the float2 in the first half
// of each 16-byte slot of R, R32[(row B1p + j) 2]).  eoff[j]: E~ record of the
// entry's ket pair; flag[j]: 0 FP32, 1 FP64.
template <int KT>
__device__ __forceinline__ void step_k_run(const QuartetClass& qc, const ClassTabs& tb, const uint32_t* herm_xyz,
                                           const PairData& pp, const double2* R, const float2* R32, int B1p,
                                           const int* flag, const long long* eoff, int j0, int j1, double2* W,
                                           float2* W32, double2* stg, int c0, int chn, int lane) {
    const int nkb = (qc.Nab + KT - 1) / KT;
    const int I = nkb * chn;
    const int J = lanes_per_item(I);
    const int rounds = (I * J + 31) / 32;
    float2* stg32 = reinterpret_cast<float2*>(stg + qc.stage_e);
    for (int jj = j0; jj < j1; ++jj) {
        const int f = flag[jj];
        const bool is64 = f == 1;
        const double2* E64 = pp.Epool + eoff[jj];
        const float2* E32 = pp.Epool32 + eoff[jj];
        if (stg) {
            if (is64)
                for (int i = lane; i < qc.ket.Etot; i += 32) stg[i] = __ldg(&E64[i]);
            else
                for (int i = lane; i < qc.ket.Etot; i += 32) stg32[i] = __ldg(&E32[i]);
            __syncwarp();
            E64 = stg;
            E32 = stg32;
        }
        for (int rd = 0; rd < rounds; ++rd) {
            const int slot = rd * 32 + lane;
            const int it = slot / J, sub = slot - it * J;
            const bool act = it < I;
            double2 a64[KT];
            float2 a32[KT];
#pragma unroll
            for (int u = 0; u < KT; ++u) {
                a64[u] = c2(0.0, 0.0);
                a32[u] = make_float2(0.0f, 0.0f);
            }
            int kb = 0, cdl = 0;
            if (act && tb.hsum) {
                // table path: R row of (K, K') = hsum[K][K']
                kb = it / chn;
                cdl = it - kb * chn;
                const int cd = c0 + cdl;
                int hb[KT];
#pragma unroll
                for (int u = 0; u < KT; ++u) {
                    const int K = kb * KT + u;
                    hb[u] = (K < qc.Nab ? K : 0) * tb.ncdh;
                }
                const int bo = tb.kbo[cd];
                const int bd = tb.kbd[cd];
                const int nbox = (bd & 255) * ((bd >> 8) & 255) * ((bd >> 16) & 255);
                for (int e = sub; e < nbox; e += J) {
                    const uint32_t kk = tb.kh[bo + e];
                    const int Kp = kk & 0xffff;
                    const bool neg = kk >> 16;
                    if (is64) {
                        double2 ev = E64[bo + e];
                        if (neg) ev = c2(-ev.x, -ev.y);
#pragma unroll
                        for (int u = 0; u < KT; ++u) a64[u] = cmac(a64[u], ev, R[tb.hsum[hb[u] + Kp] * B1p + jj]);
                    } else {
                        float2 ev = E32[bo + e];
                        if (neg) ev = make_float2(-ev.x, -ev.y);
#pragma unroll
                        for (int u = 0; u < KT; ++u) a32[u] = tmac(a32[u], ev, R32[(tb.hsum[hb[u] + Kp] * B1p + jj) * 2]);
                    }
                }
            } else if (act) {
                kb = it / chn;
                cdl = it - kb * chn;
                const int cd = c0 + cdl;
                int bk[KT], bl[KT], bm[KT];
#pragma unroll
                for (int u = 0; u < KT; ++u) {
                    const int K = kb * KT + u;
                    const uint32_t kx = herm_xyz[K < qc.Nab ? K : 0];
                    bk[u] = kx & 255;
                    bl[u] = (kx >> 8) & 255;
                    bm[u] = (kx >> 16) & 255;
                }
                const int bo = qc.ket.boxoff[cd];
                const int bd = qc.ket.boxdim[cd];
                const int nbox = (bd & 255) * ((bd >> 8) & 255) * ((bd >> 16) & 255);
                for (int e = sub; e < nbox; e += J) {
                    const uint32_t ke = qc.ket.ent[bo + e];
                    const int k2 = ke & 255, l2 = (ke >> 8) & 255, m2 = (ke >> 16) & 255;
                    const bool neg = (k2 + l2 + m2) & 1;
                    if (is64) {
                        double2 ev = E64[bo + e];
                        if (neg) ev = c2(-ev.x, -ev.y);
#pragma unroll
                        for (int u = 0; u < KT; ++u)
                            a64[u] = cmac(a64[u], ev, R[herm_index(bk[u] + k2, bl[u] + l2, bm[u] + m2) * B1p + jj]);
                    } else {
                        float2 ev = E32[bo + e];
                        if (neg) ev = make_float2(-ev.x, -ev.y);
#pragma unroll
                        for (int u = 0; u < KT; ++u)
                            a32[u] = tmac(a32[u], ev, R32[(herm_index(bk[u] + k2, bl[u] + l2, bm[u] + m2) * B1p + jj) * 2]);
                    }
                }
            }
            if (J > 1) {
#pragma unroll
                for (int u = 0; u < KT; ++u) {
                    if (is64)
                        a64[u] = group_sum(a64[u], J);
                    else
                        a32[u] = group_sum(a32[u], J);
                }
            }
            if (act && sub == 0) {
#pragma unroll
                for (int u = 0; u < KT; ++u) {
                    const int K = kb * KT + u;
                    if (K < qc.Nab) {
                        if (is64) {
                            W[K * qc.CH + cdl] = cadd(W[K * qc.CH + cdl], a64[u]);
                        } else {
                            float2& w = W32[K * qc.CH + cdl];
                            w.x += a32[u].x;
                            w.y += a32[u].y;
                        }
                    }
                }
            }
        }
        if (stg) __syncwarp();  // the next entry overwrites the staging buffer
    }
}

__device__ __forceinline__ void step_k_any(const QuartetClass& qc, const ClassTabs& tb, const uint32_t* herm_xyz,
                                           const PairData& pp, const double2* R, const float2* R32, int B1p,
                                           const int* flag, const long long* eoff, int j0, int j1, double2* W,
                                           float2* W32, double2* stg, int c0, int chn, int lane) {
    if (qc.KT == 4)
        step_k_run<4>(qc, tb, herm_xyz, pp, R, R32, B1p, flag, eoff, j0, j1, W, W32, stg, c0, chn, lane);
    else if (qc.KT == 2)
        step_k_run<2>(qc, tb, herm_xyz, pp, R, R32, B1p, flag, eoff, j0, j1, W, W32, stg, c0, chn, lane);
    else
        step_k_run<1>(qc, tb, herm_xyz, pp, R, R32, B1p, flag, eoff, j0, j1, W, W32, stg, c0, chn, lane);
}

// Bra transform of W (FP64) and W32 (FP32) into the task's output block:
//   out[ab][cd] += sum_{K in box(ab)} E~ab[K] W[K][cd].
// The bra E~ record (FP64 and/or FP32) is first copied into the warp's
// staging buffer (stg; null: read from global memory).  A work item is CT
// consecutive ket components of one bra component ab (the chunk length is a
// multiple of CT); its box entries are split over the item's J lanes.  FP32
// partial sums are added in FP64.
template <int CT>
__device__ __forceinline__ void step_b(const EriDev& d, const QuartetClass& qc, const ClassTabs& tb, const Task& tg,
                                       int ip, double2* W, float2* W32, bool use64, bool use32, double2* stg, int c0,
                                       int chn, int lane) {
    const int nab = qc.bra.nab;
    const int ncb = ncart(qc.bra.lb), ncdd = ncart(qc.ket.lb);
    const double2* Ea = d.pairs.Epool + d.pairs.Eoff[ip];
    const float2* Ea32 = d.pairs.Epool32 + d.pairs.Eoff[ip];
    if (stg) {
        float2* stg32 = reinterpret_cast<float2*>(stg + qc.stage_e);
        if (use64)
            for (int i = lane; i < qc.bra.Etot; i += 32) stg[i] = __ldg(&Ea[i]);
        if (use32)
            for (int i = lane; i < qc.bra.Etot; i += 32) stg32[i] = __ldg(&Ea32[i]);
        __syncwarp();
        Ea = stg;
        Ea32 = stg32;
    }
    const int nct = chn / CT;
    const int I = nab * nct;
    const int J = lanes_per_item(I);
    const int rounds = (I * J + 31) / 32;
    for (int rd = 0; rd < rounds; ++rd) {
        const int slot = rd * 32 + lane;
        const int it = slot / J, sub = slot - it * J;
        const bool act = it < I;
        double2 acc[CT];
        float2 acc32[CT];
#pragma unroll
        for (int u = 0; u < CT; ++u) {
            acc[u] = c2(0.0, 0.0);
            acc32[u] = make_float2(0.0f, 0.0f);
        }
        int ab = 0, cdl0 = 0;
        if (act) {
            ab = it / nct;
            cdl0 = (it - ab * nct) * CT;
            const int bo = tb.hsum ? tb.bbo[ab] : qc.bra.boxoff[ab];
            const int bd = tb.hsum ? tb.bbd[ab] : qc.bra.boxdim[ab];
            const int nbox = (bd & 255) * ((bd >> 8) & 255) * ((bd >> 16) & 255);
            auto row = [&](int e) -> int {
                if (tb.hsum) return (int)tb.bh[bo + e];
                const uint32_t ke = qc.bra.ent[bo + e];
                return herm_index(ke & 255, (ke >> 8) & 255, (ke >> 16) & 255);
            };
            if (use32) {
                for (int e = sub; e < nbox; e += J) {
                    const int K = row(e);
                    const float2 ea32 = Ea32[bo + e];
#pragma unroll
                    for (int u = 0; u < CT; ++u) acc32[u] = tmac(acc32[u], ea32, W32[K * qc.CH + cdl0 + u]);
                }
            }
            if (use64) {
                for (int e = sub; e < nbox; e += J) {
                    const int K = row(e);
                    const double2 ea = Ea[bo + e];
#pragma unroll
                    for (int u = 0; u < CT; ++u) acc[u] = cmac(acc[u], ea, W[K * qc.CH + cdl0 + u]);
                }
            }
        }
        if (J > 1) {
#pragma unroll
            for (int u = 0; u < CT; ++u) {
                if (use64) acc[u] = group_sum(acc[u], J);
                if (use32) acc32[u] = group_sum(acc32[u], J);
            }
        }
        if (act && sub == 0) {
            const int ca = ab / ncb, cb = ab - ca * ncb;
            double2* ob = d.out + tg.out_off + (long long)ca * tg.st[0] + (long long)cb * tg.st[1];
#pragma unroll
            for (int u = 0; u < CT; ++u) {
                const int cd = c0 + cdl0 + u;
                const int cc = cd / ncdd, cdd = cd - cc * ncdd;
                const double2 a = use32 ? cadd(acc[u], c2((double)acc32[u].x, (double)acc32[u].y)) : acc[u];
                double2* o = ob + (long long)cc * tg.st[2] + (long long)cdd * tg.st[3];
                *o = cadd(*o, a);
            }
        }
    }
    if (stg) __syncwarp();  // the staging buffer is reused by the next transform
}

__device__ __forceinline__ void step_b_any(const EriDev& d, const QuartetClass& qc, const ClassTabs& tb,
                                           const Task& tg, int ip, double2* W, float2* W32, bool use64, bool use32,
                                           double2* stg, int c0, int chn, int lane) {
    switch (qc.CT) {
        case 4: step_b<4>(d, qc, tb, tg, ip, W, W32, use64, use32, stg, c0, chn, lane); break;
        case 3: step_b<3>(d, qc, tb, tg, ip, W, W32, use64, use32, stg, c0, chn, lane); break;
        case 2: step_b<2>(d, qc, tb, tg, ip, W, W32, use64, use32, stg, c0, chn, lane); break;
        default: step_b<1>(d, qc, tb, tg, ip, W, W32, use64, use32, stg, c0, chn, lane); break;
    }
}

// Seeds of one primitive quartet: returns 1 (FP64 seeds in Sh), 0 (FP32
// seeds in S32) or 2 (FP32 wanted but the seeds leave the FP32 range: FP64
// seeds in Sh).  For an FP32 quartet (want32) the Boys function runs in FP32
// in its asymptotic sector and in FP64 elsewhere.
__device__ __forceinline__ int entry_seeds(const EriDev& d, int L, int want32, const QuartetArgs& qa, double2* Sh,
                                           float2* S32, long long item) {
    if (!want32) {
        quartet_seeds_rt(d, L, qa, Sh, item);
        return 1;
    }
    if (seeds32(qa.C, qa.rho, qa.tre, qa.tim, L, S32)) return 0;
    quartet_seeds_rt(d, L, qa, Sh, item);
    bool ok = true;
    for (int n = 0; n <= L; ++n) {
        ok = ok && fabs(Sh[n].x) + fabs(Sh[n].y) < 1.0e25;
        S32[n] = make_float2((float)Sh[n].x, (float)Sh[n].y);
    }
    return ok ? 0 : 2;
}

// MINB: blocks of 128 threads the register budget must leave room for (2:
// up to 255 registers per thread, no spills; 4: 128 registers, a few spills,
// twice the resident warps); the autotuner picks per class.
template <int MINB>
__global__ void __launch_bounds__(128, MINB) quartet_kernel(EriDev d, QuartetClass qc) {
    extern __shared__ double2 sm[];
    // class tables into block-shared memory, read by every warp of the block
    ClassTabs tabs{};
    if (qc.tab_words > 0) {
        int* t = reinterpret_cast<int*>(sm);
        const int ncdh = herm_count(qc.ket.Lab);
        int* kbo = t;
        int* kbd = kbo + qc.ket.nab;
        uint32_t* kh = reinterpret_cast<uint32_t*>(kbd + qc.ket.nab);
        int* bbo = reinterpret_cast<int*>(kh + qc.ket.Etot);
        int* bbd = bbo + qc.bra.nab;
        uint32_t* bh = reinterpret_cast<uint32_t*>(bbd + qc.bra.nab);
        int* hsum = reinterpret_cast<int*>(bh + qc.bra.Etot);
        for (int i = threadIdx.x; i < qc.ket.nab; i += blockDim.x) {
            kbo[i] = qc.ket.boxoff[i];
            kbd[i] = qc.ket.boxdim[i];
        }
        for (int i = threadIdx.x; i < qc.ket.Etot; i += blockDim.x) {
            const uint32_t ke = qc.ket.ent[i];
            const int k = ke & 255, l = (ke >> 8) & 255, m = (ke >> 16) & 255;
            kh[i] = (uint32_t)herm_index(k, l, m) | ((uint32_t)((k + l + m) & 1) << 16);
        }
        for (int i = threadIdx.x; i < qc.bra.nab; i += blockDim.x) {
            bbo[i] = qc.bra.boxoff[i];
            bbd[i] = qc.bra.boxdim[i];
        }
        for (int i = threadIdx.x; i < qc.bra.Etot; i += blockDim.x) {
            const uint32_t ke = qc.bra.ent[i];
            bh[i] = (uint32_t)herm_index(ke & 255, (ke >> 8) & 255, (ke >> 16) & 255);
        }
        for (int i = threadIdx.x; i < qc.Nab * ncdh; i += blockDim.x) {
            const int K = i / ncdh, Kp = i - K * ncdh;
            const uint32_t a = d.herm_xyz[K], b = d.herm_xyz[Kp];
            hsum[i] = herm_index((a & 255) + (b & 255), ((a >> 8) & 255) + ((b >> 8) & 255),
                                 ((a >> 16) & 255) + ((b >> 16) & 255));
        }
        __syncthreads();
        tabs = ClassTabs{kbo, kbd, kh, bbo, bbd, bh, hsum, ncdh};
    }
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    const int B1p = qc.B1 + 1;
    const float skip = d.skip_cut, cut32 = d.fp32_cut;
    // with the FP32 lane kernel in charge of the FP32 entries, this kernel
    // takes only the entries at or above the FP32 cutoff
    const float skip64 = qc.no32 ? fmaxf(skip, cut32) : skip;
    const WarpSmem lay =
        warp_smem(qc.NL, qc.B1, qc.Nab, qc.CH, cut32 > 0.0f, qc.stage_e, qc.stream, qc.L, cut32 > 0.0f && !qc.no32);
    const size_t tab_bytes = (((size_t)qc.tab_words * 4 + 15) / 16) * 16;
    char* base = reinterpret_cast<char*>(sm) + tab_bytes + (size_t)wib * lay.total;
    double2* R = reinterpret_cast<double2*>(base + lay.R);
    double2* W = reinterpret_cast<double2*>(base + lay.W);
    float2* W32 = reinterpret_cast<float2*>(base + lay.W32);
    int* queue = reinterpret_cast<int*>(base + lay.queue);
    int* flag = reinterpret_cast<int*>(base + lay.flag);
    long long* eoff = reinterpret_cast<long long*>(base + lay.eoff);  // E~ record of each entry's ket pair
    double2* sseed = reinterpret_cast<double2*>(base + lay.seed);  // [L+1] seeds, then X'[3] (per entry: stream)
    const int sstride = qc.L + 4;  // stream mode: seed slots per entry
    double2* stg = qc.stage_e > 0 ? reinterpret_cast<double2*>(base + lay.stage) : nullptr;  // E~ staging
    const int nab = qc.bra.nab, ncd = qc.ket.nab;
    const int ncb = ncart(qc.bra.lb), ncdd = ncart(qc.ket.lb);
    const PairData& pp = d.pairs;
    // Mixed precision runs in the same batches as FP64: every entry carries its
    // own precision (FP32 below cut32), FP32 R columns share the slots of the
    // FP64 ones (a float2 in each 16-byte slot), and W / W32 accumulate side by
    // side, so batches stay dense and each bra pair is contracted once.
    const bool mixed = cut32 > 0.0f;
    float2* const R32s = reinterpret_cast<float2*>(R);  // FP32 column j: R32s + 2 j, stride 2 B1p
    unsigned long long cnt64 = 0, cnt32 = 0;
    // A warp takes one work unit: a group of tasks with equal primitive
    // counts and one chunk of ket components (chunks of a group run on
    // different warps and write disjoint output entries).  It walks the
    // group's primitive quartets as one stream (task g, bra pair P, ket pair
    // Q; pairs in decreasing Schwarz order); each pass compacts the entries
    // of its precision into batches of up to B1 with a ballot, so screened or
    // other-precision entries cost no FP64 issue slots.
    const int nunit = qc.ngroup * qc.nchunk;
    for (int unit = blockIdx.x * wpb + wib; unit < nunit; unit += gridDim.x * wpb) {
        const int grp = unit / qc.nchunk;
        const int c0 = (unit - grp * qc.nchunk) * qc.CH;
        const unsigned first_chunk = c0 == 0;
        const int chn = min(qc.CH, ncd - c0);
        const int2 gi = qc.groups[grp];
        const Task t0 = qc.tasks[gi.x];
        const int Kab = d.basis.nprim[t0.sa] * d.basis.nprim[t0.sb];
        const int Kcd = d.basis.nprim[t0.sc] * d.basis.nprim[t0.sd];
        const int KK = Kab * Kcd;
        const int S = gi.y * KK;
        for (int g = 0; g < gi.y; ++g) {
            const Task tg = qc.tasks[gi.x + g];
            for (int it = lane; it < nab * chn; it += 32) {
                const int ab = it / chn, cd = c0 + (it - ab * chn);
                const int ca = ab / ncb, cb = ab - ca * ncb, cc = cd / ncdd, cdd = cd - cc * ncdd;
                d.out[tg.out_off + (long long)ca * tg.st[0] + (long long)cb * tg.st[1] + (long long)cc * tg.st[2] +
                      (long long)cdd * tg.st[3]] = c2(0.0, 0.0);
            }
        }
        __syncwarp();
        {
            for (int it = lane; it < qc.Nab * qc.CH; it += 32) {
                W[it] = c2(0.0, 0.0);
                if (mixed) W32[it] = make_float2(0.0f, 0.0f);
            }
            int cur = -1;  // g * Kab + P of the accumulating bra pair
            bool any64 = false, any32 = false;  // precisions accumulated into W / W32 for `cur`
            int cursor = 0;
            while (cursor < S) {
                // assemble up to B1 entries of this pass
                int nb = 0;
                __syncwarp();
                while (nb < qc.B1 && cursor < S) {
                    const int idx = cursor + lane;
                    bool valid = false;
                    if (idx < S) {
                        const int g = idx / KK, r = idx - g * KK;
                        const int P = r / Kcd, Q = r - P * Kcd;
                        const Task tg = qc.tasks[gi.x + g];
                        const int op = tg.pab + P;
                        const int oq = tg.pcd + Q;
                        const float b = pp.sbound[op] * pp.sbound[oq];
                        valid = b >= skip64;
                    }
                    const unsigned mask = __ballot_sync(0xffffffffu, valid);
                    const int cnt = __popc(mask);
                    const int take = min(cnt, qc.B1 - nb);
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
                if (qc.stream) {
                    // seeds and X' of every entry, lane-parallel; the
                    // recurrences run per entry in phase 2
                    if (lane < nb) {
                        const int idx = queue[lane];
                        const int g = idx / KK, r = idx - g * KK;
                        const int P = r / Kcd, Q = r - P * Kcd;
                        const Task tg = qc.tasks[gi.x + g];
                        const int ip = pp.order[tg.pab + P];
                        const int iq = pp.order[tg.pcd + Q];
                        const QuartetArgs qa = quartet_args(pp, ip, iq);
                        double2 Sh[BOYS_MAX_ORDER + 1];
                        float2 S32[BOYS_MAX_ORDER + 1];
                        const bool want32 = mixed && pp.sbound[tg.pab + P] *
                                                             pp.sbound[tg.pcd + Q] <
                                                         cut32;
                        int f = entry_seeds(d, qc.L, want32 ? 1 : 0, qa, Sh, S32, gi.x + g);
                        if (f == 2) f = 1;  // FP32 seeds out of range: this entry runs in FP64
                        double2* es = sseed + (size_t)lane * sstride;
                        if (f == 1) {
                            for (int n = 0; n <= qc.L; ++n) es[n] = Sh[n];
                            for (int x = 0; x < 3; ++x) es[qc.L + 1 + x] = qa.X[x];
                            cnt64 += first_chunk;
                        } else {
                            float2* s32 = reinterpret_cast<float2*>(es);
                            for (int n = 0; n <= qc.L; ++n) s32[n] = S32[n];
                            for (int x = 0; x < 3; ++x)
                                s32[qc.L + 1 + x] = make_float2((float)qa.X[x].x, (float)qa.X[x].y);
                            cnt32 += first_chunk;
                        }
                        flag[lane] = f;
                        eoff[lane] = pp.Eoff[iq];
                    }
                } else if (nb <= qc.coop) {
                    // few entries: one lane forms the seeds, the warp runs the
                    // recurrence level-parallel
                    for (int j = 0; j < nb; ++j) {
                        if (lane == 0) {
                            const int idx = queue[j];
                            const int g = idx / KK, r = idx - g * KK;
                            const int P = r / Kcd, Q = r - P * Kcd;
                            const Task tg = qc.tasks[gi.x + g];
                            const int ip = pp.order[tg.pab + P];
                            const int iq = pp.order[tg.pcd + Q];
                            const QuartetArgs qa = quartet_args(pp, ip, iq);
                            double2 Sh[BOYS_MAX_ORDER + 1];
                            float2 S32[BOYS_MAX_ORDER + 1];
                            const bool want32 =
                                mixed && pp.sbound[tg.pab + P] *
                                                 pp.sbound[tg.pcd + Q] < cut32;
                            int f = entry_seeds(d, qc.L, want32 ? 1 : 0, qa, Sh, S32, gi.x + g);
                            if (f == 2) f = 1;  // FP32 seeds out of range: this entry runs in FP64
                            if (f == 1) {
                                for (int n = 0; n <= qc.L; ++n) sseed[n] = Sh[n];
                                for (int x = 0; x < 3; ++x) sseed[qc.L + 1 + x] = qa.X[x];
                                cnt64 += first_chunk;
                            } else if (f == 0) {
                                float2* s32 = reinterpret_cast<float2*>(sseed);
                                for (int n = 0; n <= qc.L; ++n) s32[n] = S32[n];
                                for (int x = 0; x < 3; ++x)
                                    s32[qc.L + 1 + x] = make_float2((float)qa.X[x].x, (float)qa.X[x].y);
                                cnt32 += first_chunk;
                            }
                            flag[j] = f;
                            eoff[j] = pp.Eoff[iq];
                        }
                        __syncwarp();
                        if (flag[j] == 1) {
                            coop_rec<double2>(qc.L, sseed, sseed + qc.L + 1, R, B1p, j, qc.B1, d.herm_xyz, lane);
                        } else if (flag[j] == 0) {
                            const float2* s32 = reinterpret_cast<const float2*>(sseed);
                            coop_rec<float2>(qc.L, s32, s32 + qc.L + 1, R32s, 2 * B1p, 2 * j, 2 * qc.B1, d.herm_xyz,
                                             lane);
                        }
                    }
                } else if (lane < nb) {
                    const int idx = queue[lane];
                    const int g = idx / KK, r = idx - g * KK;
                    const int P = r / Kcd, Q = r - P * Kcd;
                    const Task tg = qc.tasks[gi.x + g];
                    const int ip = pp.order[tg.pab + P];
                    const int iq = pp.order[tg.pcd + Q];
                    const QuartetArgs qa = quartet_args(pp, ip, iq);
                    double2 Sh[BOYS_MAX_ORDER + 1];
                    float2 S32[BOYS_MAX_ORDER + 1];
                    const bool want32 = mixed && pp.sbound[tg.pab + P] *
                                                         pp.sbound[tg.pcd + Q] <
                                                     cut32;
                    int f = entry_seeds(d, qc.L, want32 ? 1 : 0, qa, Sh, S32, gi.x + g);
                    if (f == 2) f = 1;  // FP32 seeds out of range: this entry runs in FP64
                    if (f == 1) {
                        hermite_rec_any<double2>(d, qc.L, Sh, qa.X, R + lane, B1p);
                        cnt64 += first_chunk;
                    } else {
                        const float2 X32[3] = {make_float2((float)qa.X[0].x, (float)qa.X[0].y),
                                               make_float2((float)qa.X[1].x, (float)qa.X[1].y),
                                               make_float2((float)qa.X[2].x, (float)qa.X[2].y)};
                        hermite_rec_any<float2>(d, qc.L, S32, X32, R32s + 2 * lane, 2 * B1p);
                        cnt32 += first_chunk;
                    }
                    flag[lane] = f;
                    eoff[lane] = pp.Eoff[iq];
                }
                __syncwarp();
                // phase 2: runs of entries with the same bra pair
                for (int j0 = 0; j0 < nb;) {
                    const int key = queue[j0] / Kcd;  // g * Kab + P
                    int j1 = j0 + 1;
                    while (j1 < nb && queue[j1] / Kcd == key) ++j1;
                    if (key != cur) {
                        if (cur >= 0) {
                            __syncwarp();
                            const int cg = cur / Kab, cP = cur - cg * Kab;
                            const Task tc = qc.tasks[gi.x + cg];
                            step_b_any(d, qc, tabs, tc, pp.order[tc.pab + cP], W, W32, any64,
                                       any32, stg, c0, chn, lane);
                            __syncwarp();
                            for (int it = lane; it < qc.Nab * qc.CH; it += 32) {
                                if (any64) W[it] = c2(0.0, 0.0);
                                if (any32) W32[it] = make_float2(0.0f, 0.0f);
                            }
                            __syncwarp();
                        }
                        cur = key;
                        any64 = any32 = false;
                    }
                    bool has64 = false, has32 = false;
                    for (int jj = j0; jj < j1; ++jj) {
                        has64 = has64 || flag[jj] == 1;
                        has32 = has32 || flag[jj] == 0;
                    }
                    if (qc.stream) {
                        // entry by entry: the warp's recurrence into the
                        // two-column buffer (level 0 in column 0), then the
                        // ket transform of that column
                        for (int jj = j0; jj < j1; ++jj) {
                            __syncwarp();  // the previous entry's transform has read R
                            const double2* es = sseed + (size_t)jj * sstride;
                            if (flag[jj] == 1) {
                                coop_rec<double2>(qc.L, es, es + qc.L + 1, R, 2, 0, 1, d.herm_xyz, lane);
                            } else {
                                const float2* s32 = reinterpret_cast<const float2*>(es);
                                coop_rec<float2>(qc.L, s32, s32 + qc.L + 1, R32s, 4, 0, 2, d.herm_xyz, lane);
                            }
                            step_k_any(qc, tabs, d.herm_xyz, pp, R, R32s, 2, flag + jj, eoff + jj, 0, 1, W, W32, stg,
                                       c0, chn, lane);
                        }
                    } else {
                        step_k_any(qc, tabs, d.herm_xyz, pp, R, R32s, B1p, flag, eoff, j0, j1, W, W32, stg, c0, chn,
                                   lane);
                    }
                    any64 = any64 || has64;
                    any32 = any32 || has32;
                    j0 = j1;
                }
            }
            if (cur >= 0) {
                __syncwarp();
                const int cg = cur / Kab, cP = cur - cg * Kab;
                const Task tc = qc.tasks[gi.x + cg];
                step_b_any(d, qc, tabs, tc, pp.order[tc.pab + cP], W, W32, any64, any32, stg,
                           c0, chn, lane);
            }
            __syncwarp();
        }
    }
    if (d.counters) {
        // each primitive quartet is counted once, by the warps of chunk 0
        const unsigned long long a64 = __reduce_add_sync(0xffffffffu, (unsigned)cnt64);
        const unsigned long long a32 = __reduce_add_sync(0xffffffffu, (unsigned)cnt32);
        if (lane == 0) {
            atomicAdd(&d.counters[0], a64);
            atomicAdd(&d.counters[1], a32);
        }
    }
}

size_t quartet_smem_bytes(const QuartetClass& qc, int warps_per_block, bool mixed) {
    return (((size_t)qc.tab_words * 4 + 15) / 16) * 16 +
           (size_t)warps_per_block *
               warp_smem(qc.NL, qc.B1, qc.Nab, qc.CH, mixed, qc.stage_e, qc.stream, qc.L, mixed && !qc.no32).total;
}

static bool g_const_ready = false;

cudaError_t launch_quartets(const EriDev& dev, const QuartetClass& qc, int warps_per_block, int grid,
                            cudaStream_t s) {
    if (qc.ntask <= 0) return cudaSuccess;
    if (!g_const_ready) {
        double v[40];
        for (int i = 0; i < 40; ++i) v[i] = (double)i;
        cudaError_t e = cudaMemcpyToSymbol(c_int, v, sizeof v);
        if (e != cudaSuccess) return e;
        g_const_ready = true;
    }
    const size_t smem = quartet_smem_bytes(qc, warps_per_block, dev.fp32_cut > 0.0f);
    static size_t configured[2] = {0, 0};
    const int v = qc.minb == 4 ? 1 : 0;
    if (smem > 48 * 1024 && smem > configured[v]) {
        cudaError_t e = v ? cudaFuncSetAttribute(quartet_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)smem)
                          : cudaFuncSetAttribute(quartet_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)smem);
        if (e != cudaSuccess) return e;
        configured[v] = smem;
    }
    if (v)
        quartet_kernel<4><<<grid, warps_per_block * 32, smem, s>>>(dev, qc);
    else
        quartet_kernel<2><<<grid, warps_per_block * 32, smem, s>>>(dev, qc);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// K5: full-tensor images (src/eri.cpp:777-805).  block_info[5*i] =
// (ga, gb, gc, gd AO offsets, packed shape na | nb<<8 | nc<<16 | nd<<24).
// One thread per packed element; images written in the reference's order.
// ---------------------------------------------------------------------------

__global__ void scatter_full_kernel(const double2* packed, const long long* block_off, const int* info, int nblocks,
                                    long long n, double2* full) {
    const int bi = blockIdx.y * gridDim.x + blockIdx.x;
    if (bi >= nblocks) return;
    const int* f = info + 5 * bi;
    const int sh = f[4];
    const int na = sh & 255, nb = (sh >> 8) & 255, nc = (sh >> 16) & 255, nd = (sh >> 24) & 255;
    const int total = na * nb * nc * nd;
    const long long g[4] = {f[0], f[1], f[2], f[3]};
    const int dims[4] = {na, nb, nc, nd};
    // image m of element (x0, x1, x2, x3) sits at (x[perm[m][0]], ...):
    // (ab|cd), (cd|ab), (ba|dc)*, (dc|ba)* (src/eri.cpp:777-805)
    const int perm[4][4] = {{0, 1, 2, 3}, {2, 3, 0, 1}, {1, 0, 3, 2}, {3, 2, 1, 0}};
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int x[4] = {e / (nd * nc * nb), (e / (nd * nc)) % nb, (e / nd) % nc, e % nd};
        const double2 v = packed[block_off[bi] + e];
        const long long G[4] = {g[0] + x[0], g[1] + x[1], g[2] + x[2], g[3] + x[3]};
        for (int m = 0; m < 4; ++m) {
            long long p[4];
            for (int k = 0; k < 4; ++k) p[k] = G[perm[m][k]];
            // The reference writes the four images element by element, so
            // where images coincide (repeated shells) the last (element,
            // image) in that order wins; write only if this one is it.
            bool last = true;
            for (int m2 = 0; m2 < 4 && last; ++m2) {
                int y[4];
                bool inside = true;
                for (int k = 0; k < 4; ++k) {
                    // position k of image m2 holds global index G'[perm[m2][k]]
                    const int slot = perm[m2][k];
                    const long long loc = p[k] - g[slot];
                    inside = inside && loc >= 0 && loc < dims[slot];
                    y[slot] = (int)loc;
                }
                if (!inside) continue;
                const int e2 = ((y[0] * nb + y[1]) * nc + y[2]) * nd + y[3];
                if (e2 > e || (e2 == e && m2 > m)) last = false;
            }
            if (!last) continue;
            full[((p[0] * n + p[1]) * n + p[2]) * n + p[3]] = m < 2 ? v : cconj(v);
        }
    }
}

cudaError_t launch_scatter_full(const double2* packed, const long long* block_off, const int* block_info, int nblocks,
                                long long n, double2* full, cudaStream_t s) {
    if (nblocks <= 0) return cudaSuccess;
    const int gx = nblocks < 65535 ? nblocks : 65535;
    const int gy = (nblocks + gx - 1) / gx;
    scatter_full_kernel<<<dim3(gx, gy), 128, 0, s>>>(packed, block_off, block_info, nblocks, n, full);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Index arrays of packed pair records: dst[i] = src[i] + off.
// ---------------------------------------------------------------------------

template <typename T>
__global__ void offset_copy_kernel(T* dst, const T* src, long long n, T off) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[i] + off;
}

cudaError_t launch_offset_copy(int* dst, const int* src, long long n, int off, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    offset_copy_kernel<int><<<(int)std::min<long long>((n + 255) / 256, 4096), 256, 0, s>>>(dst, src, n, off);
    return cudaGetLastError();
}

cudaError_t launch_offset_copy(long long* dst, const long long* src, long long n, long long off, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    offset_copy_kernel<long long><<<(int)std::min<long long>((n + 255) / 256, 4096), 256, 0, s>>>(dst, src, n, off);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Output copy to page-locked host memory by the SMs (stores through the
// mapped device address, streaming loads): 16-byte words, grid-stride.  On
// the coherent host link a few dozen blocks reach the link bandwidth, and
// unlike copy-engine transfers issued right after heavy kernels the copy
// keeps that rate from call to call.
// ---------------------------------------------------------------------------

__global__ void host_copy_kernel(uint4* __restrict__ dst, const uint4* __restrict__ src, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = __ldcs(src + i);
}

cudaError_t launch_host_copy(void* dst_mapped, const void* src, long long bytes, int blocks, cudaStream_t s) {
    if (bytes <= 0) return cudaSuccess;
    if ((bytes & 15) || (reinterpret_cast<uintptr_t>(dst_mapped) & 15) || (reinterpret_cast<uintptr_t>(src) & 15))
        return cudaErrorInvalidValue;
    const long long n = bytes / 16;
    const int grid = (int)std::max<long long>(1, std::min<long long>((n + 511) / 512, blocks));
    host_copy_kernel<<<grid, 512, 0, s>>>(static_cast<uint4*>(dst_mapped), static_cast<const uint4*>(src), n);
    return cudaGetLastError();
}

// The blocks of one class copied to page-locked host memory by the SMs
// right after the class's kernels, on their stream: one warp per task, its
// entries (ca, cb, cc, cd) at out_off + ca st0 + cb st1 + cc st2 + cd st3
// (the entries the class kernels wrote), so the copy of the whole output
// overlaps the evaluation of the other classes.
__global__ void class_copy_kernel(const Task* __restrict__ tasks, int ntask, int na, int nb, int nc, int nd,
                                  const double2* __restrict__ src, double2* __restrict__ dst) {
    const int lane = threadIdx.x & 31;
    const int warp = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int nwarps = (int)((gridDim.x * (size_t)blockDim.x) >> 5);
    const int ncd = nc * nd;
    const int per = na * nb * ncd;
    for (int t = warp; t < ntask; t += nwarps) {
        const Task tk = tasks[t];
        if (tk.st[3] == 1 && tk.st[2] == nd && tk.st[1] == ncd && tk.st[0] == nb * ncd) {
            // the task's entries are one contiguous run (an unsegmented block)
            for (int e = lane; e < per; e += 32) dst[tk.out_off + e] = __ldcs(src + tk.out_off + e);
            continue;
        }
        for (int e = lane; e < per; e += 32) {
            const int ab = e / ncd, cd = e - ab * ncd;
            const int ca = ab / nb, cb = ab - ca * nb, cc = cd / nd, cdd = cd - cc * nd;
            const long long o = tk.out_off + (long long)ca * tk.st[0] + (long long)cb * tk.st[1] +
                                (long long)cc * tk.st[2] + (long long)cdd * tk.st[3];
            dst[o] = __ldcs(src + o);
        }
    }
}

cudaError_t launch_class_copy(const Task* tasks, int ntask, int la, int lb, int lc, int ld, const double2* src,
                              void* dst_mapped, int sms, cudaStream_t s) {
    if (ntask <= 0) return cudaSuccess;
    if (reinterpret_cast<uintptr_t>(dst_mapped) & 15) return cudaErrorInvalidValue;
    // a few blocks per class: the copies trail the evaluation on streams of
    // their own and are bound by the host link, so they should take few SMs
    // from the classes still running
    const int warps = 8;
    const int grid = (int)std::max(1, std::min((ntask + warps - 1) / warps, std::max(sms, 1) / 8));
    class_copy_kernel<<<grid, 32 * warps, 0, s>>>(tasks, ntask, ncart(la), ncart(lb), ncart(lc), ncart(ld), src,
                                                  static_cast<double2*>(dst_mapped));
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FMA throughput probes (FP64 and FP32): 8 independent dependent-FMA chains
// per thread, 8 resident blocks of 256 threads per SM.
// ---------------------------------------------------------------------------

template <typename T>
__global__ void fma_probe_kernel(T* out, int iters, T a, T b) {
    T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            x0 = fma(x0, a, b);
            x1 = fma(x1, a, b);
            x2 = fma(x2, a, b);
            x3 = fma(x3, a, b);
            x4 = fma(x4, a, b);
            x5 = fma(x5, a, b);
            x6 = fma(x6, a, b);
            x7 = fma(x7, a, b);
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
cudaError_t run_fma_probe(int sms, cudaStream_t s, int iters, float* ms, double* flops) {
    const int blocks = sms * 8, threads = 256;
    T* buf = nullptr;
    cudaError_t e = cudaMalloc(&buf, sizeof(T) * blocks * threads);
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    fma_probe_kernel<T><<<blocks, threads, 0, s>>>(buf, 20, (T)1.0000001, (T)1e-9);
    cudaEventRecord(a, s);
    fma_probe_kernel<T><<<blocks, threads, 0, s>>>(buf, iters, (T)1.0000001, (T)1e-9);
    cudaEventRecord(b, s);
    e = cudaEventSynchronize(b);
    cudaEventElapsedTime(ms, a, b);
    *flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(buf);
    return e == cudaSuccess ? cudaGetLastError() : e;
}

cudaError_t run_fp64_probe(int sms, cudaStream_t s, float* ms, double* flops) {
    return run_fma_probe<double>(sms, s, 1000, ms, flops);
}

cudaError_t run_fp32_probe(int sms, cudaStream_t s, float* ms, double* flops) {
    return run_fma_probe<float>(sms, s, 20000, ms, flops);
}

}  // namespace gx
