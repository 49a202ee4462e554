// Device-side building blocks shared by the GB300 kernels: complex
// arithmetic on double2, the Hermite index enumeration, and the complex Boys
// function F_0..F_L(z).
//
// FP64 budget.  On GB300 the FP64 pipe runs at 1/64 of the FP32 rate
// (measured: 1.20 TFLOP/s FP64 FMA, 1.05 TFLOP/s FP64 mma.sync, 75 TFLOP/s
// FP32 FMA), so every routine here is written to minimise FP64 instructions:
// integer indexing, table loads and shared-memory traffic are essentially
// free in comparison.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gx {

// ---------------------------------------------------------------------------
// complex helpers (double2 = re, im)
// ---------------------------------------------------------------------------

__host__ __device__ __forceinline__ double2 c2(double x, double y) { return make_double2(x, y); }
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return c2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return c2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) { return c2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ double2 cconj(double2 a) { return c2(a.x, -a.y); }
// a*b: 4 FP64 instructions (2 mul + 2 fma)
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return c2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// c + a*b: 4 FP64 fma
__host__ __device__ __forceinline__ double2 cmac(double2 c, double2 a, double2 b) {
    return c2(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
// c + s*a (s real): 2 FP64 fma
__host__ __device__ __forceinline__ double2 cmacr(double2 c, double s, double2 a) {
    return c2(fma(s, a.x, c.x), fma(s, a.y, c.y));
}

// ---------------------------------------------------------------------------
// Hermite multi-index enumeration: all (k, l, m) with k + l + m <= L, ordered
// by total degree s, then x-major within a degree (the Cartesian order of
// the reference, src/types.cpp:74-90).  Index of (k, l, m):
//   s(s+1)(s+2)/6 + (s-k)(s-k+1)/2 + m
// ---------------------------------------------------------------------------

__host__ __device__ __forceinline__ int herm_count(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }
__host__ __device__ __forceinline__ int herm_index(int k, int l, int m) {
    const int s = k + l + m;
    return s * (s + 1) * (s + 2) / 6 + (s - k) * (s - k + 1) / 2 + m;
}
__host__ __device__ __forceinline__ int ncart(int l) { return (l + 1) * (l + 2) / 2; }

// ---------------------------------------------------------------------------
// status word written by kernels (never a trap): first failure wins
// ---------------------------------------------------------------------------

struct DevStatus {
    int code;       // 0 ok, else a gx_status value
    int order;      // Boys order of the failing evaluation
    long long item; // failing work item
    double zr, zi;  // failing Boys argument
};

__device__ __forceinline__ void report(DevStatus* st, int code, long long item, int order, double zr, double zi) {
    if (atomicCAS(&st->code, 0, code) == 0) {
        st->item = item;
        st->order = order;
        st->zr = zr;
        st->zi = zi;
    }
}

// ---------------------------------------------------------------------------
// complex Boys function
//
// F_n(z) = int_0^1 t^{2n} exp(-z t^2) dt, n = 0..L <= 32, z complex.
// Output convention: F_n(z) = e0 * Sh[n].  Regions (own method; the
// reference's regions are reproduced only for diagnostics and domain
// errors):
//   * asymptotic  Re z >= 2L + 44, |Im z| <= Re z / 2:
//       F_0 = sqrt(pi)/(2 sqrt z), F_{n+1} = F_n (n + 1/2)/z, e0 = 1.
//       The dropped term is below 1e-17 relative there.
//   * Taylor grid -16 <= Re z <= 108, |Im z| <= 12:
//       scaled values S_n(z0) = e^{z0} F_n(z0) on a 1/8 grid;
//       Sh_L = sum_{k<10} S_{L+k}(z0) (-d)^k / k!, d = z - z0,
//       Sh_n = (2 z Sh_{n+1} + e^{-d}) / (2n + 1) where that downward
//       recursion is stable (Re z >= 0 and |Im z| <= 3 or Re z >= 2|Im z|:
//       error growth below 3x), the Taylor sum for every order elsewhere;
//       e0 = e^{-z0}.
//   * otherwise (|z| <= 160) adaptive Gauss-Legendre quadrature, 16 vs 32
//       points on ceil(max(|Re|,|Im|)/8) doubling segments, of the unscaled
//       integral (e0 = 1) for Re z >= 0 and of the scaled integral
//       int t^{2n} e^{z(1-t^2)} dt (e0 = e^{-z}) for Re z < 0; a quadrature
//       that does not reach tolerance in 4096 segments returns -5.
//   * outside |z| <= 160 and the reference's asymptotic sector
//       (Re z >= 2L + 60, |Im z| <= Re z / 2): domain error, as
//       src/boys.cpp:262-270.
// ---------------------------------------------------------------------------

constexpr int BOYS_MAX_ORDER = 32;
constexpr int BOYS_TAYLOR_TERMS = 10;
constexpr int BOYS_TABLE_ORDERS = BOYS_MAX_ORDER + BOYS_TAYLOR_TERMS + 1;  // 43
constexpr double BOYS_X0 = -16.0, BOYS_X1 = 108.0, BOYS_Y1 = 12.0, BOYS_H = 0.125, BOYS_INV_H = 8.0;
constexpr int BOYS_NX = 993;  // (108 + 16) * 8 + 1
constexpr int BOYS_NY = 193;  // 24 * 8 + 1

struct BoysTable {
    const double2* S;   // [(ix * NY + iy) * ORDERS + n]
    const double2* E0;  // [ix * NY + iy] = e^{-z0}
};

// Gauss-Legendre rules on [-1, 1]; filled from the host.
struct GLRules {
    double x16[16], w16[16], x32[32], w32[32];
};

__device__ __forceinline__ bool boys_domain_ok(double x, double y, int L) {
    if (!(isfinite(x) && isfinite(y))) return false;
    if (x * x + y * y <= 160.0 * 160.0) return true;
    return x >= 2.0 * L + 60.0 && fabs(y) <= 0.5 * x;
}

// Gauss-Legendre quadrature of F_n on a fixed number of segments with
// compensated sums: scaled (int t^{2n} e^{z(1-t^2)}) for Re z < 0, unscaled
// (int t^{2n} e^{-z t^2}) otherwise, so the integrand never exceeds the
// result's own scale (the reference's choice, src/boys.cpp:155-179, 272-291).
static __device__ __noinline__ void boys_quad_fixed(double x, double y, int L, int segments, int rule, const GLRules* gl,
                                                    double2* out, double2* comp) {
    for (int n = 0; n <= L; ++n) {
        out[n] = c2(0.0, 0.0);
        comp[n] = c2(0.0, 0.0);
    }
    const bool scaled = x < 0.0;
    const int npt = rule ? 32 : 16;
    const double* nodes = rule ? gl->x32 : gl->x16;
    const double* weights = rule ? gl->w32 : gl->w16;
    const double inv = 1.0 / (double)segments;
    const double hw = 0.5 * inv;
    const double ex = scaled ? exp(x) : 1.0;
    for (int s = 0; s < segments; ++s) {
        const double mid = ((double)s + 0.5) * inv;
        for (int k = 0; k < npt; ++k) {
            const double t = fma(hw, nodes[k], mid);
            const double t2 = t * t;
            const double mag = ex * exp(-x * t2) * hw * weights[k];
            double sn, cs;
            sincos(scaled ? y * (1.0 - t2) : -y * t2, &sn, &cs);
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

// Adaptive GL16/GL32 (tolerance abs 2e-15 + rel 7.5e-14, at most 4096
// segments); returns 0 or GX_EBOYS.
static __device__ __noinline__ int boys_quad_adaptive(double x, double y, int L, const GLRules* gl, double2* out,
                                                      double2* scratch) {
    double2 comp[BOYS_MAX_ORDER + 1];
    int segments = (int)ceil(fmax(fabs(x), fabs(y)) / 8.0);
    if (segments < 1) segments = 1;
    for (;;) {
        boys_quad_fixed(x, y, L, segments, 0, gl, scratch, comp);
        boys_quad_fixed(x, y, L, segments, 1, gl, out, comp);
        bool ok = true;
        for (int n = 0; n <= L; ++n) {
            const double dx = out[n].x - scratch[n].x, dy = out[n].y - scratch[n].y;
            const double e = sqrt(dx * dx + dy * dy);
            ok = ok && e <= 2.0e-15 + 7.5e-14 * sqrt(out[n].x * out[n].x + out[n].y * out[n].y);
        }
        if (ok) return 0;
        if (segments >= 4096) return -4;
        segments *= 2;
    }
}

// Evaluate Sh[0..L] and e0 with F_n = e0 * Sh[n].  Returns 0 or -4 (domain).
__device__ __forceinline__ int boys_eval(double x, double y, int L, const BoysTable& tab, const GLRules* gl,
                                         double2* Sh, double2& e0) {
    if (!boys_domain_ok(x, y, L)) return -4;
    if (x >= 2.0 * L + 44.0 && fabs(y) <= 0.5 * x) {
        const double r2 = fma(x, x, y * y);
        const double ir = rsqrt(r2);
        const double r = r2 * ir;
        const double s = sqrt(0.5 * (r + x));
        const double t = 0.5 * y / s;
        const double k0 = 0.88622692545275801365 * ir;  // sqrt(pi)/2 / |z|
        double2 f = c2(k0 * s, -k0 * t);
        const double ir2 = ir * ir;
        const double2 iz = c2(x * ir2, -y * ir2);
        Sh[0] = f;
        for (int n = 0; n < L; ++n) {
            f = cscale(cmul(f, iz), (double)n + 0.5);
            Sh[n + 1] = f;
        }
        e0 = c2(1.0, 0.0);
        return 0;
    }
    if (x >= BOYS_X0 && x <= BOYS_X1 && fabs(y) <= BOYS_Y1) {
        const int ix = __float2int_rn((float)(x - BOYS_X0) * (float)BOYS_INV_H);
        const int iy = __float2int_rn((float)(y + BOYS_Y1) * (float)BOYS_INV_H);
        const int p = ix * BOYS_NY + iy;
        const double2 d = c2(x - (BOYS_X0 + BOYS_H * ix), y - (-BOYS_Y1 + BOYS_H * iy));
        const double2* S = tab.S + (size_t)p * BOYS_TABLE_ORDERS;
        e0 = __ldg(&tab.E0[p]);
        double2 w[BOYS_TAYLOR_TERMS];
#pragma unroll
        for (int k = 1; k < BOYS_TAYLOR_TERMS; ++k) w[k] = cscale(d, -1.0 / (double)k);
        if (x >= 0.0 && (fabs(y) <= 3.0 || x >= 2.0 * fabs(y))) {
            double2 acc = __ldg(&S[L + BOYS_TAYLOR_TERMS - 1]);
#pragma unroll
            for (int k = BOYS_TAYLOR_TERMS - 1; k >= 1; --k) acc = cmac(__ldg(&S[L + k - 1]), acc, w[k]);
            Sh[L] = acc;
            if (L > 0) {
                double2 em = c2(1.0, 0.0);
#pragma unroll
                for (int k = BOYS_TAYLOR_TERMS - 1; k >= 1; --k) em = cmac(c2(1.0, 0.0), em, w[k]);
                const double2 z2 = c2(x + x, y + y);
                for (int n = L - 1; n >= 0; --n) {
                    acc = cscale(cmac(em, z2, acc), 1.0 / (double)(2 * n + 1));
                    Sh[n] = acc;
                }
            }
        } else {
            for (int n = 0; n <= L; ++n) {
                double2 acc = __ldg(&S[n + BOYS_TAYLOR_TERMS - 1]);
#pragma unroll
                for (int k = BOYS_TAYLOR_TERMS - 1; k >= 1; --k) acc = cmac(__ldg(&S[n + k - 1]), acc, w[k]);
                Sh[n] = acc;
            }
        }
        return 0;
    }
    double2 tmp[BOYS_MAX_ORDER + 1], scratch[BOYS_MAX_ORDER + 1];
    if (boys_quad_adaptive(x, y, L, gl, tmp, scratch)) return -5;
    for (int n = 0; n <= L; ++n) Sh[n] = tmp[n];
    if (x < 0.0) {
        double sn, cs;
        sincos(-y, &sn, &cs);
        const double m = exp(-x);
        e0 = c2(m * cs, m * sn);
    } else {
        e0 = c2(1.0, 0.0);
    }
    return 0;
}


// ---------------------------------------------------------------------------
// FP32 Boys values for the mixed-precision path, large |T| only: the
// asymptotic form F_0 = sqrt(pi)/(2 sqrt z), F_{n+1} = F_n (n + 1/2)/z (an
// upward recurrence) for Re z >= 2L + 24, |Im z| <= Re z / 2.  The dropped
// tail is e^{-Re z} |z|^{n-1/2}/Gamma(n+1/2) relative, below 5e-8 there for
// every order.  Small and moderate |T| (the Taylor grid with its downward
// recursion, the quadrature) stay in FP64: the function returns false and
// the caller uses boys_eval, which also reports every domain error exactly
// as without mixed precision.  z itself is formed in FP64 by the caller.
// ---------------------------------------------------------------------------

__device__ __forceinline__ float2 f2mul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

__device__ __forceinline__ bool boys_eval32(double x, double y, int L, float2* Sh) {
    if (!(x >= 2.0 * L + 24.0 && fabs(y) <= 0.5 * x && (x * x + y * y <= 160.0 * 160.0 || x >= 2.0 * L + 60.0)))
        return false;
    const float xf = (float)x, yf = (float)y;
    const float r2 = fmaf(xf, xf, yf * yf);
    const float ir = rsqrtf(r2);
    const float r = r2 * ir;
    const float s = sqrtf(0.5f * (r + xf));
    const float t = 0.5f * yf / s;
    const float k0 = 0.886226925452758f * ir;  // sqrt(pi)/2 / |z|
    float2 f = make_float2(k0 * s, -k0 * t);
    const float ir2 = ir * ir;
    const float2 iz = make_float2(xf * ir2, -yf * ir2);
    Sh[0] = f;
    for (int n = 0; n < L; ++n) {
        f = f2mul(f, iz);
        f.x *= (float)n + 0.5f;
        f.y *= (float)n + 0.5f;
        Sh[n + 1] = f;
    }
    return true;
}

// FP32 seeds C (-2 rho)^n F_n for a primitive quartet whose C = F_ab F_cd /
// sqrt(p + q) and T = (tre, tim) were formed in FP64.  False (use FP64 Boys)
// outside the asymptotic sector or when a seed would leave the range in
// which the FP32 recurrence is safe (|seed| < 1e25, |C| in [1e-30, 1e30]).
__device__ __forceinline__ bool seeds32(double2 C, double rho, double tre, double tim, int L, float2* S32) {
    if (!boys_eval32(tre, tim, L, S32)) return false;
    float2 c = make_float2((float)C.x, (float)C.y);
    const float mag = fabsf(c.x) + fabsf(c.y);
    if (!(mag >= 1.0e-30f && mag <= 1.0e30f)) return false;
    const float m2r = (float)(-2.0 * rho);
    bool ok = true;
    for (int n = 0; n <= L; ++n) {
        S32[n] = f2mul(c, S32[n]);
        ok = ok && fabsf(S32[n].x) + fabsf(S32[n].y) < 1.0e25f;  // false for NaN too
        c.x *= m2r;
        c.y *= m2r;
    }
    return ok;
}

}  // namespace gx
