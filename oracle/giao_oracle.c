/*
 * CPU oracle for the GIAO electron-repulsion hot path -- TEST INFRASTRUCTURE.
 *
 * A plain-C restatement of the reference algorithm (simenkva/GIAOINT v0.11.1),
 * used only by tests/, __graft_entry__.smoke() and the CPU-baseline legs of
 * bench.py, always as the checker or as the timed CPU baseline, never as the
 * product path.  Each function cites the reference file:line it restates.
 *
 *   normalisation        include/giao_integrals/types.hpp:39-132, src/types.cpp:20-171
 *   London wave vector   src/types.cpp:179-186
 *   Gaussian product     src/overlap.cpp:60-95
 *   Hermite E (1-D)      src/hermite.cpp:8-40
 *   complex Boys         src/boys.cpp:1-302
 *   primitive ERI        src/eri.cpp:67-384 (MD, six-index complex R table,
 *                        exact-zero-field collapsed real path)
 *   shell quartet        src/eri.cpp:454-585
 *   quartet batches      src/eri.cpp:644-767 (OpenMP dynamic,1)
 *   full tensor          src/eri.cpp:414-429, 777-847
 *   Schwarz bounds       src/eri.cpp:587-619
 *   Cholesky selections  src/cholesky.cpp:17-323
 *
 * Status codes: 0 ok, -1 invalid argument, -2 index out of range,
 * -3 length error, -4 Boys numerical error.  The message is kept per thread
 * and read with or_last_error().
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

static _Thread_local char g_err[512];
const char* or_last_error(void) { return g_err; }

static int set_err(int code, const char* msg) {
    snprintf(g_err, sizeof g_err, "%s", msg);
    return code;
}

/* ------------------------------------------------------------------ */
/* normalisation (src/types.cpp:20-72)                                  */
/* ------------------------------------------------------------------ */

static double log_odd_double_factorial(int l) {
    if (l == 0) return 0.0;
    const double n = (double)l;
    return n * log(2.0) + lgamma(n + 0.5) - 0.5 * log(M_PI);
}

double or_primitive_normalization(double alpha, int lx, int ly, int lz) {
    const double total = (double)(lx + ly + lz);
    const double log_den = log_odd_double_factorial(lx) + log_odd_double_factorial(ly) +
                           log_odd_double_factorial(lz);
    return exp(0.75 * log(2.0 * alpha / M_PI) + 0.5 * (total * log(4.0 * alpha) - log_den));
}

static double same_center_overlap(double a, double b, int l) {
    const double norm = or_primitive_normalization(a, l, 0, 0) * or_primitive_normalization(b, l, 0, 0);
    const double p = a + b;
    const double lm = lgamma(l + 0.5) - (l + 0.5) * log(p);
    return norm * exp(lm) * M_PI / p;
}

/* Contraction normalisation of one shell (src/types.cpp:136-157). coefs is
 * contraction-major [ncontr][nprim]; normalised in place. */
int or_normalize_shell(int l, int nprim, int ncontr, const double* exps, double* coefs) {
    for (int x = 0; x < ncontr; ++x) {
        double* c = coefs + (size_t)x * nprim;
        int nonzero = 0;
        for (int i = 0; i < nprim; ++i) nonzero |= (c[i] != 0.0);
        if (!nonzero) return set_err(-1, "a shell contraction cannot have all-zero coefficients");
        double s = 0.0;
        for (int i = 0; i < nprim; ++i)
            for (int j = 0; j < nprim; ++j) s += c[i] * c[j] * same_center_overlap(exps[i], exps[j], l);
        if (!isfinite(s) || s <= 0.0) return set_err(-1, "contraction has a non-positive or non-finite norm");
        const double scale = 1.0 / sqrt(s);
        for (int i = 0; i < nprim; ++i) c[i] *= scale;
    }
    return 0;
}

/* x-major Cartesian order (src/types.cpp:74-90). */
static int cart_components(int l, int (*out)[3]) {
    int k = 0;
    for (int x = l; x >= 0; --x)
        for (int y = l - x; y >= 0; --y) {
            out[k][0] = x;
            out[k][1] = y;
            out[k][2] = l - x - y;
            ++k;
        }
    return k;
}

/* ------------------------------------------------------------------ */
/* field and pair data (src/types.cpp:179-186, src/overlap.cpp:60-95)   */
/* ------------------------------------------------------------------ */

typedef struct {
    double B[3], O[3];
} field_t;

static void london_k(const field_t* f, const double* c, double* k) {
    const double d0 = c[0] - f->O[0], d1 = c[1] - f->O[1], d2 = c[2] - f->O[2];
    k[0] = 0.5 * (f->B[1] * d2 - f->B[2] * d1);
    k[1] = 0.5 * (f->B[2] * d0 - f->B[0] * d2);
    k[2] = 0.5 * (f->B[0] * d1 - f->B[1] * d0);
}

typedef struct {
    double p, mu, P[3], q[3];
    cplx Pc[3];
    double K;      /* exp(-mu |A-B|^2) */
    cplx london;   /* exp(-q.q/4p - i q.P) */
} pair_t;

static void gaussian_product(double a, const double* A, double b, const double* Bc, const field_t* f, pair_t* out) {
    const double p = a + b;
    out->p = p;
    out->mu = a * b / p;
    for (int i = 0; i < 3; ++i) out->P[i] = (a * A[i] + b * Bc[i]) / p;
    double ka[3], kb[3];
    london_k(f, A, ka);
    london_k(f, Bc, kb);
    for (int i = 0; i < 3; ++i) out->q[i] = kb[i] - ka[i];
    double r2 = 0.0;
    for (int i = 0; i < 3; ++i) r2 += (A[i] - Bc[i]) * (A[i] - Bc[i]);
    out->K = exp(-out->mu * r2);
    const double phase = -(out->q[0] * out->P[0] + out->q[1] * out->P[1] + out->q[2] * out->P[2]);
    const double damping = -(out->q[0] * out->q[0] + out->q[1] * out->q[1] + out->q[2] * out->q[2]) / (4.0 * p);
    out->london = cexp(CMPLX(damping, phase));
    for (int i = 0; i < 3; ++i) out->Pc[i] = CMPLX(out->P[i], -0.5 * out->q[i] / p);
}

/* 1-D MD Hermite coefficients by repeated raising (src/hermite.cpp:8-40). */
static void hermite_1d(int la, int lb, double A, double Bc, double P, double p, double* e) {
    double cur[72], nxt[72];
    const int maxo = la + lb;
    for (int t = 0; t < maxo + 2; ++t) cur[t] = 0.0;
    cur[0] = 1.0;
    int active = 0;
    const double inv2p = 0.5 / p;
    for (int step = 0; step < la + lb; ++step) {
        const double disp = step < la ? P - A : P - Bc;
        for (int t = 0; t < maxo + 2; ++t) nxt[t] = 0.0;
        for (int t = 0; t <= active + 1; ++t) {
            const double lower = t == 0 ? 0.0 : cur[t - 1];
            const double same = t <= active ? cur[t] : 0.0;
            const double upper = t < active ? cur[t + 1] : 0.0;
            nxt[t] = inv2p * lower + disp * same + (double)(t + 1) * upper;
        }
        ++active;
        memcpy(cur, nxt, sizeof(double) * (maxo + 2));
    }
    for (int t = 0; t <= maxo; ++t) e[t] = cur[t];
}

/* ------------------------------------------------------------------ */
/* complex Boys function (src/boys.cpp:16-302)                          */
/* ------------------------------------------------------------------ */

enum { REGION_SERIES = 0, REGION_QUADRATURE = 1, REGION_SCALED_QUADRATURE = 2, REGION_ASYMPTOTIC = 3 };

static double gl_nodes[2][32], gl_weights[2][32];
static int gl_ready = 0;

/* Gauss-Legendre nodes by Newton iteration on P_n (the published textbook
 * construction the reference uses at src/boys.cpp:26-110). */
static void gl_build(int n, double* nodes, double* weights) {
    for (int i = 0; i < n / 2; ++i) {
        double root = cos(M_PI * ((double)i + 0.75) / ((double)n + 0.5));
        double deriv = 0.0;
        for (int it = 0; it < 20; ++it) {
            double prev = 1.0, cur = root;
            for (int deg = 2; deg <= n; ++deg) {
                const double nx = ((2.0 * deg - 1.0) * root * cur - (deg - 1.0) * prev) / deg;
                prev = cur;
                cur = nx;
            }
            deriv = n * (root * cur - prev) / (root * root - 1.0);
            const double upd = cur / deriv;
            root -= upd;
            if (fabs(upd) < 4.0 * 2.220446049250313e-16) break;
        }
        const double w = 2.0 / ((1.0 - root * root) * deriv * deriv);
        nodes[i] = -root;
        nodes[n - 1 - i] = root;
        weights[i] = w;
        weights[n - 1 - i] = w;
    }
}

static void gl_init(void) {
    if (gl_ready) return;
#pragma omp critical(or_gl_init)
    {
        if (!gl_ready) {
            gl_build(16, gl_nodes[0], gl_weights[0]);
            gl_build(32, gl_nodes[1], gl_weights[1]);
            gl_ready = 1;
        }
    }
}

static const double BOYS_ABS = 2.0e-15, BOYS_REL = 7.5e-14;

static void boys_quad(cplx z, int scaled, long segments, int rule, int nmax, cplx* v) {
    const int npt = rule ? 32 : 16;
    for (int n = 0; n <= nmax; ++n) v[n] = 0.0;
    const double inv = 1.0 / (double)segments;
    for (long s = 0; s < segments; ++s) {
        const double mid = ((double)s + 0.5) * inv, hw = 0.5 * inv;
        for (int k = 0; k < npt; ++k) {
            const double t = mid + hw * gl_nodes[rule][k];
            const double t2 = t * t;
            const cplx ex = scaled ? z * (1.0 - t2) : -z * t2;
            const cplx common = hw * gl_weights[rule][k] * cexp(ex);
            double pw = 1.0;
            for (int n = 0; n <= nmax; ++n) {
                v[n] += common * pw;
                pw *= t2;
            }
        }
    }
}

static int boys_adaptive(cplx z, int scaled, int nmax, cplx* v, double* err, long* segs) {
    const double diff = fmax(fabs(creal(z)), fabs(cimag(z)));
    long segments = (long)ceil(diff / 8.0);
    if (segments < 1) segments = 1;
    cplx lo[33], hi[33];
    for (;;) {
        boys_quad(z, scaled, segments, 0, nmax, lo);
        boys_quad(z, scaled, segments, 1, nmax, hi);
        int ok = 1;
        double worst = 0.0;
        for (int n = 0; n <= nmax; ++n) {
            const double e = cabs(hi[n] - lo[n]);
            worst = fmax(worst, e);
            ok = ok && e <= BOYS_ABS + BOYS_REL * cabs(hi[n]);
        }
        if (ok) {
            for (int n = 0; n <= nmax; ++n) v[n] = hi[n];
            *err = worst;
            *segs = segments;
            return 0;
        }
        if (segments >= 4096) return set_err(-4, "adaptive complex Boys quadrature did not reach tolerance");
        segments *= 2;
    }
}

/* Returns the region; values F_0..F_nmax (or e^z F_n when scaled). */
int or_boys(double zr, double zi, int nmax, int scaled, double* out, int* region, double* est_error, long* segments) {
    gl_init();
    cplx z = CMPLX(zr, zi);
    cplx* v = (cplx*)out;
    double err = 0.0;
    long segs = 0;
    int reg;
    if (nmax < 0) return set_err(-1, "Boys output must contain at least F_0");
    if (nmax > 32) return set_err(-1, "complex Boys supports orders through 32");
    if (!isfinite(zr) || !isfinite(zi)) return set_err(-1, "complex Boys argument must be finite");
    const double mag = cabs(z);
    if (mag <= 0.75) {
        /* compensated power series (src/boys.cpp:137-169) */
        double worst = 0.0;
        for (int n = 0; n <= nmax; ++n) {
            cplx pof = 1.0, sum = 0.0, comp = 0.0;
            double last = 0.0;
            for (int k = 0; k < 256; ++k) {
                const cplx term = pof / (double)(2 * n + 2 * k + 1);
                const cplx corr = term - comp;
                const cplx nx = sum + corr;
                comp = (nx - sum) - corr;
                sum = nx;
                last = cabs(term);
                if (k > 2 && last <= BOYS_ABS + BOYS_REL * cabs(sum)) break;
                pof *= -z / (double)(k + 1);
                if (k == 255) return set_err(-4, "complex Boys power series did not converge");
            }
            v[n] = scaled ? cexp(z) * sum : sum;
            worst = fmax(worst, last);
        }
        *region = REGION_SERIES;
        *est_error = worst;
        *segments = 0;
        return 0;
    }
    const double asym = 2.0 * nmax + 60.0;
    if (zr >= asym && fabs(zi) <= 0.5 * zr) {
        /* asymptotic sector (src/boys.cpp:209-231, 258-261) */
        const cplx sq = csqrt(z);
        cplx invp = 1.0 / sq;
        double gamma = sqrt(M_PI);
        for (int n = 0; n <= nmax; ++n) {
            cplx val = 0.5 * gamma * invp;
            if (scaled) val *= cexp(z);
            if (!isfinite(creal(val)) || !isfinite(cimag(val)))
                return set_err(-4, "requested Boys scaling is not representable for this argument");
            v[n] = val;
            gamma *= (double)n + 0.5;
            invp /= z;
        }
        *region = REGION_ASYMPTOTIC;
        *est_error = cabs(cexp(-z)) / fmax(1.0, 2.0 * cabs(z));
        *segments = 0;
        return 0;
    }
    if (mag > 160.0) {
        snprintf(g_err, sizeof g_err,
                 "complex Boys argument (%.17g,%.17g) at order %d is outside the verified direct domain |z| <= 160 "
                 "and the conservative large-positive asymptotic sector",
                 zr, zi, nmax);
        return -4;
    }
    if (zr < 0.0) {
        int rc = boys_adaptive(z, 1, nmax, v, &err, &segs);
        if (rc) return rc;
        reg = REGION_SCALED_QUADRATURE;
        if (!scaled) {
            const cplx f = cexp(-z);
            for (int n = 0; n <= nmax; ++n) {
                v[n] *= f;
                if (!isfinite(creal(v[n])) || !isfinite(cimag(v[n])))
                    return set_err(-4, "unscaled Boys value is not representable for this argument");
            }
            err *= cabs(f);
        }
    } else {
        int rc = boys_adaptive(z, scaled, nmax, v, &err, &segs);
        if (rc) return rc;
        reg = REGION_QUADRATURE;
    }
    *region = reg;
    *est_error = err;
    *segments = segs;
    return 0;
}

/* ------------------------------------------------------------------ */
/* primitive ERI kernel (src/eri.cpp:67-384)                            */
/* ------------------------------------------------------------------ */

typedef struct {
    double alpha;
    double center[3];
    int ang[3];
} prim_t;

typedef struct {
    cplx* aux;
    size_t aux_cap;
    double* raux;
    size_t raux_cap;
    cplx boys[33];
    int boys_valid;
    cplx boys_arg;
    int boys_scaled, boys_nmax;
} ws_t;

static void ws_free(ws_t* w) {
    free(w->aux);
    free(w->raux);
    memset(w, 0, sizeof *w);
}

static int ws_aux(ws_t* w, size_t n) {
    if (n > w->aux_cap) {
        cplx* p = (cplx*)realloc(w->aux, n * sizeof(cplx));
        if (!p) return set_err(-3, "out of memory");
        w->aux = p;
        w->aux_cap = n;
    }
    return 0;
}

static int ws_raux(ws_t* w, size_t n) {
    if (n > w->raux_cap) {
        double* p = (double*)realloc(w->raux, n * sizeof(double));
        if (!p) return set_err(-3, "out of memory");
        w->raux = p;
        w->raux_cap = n;
    }
    return 0;
}

/* hin (may be NULL): the 1-D Hermite coefficients of the six axes (bra x, y,
 * z, then ket x, y, z) computed beforehand by hermite_1d with the same
 * arguments, so that callers looping over primitive and Cartesian
 * combinations compute each once (the reference keeps them in a cache,
 * src/eri.cpp:107-160). */
static int eri_kernel_h(const prim_t* pr, const pair_t* ab, const pair_t* cd, int real_zero, ws_t* w,
                        const double* const* hin, cplx* result) {
    int maxima[6];
    for (int i = 0; i < 3; ++i) {
        maxima[i] = pr[0].ang[i] + pr[1].ang[i];
        maxima[3 + i] = pr[2].ang[i] + pr[3].ang[i];
    }
    int L = 0;
    for (int k = 0; k < 4; ++k) L += pr[k].ang[0] + pr[k].ang[1] + pr[k].ang[2];
    if (L > 32) return set_err(-1, "electron repulsion supports combined angular order through 32");
    size_t dims = (size_t)(L + 1);
    for (int i = 0; i < 6; ++i) dims *= (size_t)(maxima[i] + 1);
    if (dims > 4000000u) return set_err(-3, "ERI auxiliary exceeds the workspace limit");

    /* pair Hermite products (src/eri.cpp:107-160) */
    double herm[6][34];
    double* prod[2];
    double prodbuf[2][17 * 17 * 17];
    for (int pi = 0; pi < 2; ++pi) {
        const prim_t* l = &pr[2 * pi];
        const prim_t* r = &pr[2 * pi + 1];
        const pair_t* pd = pi ? cd : ab;
        const double* hx[3];
        for (int ax = 0; ax < 3; ++ax) {
            if (hin) {
                hx[ax] = hin[3 * pi + ax];
            } else {
                hermite_1d(l->ang[ax], r->ang[ax], l->center[ax], r->center[ax], pd->P[ax], pd->p, herm[3 * pi + ax]);
                hx[ax] = herm[3 * pi + ax];
            }
        }
        const int xe = maxima[3 * pi] + 1, ye = maxima[3 * pi + 1] + 1, ze = maxima[3 * pi + 2] + 1;
        prod[pi] = prodbuf[pi];
        for (int x = 0; x < xe; ++x)
            for (int y = 0; y < ye; ++y)
                for (int zz = 0; zz < ze; ++zz)
                    prod[pi][(x * ye + y) * ze + zz] = hx[0][x] * hx[1][y] * hx[2][zz];
    }

    const double p = ab->p, q = cd->p;
    const double rho = p * q / (p + q);
    cplx disp[3];
    for (int i = 0; i < 3; ++i) disp[i] = ab->Pc[i] - cd->Pc[i];
    const cplx arg = rho * (disp[0] * disp[0] + disp[1] * disp[1] + disp[2] * disp[2]);
    const int scaled = creal(arg) < 0.0;
    if (!w->boys_valid || w->boys_arg != arg || w->boys_scaled != scaled || w->boys_nmax < L) {
        int region;
        double e;
        long s;
        int rc = or_boys(creal(arg), cimag(arg), L, scaled, (double*)w->boys, &region, &e, &s);
        if (rc) return rc;
        w->boys_arg = arg;
        w->boys_scaled = scaled;
        w->boys_nmax = L;
        w->boys_valid = 1;
    }

    cplx common = ab->london * cd->london;
    if (scaled) {
        double rd[3], tw[3], wc[3];
        for (int i = 0; i < 3; ++i) {
            rd[i] = ab->P[i] - cd->P[i];
            tw[i] = ab->q[i] + cd->q[i];
            wc[i] = (p * ab->P[i] + q * cd->P[i]) / (p + q);
        }
        const double re = -rho * (rd[0] * rd[0] + rd[1] * rd[1] + rd[2] * rd[2]) -
                          (tw[0] * tw[0] + tw[1] * tw[1] + tw[2] * tw[2]) / (4.0 * (p + q));
        common = cexp(CMPLX(re, -(tw[0] * wc[0] + tw[1] * wc[1] + tw[2] * wc[2])));
    }

    cplx contraction = 0.0;
    if (L == 0) {
        contraction = common * w->boys[0];
    } else if (real_zero) {
        /* collapsed real table (src/eri.cpp:215-282) */
        const int comb[3] = {maxima[0] + maxima[3], maxima[1] + maxima[4], maxima[2] + maxima[5]};
        const size_t orders = (size_t)L + 1;
        const size_t st[3] = {(size_t)(comb[1] + 1) * (comb[2] + 1) * orders, (size_t)(comb[2] + 1) * orders, orders};
        const size_t size = (size_t)(comb[0] + 1) * st[0];
        if (ws_raux(w, size)) return -3;
        double* t = w->raux;
        double radial = 1.0;
        for (int n = 0; n <= L; ++n) {
            t[n] = radial * creal(w->boys[n]);
            radial *= -2.0 * rho;
        }
        for (int x = 0; x <= comb[0]; ++x)
            for (int y = 0; y <= comb[1]; ++y)
                for (int zz = 0; zz <= comb[2]; ++zz) {
                    const int deg = x + y + zz;
                    if (deg == 0) continue;
                    const int axis = x > 0 ? 0 : (y > 0 ? 1 : 2);
                    const int power = axis == 0 ? x : (axis == 1 ? y : zz);
                    const size_t idx = x * st[0] + y * st[1] + zz * st[2];
                    const size_t lower = idx - st[axis];
                    const double shift = creal(disp[axis]);
                    for (int n = 0; n <= L - deg; ++n) {
                        double val = shift * t[lower + n + 1];
                        if (power > 1) val += (double)(power - 1) * t[lower - st[axis] + n + 1];
                        t[idx + n] = val;
                    }
                }
        double rc = 0.0;
        for (int tt = 0; tt <= maxima[0]; ++tt)
            for (int u = 0; u <= maxima[1]; ++u)
                for (int v = 0; v <= maxima[2]; ++v) {
                    const double cab = prod[0][(tt * (maxima[1] + 1) + u) * (maxima[2] + 1) + v];
                    for (int ta = 0; ta <= maxima[3]; ++ta)
                        for (int ph = 0; ph <= maxima[4]; ++ph)
                            for (int ch = 0; ch <= maxima[5]; ++ch) {
                                const double sign = (ta + ph + ch) % 2 == 0 ? 1.0 : -1.0;
                                rc += cab * prod[1][(ta * (maxima[4] + 1) + ph) * (maxima[5] + 1) + ch] *
                                      (sign * t[(tt + ta) * st[0] + (u + ph) * st[1] + (v + ch) * st[2]]);
                            }
                }
        contraction = rc;
    } else {
        /* six-index complex recurrence (src/eri.cpp:283-368) */
        const size_t orders = (size_t)L + 1;
        size_t st[6];
        st[5] = orders;
        for (int ax = 5; ax > 0; --ax) st[ax - 1] = st[ax] * (size_t)(maxima[ax] + 1);
        const size_t entries = st[0] * (size_t)(maxima[0] + 1) / orders;
        if (ws_aux(w, entries * orders)) return -3;
        cplx* a = w->aux;
        double radial = 1.0;
        for (int n = 0; n <= L; ++n) {
            a[n] = common * radial * w->boys[n];
            radial *= -2.0 * rho;
        }
        const double waves[6] = {ab->q[0], ab->q[1], ab->q[2], cd->q[0], cd->q[1], cd->q[2]};
        for (size_t e = 1; e < entries; ++e) {
            int pw[6];
            size_t rem = e;
            int deg = 0;
            for (int ax = 6; ax-- > 0;) {
                pw[ax] = (int)(rem % (size_t)(maxima[ax] + 1));
                rem /= (size_t)(maxima[ax] + 1);
                deg += pw[ax];
            }
            int axis = 0;
            while (pw[axis] == 0) ++axis;
            const size_t idx = e * orders;
            const size_t lower = idx - st[axis];
            const int coord = axis % 3;
            const cplx shift = axis < 3 ? disp[coord] : -disp[coord];
            const cplx wave = CMPLX(0.0, -waves[axis]);
            for (int n = 0; n <= L - deg; ++n) {
                cplx val = wave * a[lower + n];
                val += shift * a[lower + n + 1];
                if (pw[axis] > 1) val += (double)(pw[axis] - 1) * a[lower - st[axis] + n + 1];
                if (axis < 3 && pw[axis + 3] > 0) val -= (double)pw[axis + 3] * a[lower - st[axis + 3] + n + 1];
                a[idx + n] = val;
            }
        }
        const int aye = maxima[1] + 1, aze = maxima[2] + 1, cye = maxima[4] + 1, cze = maxima[5] + 1;
        for (int tt = 0; tt <= maxima[0]; ++tt)
            for (int u = 0; u <= maxima[1]; ++u)
                for (int v = 0; v <= maxima[2]; ++v) {
                    const double cab = prod[0][(tt * aye + u) * aze + v];
                    for (int ta = 0; ta <= maxima[3]; ++ta)
                        for (int ph = 0; ph <= maxima[4]; ++ph)
                            for (int ch = 0; ch <= maxima[5]; ++ch)
                                contraction += cab * prod[1][(ta * cye + ph) * cze + ch] *
                                               a[tt * st[0] + u * st[1] + v * st[2] + ta * st[3] + ph * st[4] +
                                                 ch * st[5]];
                }
    }
    const double pref = 2.0 * pow(M_PI, 2.5) / (p * q * sqrt(p + q));
    *result = pref * ab->K * cd->K * contraction;
    return 0;
}

static int eri_kernel(const prim_t* pr, const pair_t* ab, const pair_t* cd, int real_zero, ws_t* w, cplx* result) {
    return eri_kernel_h(pr, ab, cd, real_zero, w, NULL, result);
}

/* 1-D Hermite coefficients of a primitive pair for every pair of axis powers
 * (a <= la, b <= lb) on each axis: h[((ax * (la + 1) + a) * (lb + 1) + b) *
 * (la + lb + 1) + t]. */
static double* pair_hermite_cache(int la, int lb, const double* A, const double* Bc, const pair_t* pd) {
    const size_t stride = (size_t)(la + lb + 1);
    double* h = (double*)malloc(sizeof(double) * 3 * (size_t)(la + 1) * (size_t)(lb + 1) * stride);
    if (!h) return NULL;
    for (int ax = 0; ax < 3; ++ax)
        for (int a = 0; a <= la; ++a)
            for (int b = 0; b <= lb; ++b)
                hermite_1d(a, b, A[ax], Bc[ax], pd->P[ax], pd->p,
                           h + (((size_t)ax * (la + 1) + a) * (lb + 1) + b) * stride);
    return h;
}

/* primitive_eri (src/eri.cpp:438-452) with the primitive's own coefficient
 * and optional normalisation (src/eri.cpp:371-383). */
int or_primitive_eri(const double* exps, const double* centers, const int* angular, const double* coefs,
                     const int* normalized, const double* B, const double* O, double* out) {
    field_t f;
    memcpy(f.B, B, sizeof f.B);
    memcpy(f.O, O, sizeof f.O);
    prim_t pr[4];
    for (int i = 0; i < 4; ++i) {
        if (!isfinite(exps[i]) || exps[i] <= 0.0) return set_err(-1, "Gaussian exponent must be finite and positive");
        pr[i].alpha = exps[i];
        for (int k = 0; k < 3; ++k) {
            pr[i].center[k] = centers[3 * i + k];
            pr[i].ang[k] = angular[3 * i + k];
        }
    }
    pair_t ab, cd;
    gaussian_product(pr[0].alpha, pr[0].center, pr[1].alpha, pr[1].center, &f, &ab);
    gaussian_product(pr[2].alpha, pr[2].center, pr[3].alpha, pr[3].center, &f, &cd);
    const int real_zero = B[0] == 0.0 && B[1] == 0.0 && B[2] == 0.0;
    ws_t w;
    memset(&w, 0, sizeof w);
    cplx v;
    int rc = eri_kernel(pr, &ab, &cd, real_zero, &w, &v);
    ws_free(&w);
    if (rc) return rc;
    double scale = 1.0;
    for (int i = 0; i < 4; ++i) {
        scale *= coefs[i];
        if (normalized[i]) scale *= or_primitive_normalization(pr[i].alpha, pr[i].ang[0], pr[i].ang[1], pr[i].ang[2]);
    }
    v *= scale;
    out[0] = creal(v);
    out[1] = cimag(v);
    return 0;
}

/* ------------------------------------------------------------------ */
/* basis and shell quartets (src/eri.cpp:454-585)                       */
/* ------------------------------------------------------------------ */

typedef struct {
    int ns;
    const double* centers;
    const int* ls;
    const int* nprims;
    const int* ncontrs;
    const double* exps;   /* concatenated */
    const double* coefs;  /* concatenated, already contraction-normalised */
    size_t* eoff;
    size_t* coff;
    size_t* aooff;
    size_t nao;
} basis_t;

static int basis_init(basis_t* b, int ns, const double* centers, const int* ls, const int* nprims, const int* ncontrs,
                      const double* exps, const double* coefs) {
    b->ns = ns;
    b->centers = centers;
    b->ls = ls;
    b->nprims = nprims;
    b->ncontrs = ncontrs;
    b->exps = exps;
    b->coefs = coefs;
    b->eoff = (size_t*)malloc(sizeof(size_t) * (ns + 1));
    b->coff = (size_t*)malloc(sizeof(size_t) * (ns + 1));
    b->aooff = (size_t*)malloc(sizeof(size_t) * (ns + 1));
    size_t e = 0, c = 0, a = 0;
    for (int s = 0; s < ns; ++s) {
        if (ls[s] < 0 || ls[s] > 16) return set_err(-1, "shell angular momentum out of supported range");
        b->eoff[s] = e;
        b->coff[s] = c;
        b->aooff[s] = a;
        e += nprims[s];
        c += (size_t)nprims[s] * ncontrs[s];
        a += (size_t)ncontrs[s] * (ls[s] + 1) * (ls[s] + 2) / 2;
    }
    b->eoff[ns] = e;
    b->coff[ns] = c;
    b->aooff[ns] = a;
    b->nao = a;
    return 0;
}

static void basis_free(basis_t* b) {
    free(b->eoff);
    free(b->coff);
    free(b->aooff);
}

static inline int ncart(int l) { return (l + 1) * (l + 2) / 2; }
static inline size_t shell_ao(const basis_t* b, int s) { return (size_t)b->ncontrs[s] * ncart(b->ls[s]); }

static int shell_quartet(const basis_t* bs, const int* sh, const field_t* f, ws_t* w, cplx* out) {
    int comps[4][153][3];
    int nc[4];
    size_t shape[4];
    for (int k = 0; k < 4; ++k) {
        nc[k] = cart_components(bs->ls[sh[k]], comps[k]);
        shape[k] = shell_ao(bs, sh[k]);
    }
    const size_t total = shape[0] * shape[1] * shape[2] * shape[3];
    for (size_t i = 0; i < total; ++i) out[i] = 0.0;
    /* per-component primitive normalisations (src/eri.cpp:474-487) */
    double* norms[4];
    for (int k = 0; k < 4; ++k) {
        const int s = sh[k];
        norms[k] = (double*)malloc(sizeof(double) * nc[k] * bs->nprims[s]);
        for (int c = 0; c < nc[k]; ++c)
            for (int p = 0; p < bs->nprims[s]; ++p)
                norms[k][c * bs->nprims[s] + p] =
                    or_primitive_normalization(bs->exps[bs->eoff[s] + p], comps[k][c][0], comps[k][c][1], comps[k][c][2]);
    }
    const int real_zero = f->B[0] == 0.0 && f->B[1] == 0.0 && f->B[2] == 0.0;
    const int sa = sh[0], sb = sh[1], sc = sh[2], sd = sh[3];
    const double* A = bs->centers + 3 * sa;
    const double* Bc = bs->centers + 3 * sb;
    const double* C = bs->centers + 3 * sc;
    const double* D = bs->centers + 3 * sd;
    int rc = 0;
    w->boys_valid = 0;
    const int la = bs->ls[sa], lb = bs->ls[sb], lc = bs->ls[sc], ld = bs->ls[sd];
    const size_t sab = (size_t)(la + lb + 1), scd = (size_t)(lc + ld + 1);
    for (int pa = 0; pa < bs->nprims[sa] && !rc; ++pa)
        for (int pb = 0; pb < bs->nprims[sb] && !rc; ++pb) {
            pair_t ab;
            gaussian_product(bs->exps[bs->eoff[sa] + pa], A, bs->exps[bs->eoff[sb] + pb], Bc, f, &ab);
            double* hab = pair_hermite_cache(la, lb, A, Bc, &ab);
            if (!hab) {
                rc = set_err(-3, "out of memory");
                break;
            }
            for (int pc = 0; pc < bs->nprims[sc] && !rc; ++pc)
                for (int pd = 0; pd < bs->nprims[sd] && !rc; ++pd) {
                    pair_t cd;
                    gaussian_product(bs->exps[bs->eoff[sc] + pc], C, bs->exps[bs->eoff[sd] + pd], D, f, &cd);
                    double* hcd = pair_hermite_cache(lc, ld, C, D, &cd);
                    if (!hcd) {
                        rc = set_err(-3, "out of memory");
                        break;
                    }
                    const int pidx[4] = {pa, pb, pc, pd};
                    for (int ca = 0; ca < nc[0] && !rc; ++ca)
                        for (int cb = 0; cb < nc[1] && !rc; ++cb)
                            for (int cc = 0; cc < nc[2] && !rc; ++cc)
                                for (int cdd = 0; cdd < nc[3] && !rc; ++cdd) {
                                    const int cix[4] = {ca, cb, cc, cdd};
                                    prim_t pr[4];
                                    for (int k = 0; k < 4; ++k) {
                                        const int s = sh[k];
                                        pr[k].alpha = bs->exps[bs->eoff[s] + pidx[k]];
                                        for (int x = 0; x < 3; ++x) {
                                            pr[k].center[x] = bs->centers[3 * s + x];
                                            pr[k].ang[x] = comps[k][cix[k]][x];
                                        }
                                    }
                                    const double* hin[6];
                                    for (int ax = 0; ax < 3; ++ax) {
                                        hin[ax] = hab + (((size_t)ax * (la + 1) + comps[0][ca][ax]) * (lb + 1) +
                                                         comps[1][cb][ax]) * sab;
                                        hin[3 + ax] = hcd + (((size_t)ax * (lc + 1) + comps[2][cc][ax]) * (ld + 1) +
                                                             comps[3][cdd][ax]) * scd;
                                    }
                                    cplx val;
                                    rc = eri_kernel_h(pr, &ab, &cd, real_zero, w, hin, &val);
                                    if (rc) break;
                                    for (int k = 0; k < 4; ++k)
                                        val *= norms[k][cix[k] * bs->nprims[sh[k]] + pidx[k]];
                                    for (int xa = 0; xa < bs->ncontrs[sa]; ++xa) {
                                        const size_t ia = (size_t)xa * nc[0] + ca;
                                        const double ka = bs->coefs[bs->coff[sa] + (size_t)xa * bs->nprims[sa] + pa];
                                        for (int xb = 0; xb < bs->ncontrs[sb]; ++xb) {
                                            const size_t ib = (size_t)xb * nc[1] + cb;
                                            const double kb = bs->coefs[bs->coff[sb] + (size_t)xb * bs->nprims[sb] + pb];
                                            for (int xc = 0; xc < bs->ncontrs[sc]; ++xc) {
                                                const size_t ic = (size_t)xc * nc[2] + cc;
                                                const double kc =
                                                    bs->coefs[bs->coff[sc] + (size_t)xc * bs->nprims[sc] + pc];
                                                for (int xd = 0; xd < bs->ncontrs[sd]; ++xd) {
                                                    const size_t id = (size_t)xd * nc[3] + cdd;
                                                    const double kd =
                                                        bs->coefs[bs->coff[sd] + (size_t)xd * bs->nprims[sd] + pd];
                                                    out[((ia * shape[1] + ib) * shape[2] + ic) * shape[3] + id] +=
                                                        ka * kb * kc * kd * val;
                                                }
                                            }
                                        }
                                    }
                                }
                    free(hcd);
                }
            free(hab);
        }
    for (int k = 0; k < 4; ++k) free(norms[k]);
    return rc;
}

#define BASIS_ARGS int ns, const double *centers, const int *ls, const int *nprims, const int *ncontrs, \
                   const double *exps, const double *coefs

int or_eri_shell(BASIS_ARGS, const int* sh, const double* B, const double* O, double* out) {
    basis_t bs;
    int rc = basis_init(&bs, ns, centers, ls, nprims, ncontrs, exps, coefs);
    if (!rc) {
        for (int k = 0; k < 4; ++k)
            if (sh[k] < 0 || sh[k] >= ns) rc = set_err(-2, "ERI shell-quartet index is out of range");
    }
    if (!rc) {
        field_t f;
        memcpy(f.B, B, sizeof f.B);
        memcpy(f.O, O, sizeof f.O);
        ws_t w;
        memset(&w, 0, sizeof w);
        rc = shell_quartet(&bs, sh, &f, &w, (cplx*)out);
        ws_free(&w);
    }
    basis_free(&bs);
    return rc;
}

/* Packed batch (src/eri.cpp:644-767): blocks in input order; offsets[i] is
 * the complex-element offset of block i (offsets has nq+1 entries). */
int or_eri_batch(BASIS_ARGS, const uint32_t* quartets, long nq, const double* B, const double* O, int threads,
                 double* out, long* offsets) {
    basis_t bs;
    int rc = basis_init(&bs, ns, centers, ls, nprims, ncontrs, exps, coefs);
    if (rc) {
        basis_free(&bs);
        return rc;
    }
    long pos = 0;
    for (long i = 0; i < nq; ++i) {
        offsets[i] = pos;
        size_t sz = 1;
        for (int k = 0; k < 4; ++k) {
            if (quartets[4 * i + k] >= (uint32_t)ns) {
                basis_free(&bs);
                return set_err(-2, "ERI shell-quartet index is out of range");
            }
            sz *= shell_ao(&bs, (int)quartets[4 * i + k]);
        }
        pos += (long)sz;
    }
    offsets[nq] = pos;
    field_t f;
    memcpy(f.B, B, sizeof f.B);
    memcpy(f.O, O, sizeof f.O);
    int failed = 0;
    char first_err[512] = {0};
#pragma omp parallel num_threads(threads > 0 ? threads : 1)
    {
        ws_t w;
        memset(&w, 0, sizeof w);
#pragma omp for schedule(dynamic, 1)
        for (long i = 0; i < nq; ++i) {
            if (failed) continue;
            const int sh[4] = {(int)quartets[4 * i], (int)quartets[4 * i + 1], (int)quartets[4 * i + 2],
                               (int)quartets[4 * i + 3]};
            int r = shell_quartet(&bs, sh, &f, &w, (cplx*)out + offsets[i]);
            if (r) {
#pragma omp critical(or_batch_err)
                {
                    if (!failed) {
                        failed = r;
                        snprintf(first_err, sizeof first_err, "%s", g_err);
                    }
                }
            }
        }
        ws_free(&w);
    }
    basis_free(&bs);
    if (failed) return set_err(failed, first_err);
    return 0;
}

/* canonical representative of the four-member finite-field orbit
 * (src/eri.cpp:414-429) */
static int is_canonical(int a, int b, int c, int d) {
    const int cand[3][4] = {{c, d, a, b}, {b, a, d, c}, {d, c, b, a}};
    const int q[4] = {a, b, c, d};
    for (int k = 0; k < 3; ++k) {
        for (int i = 0; i < 4; ++i) {
            if (cand[k][i] < q[i]) return 0;
            if (cand[k][i] > q[i]) break;
        }
    }
    return 1;
}

long or_canonical_quartets(int ns, uint32_t* out) {
    long n = 0;
    for (int a = 0; a < ns; ++a)
        for (int b = 0; b < ns; ++b)
            for (int c = 0; c < ns; ++c)
                for (int d = 0; d < ns; ++d)
                    if (is_canonical(a, b, c, d)) {
                        if (out) {
                            out[4 * n] = a;
                            out[4 * n + 1] = b;
                            out[4 * n + 2] = c;
                            out[4 * n + 3] = d;
                        }
                        ++n;
                    }
    return n;
}

/* Full symmetric tensor (src/eri.cpp:777-847). */
int or_eri_full(BASIS_ARGS, const double* B, const double* O, int threads, double* out) {
    basis_t bs;
    int rc = basis_init(&bs, ns, centers, ls, nprims, ncontrs, exps, coefs);
    const size_t n = bs.nao;
    basis_free(&bs);
    if (rc) return rc;
    const long nq = or_canonical_quartets(ns, NULL);
    uint32_t* q = (uint32_t*)malloc(sizeof(uint32_t) * 4 * (nq > 0 ? nq : 1));
    or_canonical_quartets(ns, q);
    long* off = (long*)malloc(sizeof(long) * (nq + 1));
    /* total packed size */
    rc = basis_init(&bs, ns, centers, ls, nprims, ncontrs, exps, coefs);
    size_t packed = 0;
    for (long i = 0; i < nq; ++i) {
        size_t sz = 1;
        for (int k = 0; k < 4; ++k) sz *= shell_ao(&bs, (int)q[4 * i + k]);
        packed += sz;
    }
    cplx* vals = (cplx*)malloc(sizeof(cplx) * (packed > 0 ? packed : 1));
    rc = or_eri_batch(ns, centers, ls, nprims, ncontrs, exps, coefs, q, nq, B, O, threads, (double*)vals, off);
    cplx* o = (cplx*)out;
    if (!rc) {
        memset(o, 0, sizeof(cplx) * n * n * n * n);
        for (long i = 0; i < nq; ++i) {
            const int s[4] = {(int)q[4 * i], (int)q[4 * i + 1], (int)q[4 * i + 2], (int)q[4 * i + 3]};
            size_t sh[4];
            for (int k = 0; k < 4; ++k) sh[k] = shell_ao(&bs, s[k]);
            const cplx* blk = vals + off[i];
            for (size_t ia = 0; ia < sh[0]; ++ia)
                for (size_t ib = 0; ib < sh[1]; ++ib)
                    for (size_t ic = 0; ic < sh[2]; ++ic)
                        for (size_t id = 0; id < sh[3]; ++id) {
                            const cplx v = blk[((ia * sh[1] + ib) * sh[2] + ic) * sh[3] + id];
                            const size_t ga = bs.aooff[s[0]] + ia, gb = bs.aooff[s[1]] + ib, gc = bs.aooff[s[2]] + ic,
                                         gd = bs.aooff[s[3]] + id;
                            o[((ga * n + gb) * n + gc) * n + gd] = v;
                            o[((gc * n + gd) * n + ga) * n + gb] = v;
                            o[((gb * n + ga) * n + gd) * n + gc] = conj(v);
                            o[((gd * n + gc) * n + gb) * n + ga] = conj(v);
                        }
        }
    }
    basis_free(&bs);
    free(vals);
    free(off);
    free(q);
    return rc;
}

/* Schwarz factors Q_ab = nextafter(sqrt(max|(ab|ba)|)(1+64 eps)) (src/eri.cpp:587-619). */
int or_schwarz(BASIS_ARGS, const double* B, const double* O, double* out) {
    basis_t bs;
    int rc = basis_init(&bs, ns, centers, ls, nprims, ncontrs, exps, coefs);
    field_t f;
    memcpy(f.B, B, sizeof f.B);
    memcpy(f.O, O, sizeof f.O);
    ws_t w;
    memset(&w, 0, sizeof w);
    for (int a = 0; a < ns && !rc; ++a)
        for (int b = a; b < ns && !rc; ++b) {
            const size_t na = shell_ao(&bs, a), nb = shell_ao(&bs, b);
            cplx* blk = (cplx*)malloc(sizeof(cplx) * na * nb * nb * na);
            const int sh[4] = {a, b, b, a};
            rc = shell_quartet(&bs, sh, &f, &w, blk);
            double m = 0.0;
            for (size_t i = 0; i < na; ++i)
                for (size_t j = 0; j < nb; ++j) m = fmax(m, cabs(blk[((i * nb + j) * nb + j) * na + i]));
            free(blk);
            const double bound = nextafter(sqrt(m) * (1.0 + 64.0 * 2.220446049250313e-16), INFINITY);
            out[a * ns + b] = bound;
            out[b * ns + a] = bound;
        }
    ws_free(&w);
    basis_free(&bs);
    return rc;
}

/* ------------------------------------------------------------------ */
/* Cholesky selected entries (src/cholesky.cpp:17-323)                  */
/* ------------------------------------------------------------------ */

/* One contracted AO-level entry (mu nu|lam sig) for AOs local to shells sh,
 * via the full-shell kernel (the reference's selected path is bitwise equal
 * to full shells: tests/python/test_cholesky_selected.py). */
static int one_entry(const basis_t* bs, const int* sh, const size_t* local, const field_t* f, ws_t* w, cplx* value,
                     cplx* scratch, size_t* scratch_shape) {
    (void)scratch_shape;
    int rc = shell_quartet(bs, sh, f, w, scratch);
    if (rc) return rc;
    size_t s[4];
    for (int k = 0; k < 4; ++k) s[k] = shell_ao(bs, sh[k]);
    *value = scratch[((local[0] * s[1] + local[1]) * s[2] + local[2]) * s[3] + local[3]];
    return 0;
}

static int* shell_owner(const basis_t* bs) {
    int* o = (int*)malloc(sizeof(int) * (bs->nao > 0 ? bs->nao : 1));
    for (int s = 0; s < bs->ns; ++s)
        for (size_t i = bs->aooff[s]; i < bs->aooff[s + 1]; ++i) o[i] = s;
    return o;
}

/* Diagonal D[(mu,nu)] = Re(mu nu|nu mu), placed as src/cholesky.cpp:305-311. */
int or_cholesky_diagonal(BASIS_ARGS, const long* pairs, long npairs, const double* B, const double* O, int threads,
                         double* out) {
    basis_t bs;
    int rc = basis_init(&bs, ns, centers, ls, nprims, ncontrs, exps, coefs);
    if (rc) {
        basis_free(&bs);
        return rc;
    }
    const size_t n = bs.nao;
    memset(out, 0, sizeof(double) * n * n);
    for (long i = 0; i < npairs; ++i) {
        const long a = pairs[2 * i], b = pairs[2 * i + 1];
        if (a < 0 || b < 0 || a >= ns || b >= ns || a > b) {
            basis_free(&bs);
            return set_err(-2, "Cholesky diagonal shell pair must be valid and ordered");
        }
    }
    field_t f;
    memcpy(f.B, B, sizeof f.B);
    memcpy(f.O, O, sizeof f.O);
    int failed = 0;
#pragma omp parallel num_threads(threads > 0 ? threads : 1)
    {
        ws_t w;
        memset(&w, 0, sizeof w);
#pragma omp for schedule(dynamic, 1)
        for (long i = 0; i < npairs; ++i) {
            const int a = (int)pairs[2 * i], b = (int)pairs[2 * i + 1];
            const int sh[4] = {a, b, b, a};
            const size_t na = shell_ao(&bs, a), nb = shell_ao(&bs, b);
            cplx* blk = (cplx*)malloc(sizeof(cplx) * na * nb * nb * na);
            int r = shell_quartet(&bs, sh, &f, &w, blk);
            if (r) {
#pragma omp atomic write
                failed = r;
            } else {
                for (size_t ii = 0; ii < na; ++ii)
                    for (size_t jj = 0; jj < nb; ++jj) {
                        const double v = creal(blk[((ii * nb + jj) * nb + jj) * na + ii]);
                        const size_t mu = bs.aooff[a] + ii, nu = bs.aooff[b] + jj;
                        out[nu * n + mu] = v;
                        if (a != b) out[mu * n + nu] = v;
                    }
            }
            free(blk);
        }
        ws_free(&w);
    }
    basis_free(&bs);
    return failed;
}

/* Columns out[k, mu, nu] = (mu nu | p1 p0) for pivots (p0,p1) sharing one
 * shell pair (src/cholesky.cpp:203-282).  real != 0 selects the zero-phase
 * real path: only b >= a shell pairs, mirrored, same-shell entries averaged.
 * Output is float64[k][n][n] when real, complex128 otherwise. */
int or_cholesky_columns(BASIS_ARGS, const long* pivots, long npiv, const double* B, const double* O, int threads,
                        int real, double* out) {
    (void)one_entry;
    basis_t bs;
    int rc = basis_init(&bs, ns, centers, ls, nprims, ncontrs, exps, coefs);
    if (rc) {
        basis_free(&bs);
        return rc;
    }
    const size_t n = bs.nao;
    if (npiv == 0) {
        basis_free(&bs);
        return 0;
    }
    for (long k = 0; k < npiv; ++k)
        if (pivots[2 * k] < 0 || pivots[2 * k + 1] < 0 || (size_t)pivots[2 * k] >= n || (size_t)pivots[2 * k + 1] >= n) {
            basis_free(&bs);
            return set_err(-2, "Cholesky pivot AO index is out of range");
        }
    int* owner = shell_owner(&bs);
    const int sa = owner[pivots[0]], sb = owner[pivots[1]];
    for (long k = 0; k < npiv; ++k)
        if (owner[pivots[2 * k]] != sa || owner[pivots[2 * k + 1]] != sb) {
            free(owner);
            basis_free(&bs);
            return set_err(-1, "Cholesky candidate pivots must share a shell pair");
        }
    field_t f;
    memcpy(f.B, B, sizeof f.B);
    memcpy(f.O, O, sizeof f.O);
    /* group list: (a,b) with b >= a in the real path, all pairs otherwise */
    long ng = 0;
    int* ga = (int*)malloc(sizeof(int) * ns * ns);
    int* gb = (int*)malloc(sizeof(int) * ns * ns);
    for (int a = 0; a < ns; ++a)
        for (int b = real ? a : 0; b < ns; ++b) {
            ga[ng] = a;
            gb[ng] = b;
            ++ng;
        }
    int failed = 0;
#pragma omp parallel num_threads(threads > 0 ? threads : 1)
    {
        ws_t w;
        memset(&w, 0, sizeof w);
#pragma omp for schedule(dynamic, 1)
        for (long g = 0; g < ng; ++g) {
            const int a = ga[g], b = gb[g];
            const int sh[4] = {a, b, sb, sa};
            const size_t na = shell_ao(&bs, a), nb = shell_ao(&bs, b), nc = shell_ao(&bs, sb), nd = shell_ao(&bs, sa);
            cplx* blk = (cplx*)malloc(sizeof(cplx) * na * nb * nc * nd);
            int r = shell_quartet(&bs, sh, &f, &w, blk);
            if (r) {
#pragma omp atomic write
                failed = r;
            } else {
                for (long k = 0; k < npiv; ++k) {
                    const size_t c = (size_t)pivots[2 * k + 1] - bs.aooff[sb];
                    const size_t d = (size_t)pivots[2 * k] - bs.aooff[sa];
                    for (size_t i = 0; i < na; ++i)
                        for (size_t j = 0; j < nb; ++j) {
                            const cplx v = blk[((i * nb + j) * nc + c) * nd + d];
                            const size_t mu = bs.aooff[a] + i, nu = bs.aooff[b] + j;
                            if (real) {
                                double s = creal(v);
                                if (a == b) s = (s + creal(blk[((j * nb + i) * nc + c) * nd + d])) * 0.5;
                                out[(k * n + mu) * n + nu] = s;
                                if (a != b) out[(k * n + nu) * n + mu] = s;
                            } else {
                                ((cplx*)out)[(k * n + mu) * n + nu] = v;
                            }
                        }
                }
            }
            free(blk);
        }
        ws_free(&w);
    }
    free(ga);
    free(gb);
    free(owner);
    basis_free(&bs);
    return failed;
}


/* ------------------------------------------------------------------ */
/* nuclear attraction (src/nuclear.cpp:27-170, 207-330)                 */
/* ------------------------------------------------------------------ */

/* One primitive pair and one point charge, unit coefficients and no
 * primitive normalisation (the reference's NuclearKernel::compute): the
 * four-index table R^n_{tuv} of the complex displacement P' - C with the
 * -i q terms of the London phase, filled by increasing degree t+u+v. */
static int nuclear_kernel(const prim_t* a, const prim_t* b, double Z, const double* C, const field_t* f, cplx* out) {
    pair_t pr;
    gaussian_product(a->alpha, a->center, b->alpha, b->center, f, &pr);
    const int mx = a->ang[0] + b->ang[0], my = a->ang[1] + b->ang[1], mz = a->ang[2] + b->ang[2];
    const int L = mx + my + mz;
    if (L > 32) return set_err(-1, "nuclear attraction supports combined angular order through 32");
    double herm[3][34];
    for (int ax = 0; ax < 3; ++ax)
        hermite_1d(a->ang[ax], b->ang[ax], a->center[ax], b->center[ax], pr.P[ax], pr.p, herm[ax]);
    cplx d[3];
    for (int i = 0; i < 3; ++i) d[i] = pr.Pc[i] - C[i];
    const cplx arg = pr.p * (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const int scaled = creal(arg) < 0.0;
    cplx boys[33];
    int region;
    double e;
    long segs;
    int rc = or_boys(creal(arg), cimag(arg), L, scaled, (double*)boys, &region, &e, &segs);
    if (rc) return rc;
    cplx common = pr.london;
    if (scaled) {
        const double dx = pr.P[0] - C[0], dy = pr.P[1] - C[1], dz = pr.P[2] - C[2];
        const double qc = pr.q[0] * C[0] + pr.q[1] * C[1] + pr.q[2] * C[2];
        common = cexp(CMPLX(-pr.p * (dx * dx + dy * dy + dz * dz), -qc));
    }
    const size_t sx = (size_t)(my + 1) * (mz + 1), sy = (size_t)(mz + 1), per_n = (size_t)(mx + 1) * sx;
    cplx* R = (cplx*)calloc((size_t)(L + 1) * per_n, sizeof(cplx));
    if (!R) return set_err(-3, "out of memory");
#define RN(n, t, u, v) R[(size_t)(n) * per_n + (size_t)(t) * sx + (size_t)(u) * sy + (size_t)(v)]
    double radial = 1.0;
    for (int n = 0; n <= L; ++n) {
        RN(n, 0, 0, 0) = common * radial * boys[n];
        radial *= -2.0 * pr.p;
    }
    for (int deg = 1; deg <= L; ++deg)
        for (int t = 0; t <= mx && t <= deg; ++t)
            for (int u = 0; u <= my && t + u <= deg; ++u) {
                const int v = deg - t - u;
                if (v > mz) continue;
                for (int n = 0; n + deg <= L; ++n) {
                    cplx val;
                    if (t > 0) {
                        val = CMPLX(0.0, -pr.q[0]) * RN(n, t - 1, u, v) + d[0] * RN(n + 1, t - 1, u, v);
                        if (t > 1) val += (double)(t - 1) * RN(n + 1, t - 2, u, v);
                    } else if (u > 0) {
                        val = CMPLX(0.0, -pr.q[1]) * RN(n, t, u - 1, v) + d[1] * RN(n + 1, t, u - 1, v);
                        if (u > 1) val += (double)(u - 1) * RN(n + 1, t, u - 2, v);
                    } else {
                        val = CMPLX(0.0, -pr.q[2]) * RN(n, t, u, v - 1) + d[2] * RN(n + 1, t, u, v - 1);
                        if (v > 1) val += (double)(v - 1) * RN(n + 1, t, u, v - 2);
                    }
                    RN(n, t, u, v) = val;
                }
            }
    cplx acc = 0.0;
    for (int t = 0; t <= mx; ++t)
        for (int u = 0; u <= my; ++u)
            for (int v = 0; v <= mz; ++v) acc += herm[0][t] * herm[1][u] * herm[2][v] * RN(0, t, u, v);
#undef RN
    free(R);
    *out = -Z * (2.0 * M_PI / pr.p) * pr.K * acc;
    return 0;
}

/* Full AO matrix out[mu][nu] (complex, row-major n x n): every ordered shell
 * pair, primitive pairs and Cartesian components in the reference's loop
 * order (src/nuclear.cpp:207-302), coefficients (contraction-normalised) and
 * primitive normalisations applied per component. */
int or_nuclear_matrix(BASIS_ARGS, int nnuc, const double* charges, const double* ncenters, const double* B,
                      const double* O, double* out_) {
    basis_t bs;
    int rc = basis_init(&bs, ns, centers, ls, nprims, ncontrs, exps, coefs);
    cplx* out = (cplx*)out_;
    if (!rc) {
        field_t f;
        memcpy(f.B, B, sizeof f.B);
        memcpy(f.O, O, sizeof f.O);
        const size_t n = bs.nao;
        for (size_t i = 0; i < n * n; ++i) out[i] = 0.0;
        int ca[153][3], cb[153][3];
        for (int sa = 0; sa < ns && !rc; ++sa)
            for (int sb = 0; sb < ns && !rc; ++sb) {
                const int na = cart_components(ls[sa], ca), nb = cart_components(ls[sb], cb);
                for (int pa = 0; pa < nprims[sa] && !rc; ++pa)
                    for (int pb = 0; pb < nprims[sb] && !rc; ++pb)
                        for (int ia = 0; ia < na && !rc; ++ia)
                            for (int ib = 0; ib < nb && !rc; ++ib) {
                                prim_t a, b;
                                a.alpha = exps[bs.eoff[sa] + pa];
                                b.alpha = exps[bs.eoff[sb] + pb];
                                for (int x = 0; x < 3; ++x) {
                                    a.center[x] = centers[3 * sa + x];
                                    b.center[x] = centers[3 * sb + x];
                                    a.ang[x] = ca[ia][x];
                                    b.ang[x] = cb[ib][x];
                                }
                                cplx v = 0.0;
                                for (int c = 0; c < nnuc && !rc; ++c) {
                                    cplx term;
                                    rc = nuclear_kernel(&a, &b, charges[c], ncenters + 3 * c, &f, &term);
                                    v += term;
                                }
                                if (rc) break;
                                v *= or_primitive_normalization(a.alpha, a.ang[0], a.ang[1], a.ang[2]) *
                                     or_primitive_normalization(b.alpha, b.ang[0], b.ang[1], b.ang[2]);
                                for (int xa = 0; xa < ncontrs[sa]; ++xa)
                                    for (int xb = 0; xb < ncontrs[sb]; ++xb) {
                                        const size_t mu = bs.aooff[sa] + (size_t)xa * na + ia;
                                        const size_t nu = bs.aooff[sb] + (size_t)xb * nb + ib;
                                        out[mu * n + nu] += coefs[bs.coff[sa] + (size_t)xa * nprims[sa] + pa] *
                                                            coefs[bs.coff[sb] + (size_t)xb * nprims[sb] + pb] * v;
                                    }
                            }
            }
    }
    basis_free(&bs);
    return rc;
}

/* ------------------------------------------------------------------ */
/* ERI centre derivatives (src/derivatives.cpp:53-87, 215-245, 556-640,  */
/* 954-959)                                                             */
/* ------------------------------------------------------------------ */

/* Unit-coefficient primitive ERI with the angular part of slot k replaced. */
static int eri_shifted(const prim_t* pr, int k, const int* ang, const pair_t* ab, const pair_t* cd, int real_zero,
                       ws_t* w, cplx* v) {
    prim_t q[4];
    memcpy(q, pr, sizeof q);
    for (int x = 0; x < 3; ++x) q[k].ang[x] = ang[x];
    return eri_kernel(q, ab, cd, real_zero, w, v);
}

/* d/dR_slot,axis of one primitive quartet (raw primitives: coefficient 1,
 * no normalisation): -l e(l-1) + 2 alpha e(l+1) + i phi sum_c (B x e_axis)_c
 * [e(l+1_c) + R_c e(l)], phi = +1/2 on the bra side of each pair (slots 0,
 * 2), -1/2 on the ket side (src/derivatives.cpp:53-87). */
static int primitive_center_derivatives(const prim_t* pr, const pair_t* ab, const pair_t* cd, const field_t* f,
                                        int real_zero, ws_t* w, cplx* out12) {
    cplx base;
    int rc = eri_kernel(pr, ab, cd, real_zero, w, &base);
    if (rc) return rc;
    for (int k = 0; k < 4; ++k) {
        const double phi = (k % 2 == 0) ? 0.5 : -0.5;
        cplx up[3];
        for (int c = 0; c < 3; ++c) {
            int a[3] = {pr[k].ang[0], pr[k].ang[1], pr[k].ang[2]};
            ++a[c];
            if ((rc = eri_shifted(pr, k, a, ab, cd, real_zero, w, &up[c]))) return rc;
        }
        for (int axis = 0; axis < 3; ++axis) {
            cplx r = 2.0 * pr[k].alpha * up[axis];
            if (pr[k].ang[axis] > 0) {
                int a[3] = {pr[k].ang[0], pr[k].ang[1], pr[k].ang[2]};
                --a[axis];
                cplx dn;
                if ((rc = eri_shifted(pr, k, a, ab, cd, real_zero, w, &dn))) return rc;
                r -= (double)pr[k].ang[axis] * dn;
            }
            /* (B x e_axis) */
            double e[3] = {0.0, 0.0, 0.0};
            e[axis] = 1.0;
            const double bx[3] = {f->B[1] * e[2] - f->B[2] * e[1], f->B[2] * e[0] - f->B[0] * e[2],
                                  f->B[0] * e[1] - f->B[1] * e[0]};
            for (int c = 0; c < 3; ++c) {
                const double coef = phi * bx[c];
                if (coef == 0.0) continue;
                r += CMPLX(0.0, coef) * (up[c] + pr[k].center[c] * base);
            }
            out12[3 * k + axis] = r;
        }
    }
    return 0;
}

/* d/dB_b of one primitive quartet (raw primitives): sum over slots k of
 * i phi_k sum_c (e_b x (R_k - O))_c [e(l_k + 1_c) + R_{k,c} e(l)], phi = +1/2
 * on slots 0, 2 and -1/2 on slots 1, 3 (src/derivatives.cpp:88-106, 268-280). */
static int primitive_magnetic_derivatives(const prim_t* pr, const pair_t* ab, const pair_t* cd, const field_t* f,
                                          int real_zero, ws_t* w, cplx* out3) {
    cplx base;
    int rc = eri_kernel(pr, ab, cd, real_zero, w, &base);
    if (rc) return rc;
    cplx up[4][3];
    for (int k = 0; k < 4; ++k)
        for (int c = 0; c < 3; ++c) {
            int a[3] = {pr[k].ang[0], pr[k].ang[1], pr[k].ang[2]};
            ++a[c];
            if ((rc = eri_shifted(pr, k, a, ab, cd, real_zero, w, &up[k][c]))) return rc;
        }
    for (int b = 0; b < 3; ++b) {
        cplx r = 0.0;
        for (int k = 0; k < 4; ++k) {
            const double phi = (k % 2 == 0) ? 0.5 : -0.5;
            double d[3], e[3] = {0.0, 0.0, 0.0};
            for (int x = 0; x < 3; ++x) d[x] = pr[k].center[x] - f->O[x];
            e[b] = 1.0;
            const double ph[3] = {e[1] * d[2] - e[2] * d[1], e[2] * d[0] - e[0] * d[2], e[0] * d[1] - e[1] * d[0]};
            cplx t = 0.0;
            for (int c = 0; c < 3; ++c) {
                const double coef = phi * ph[c];
                if (coef == 0.0) continue;
                t += CMPLX(0.0, coef) * (up[k][c] + pr[k].center[c] * base);
            }
            r += t;
        }
        out3[b] = r;
    }
    return 0;
}

/* ERI of quartet q with slot j shifted by +1_c (j < 0: none). */
static int eval_shift(const prim_t* q, int j, int c, const pair_t* ab, const pair_t* cd, int real_zero, ws_t* w,
                      cplx* v) {
    prim_t t[4];
    memcpy(t, q, sizeof t);
    if (j >= 0) ++t[j].ang[c];
    return eri_kernel(t, ab, cd, real_zero, w, v);
}

/* d/dB_b of quartet q (all four slots' London response, src/derivatives.cpp:88-106, 268-280). */
static int magnetic_of(const prim_t* q, int b, const pair_t* ab, const pair_t* cd, const field_t* f, int real_zero,
                       ws_t* w, cplx* out) {
    cplx base;
    int rc = eval_shift(q, -1, 0, ab, cd, real_zero, w, &base);
    if (rc) return rc;
    cplx r = 0.0;
    for (int j = 0; j < 4; ++j) {
        const double phi = (j % 2 == 0) ? 0.5 : -0.5;
        double d[3], e[3] = {0.0, 0.0, 0.0};
        for (int x = 0; x < 3; ++x) d[x] = q[j].center[x] - f->O[x];
        e[b] = 1.0;
        const double ph[3] = {e[1] * d[2] - e[2] * d[1], e[2] * d[0] - e[0] * d[2], e[0] * d[1] - e[1] * d[0]};
        for (int c = 0; c < 3; ++c) {
            const double coef = phi * ph[c];
            if (coef == 0.0) continue;
            cplx up;
            if ((rc = eval_shift(q, j, c, ab, cd, real_zero, w, &up))) return rc;
            r += CMPLX(0.0, coef) * (up + q[j].center[c] * base);
        }
    }
    *out = r;
    return 0;
}

/* d2/dR_{k,r} dB_b of one primitive quartet, index (k*3 + r)*3 + b: the centre
 * response of slot k applied to the field derivative, plus the cross term
 * i phi_k sum_c (e_b x e_r)_c [e(l_k + 1_c) + R_{k,c} e]
 * (src/derivatives.cpp:160-181, 232-245). */
static int primitive_mixed_derivatives(const prim_t* pr, const pair_t* ab, const pair_t* cd, const field_t* f,
                                       int real_zero, ws_t* w, cplx* out36) {
    int rc;
    cplx base;
    if ((rc = eval_shift(pr, -1, 0, ab, cd, real_zero, w, &base))) return rc;
    for (int k = 0; k < 4; ++k) {
        const double phi = (k % 2 == 0) ? 0.5 : -0.5;
        cplx up[3];
        for (int c = 0; c < 3; ++c)
            if ((rc = eval_shift(pr, k, c, ab, cd, real_zero, w, &up[c]))) return rc;
        for (int b = 0; b < 3; ++b) {
            /* field derivative of the quartet with slot k shifted: +1_c (c = 0..2), -1_r, raw */
            cplx mup[3], mraw;
            for (int c = 0; c < 3; ++c) {
                prim_t q[4];
                memcpy(q, pr, sizeof q);
                ++q[k].ang[c];
                if ((rc = magnetic_of(q, b, ab, cd, f, real_zero, w, &mup[c]))) return rc;
            }
            if ((rc = magnetic_of(pr, b, ab, cd, f, real_zero, w, &mraw))) return rc;
            for (int r = 0; r < 3; ++r) {
                cplx v = 2.0 * pr[k].alpha * mup[r];
                if (pr[k].ang[r] > 0) {
                    prim_t q[4];
                    memcpy(q, pr, sizeof q);
                    --q[k].ang[r];
                    cplx mdn;
                    if ((rc = magnetic_of(q, b, ab, cd, f, real_zero, w, &mdn))) return rc;
                    v -= (double)pr[k].ang[r] * mdn;
                }
                double e[3] = {0.0, 0.0, 0.0};
                e[r] = 1.0;
                const double bx[3] = {f->B[1] * e[2] - f->B[2] * e[1], f->B[2] * e[0] - f->B[0] * e[2],
                                      f->B[0] * e[1] - f->B[1] * e[0]};
                for (int c = 0; c < 3; ++c) {
                    const double coef = phi * bx[c];
                    if (coef == 0.0) continue;
                    v += CMPLX(0.0, coef) * (mup[c] + pr[k].center[c] * mraw);
                }
                /* (e_b x e_r) */
                double eb[3] = {0.0, 0.0, 0.0};
                eb[b] = 1.0;
                const double cr[3] = {eb[1] * e[2] - eb[2] * e[1], eb[2] * e[0] - eb[0] * e[2],
                                      eb[0] * e[1] - eb[1] * e[0]};
                for (int c = 0; c < 3; ++c) {
                    const double coef = phi * cr[c];
                    if (coef == 0.0) continue;
                    v += CMPLX(0.0, coef) * (up[c] + pr[k].center[c] * base);
                }
                out36[(k * 3 + r) * 3 + b] = v;
            }
        }
    }
    return 0;
}

/* Blocks (ncomp, na, nb, nc, nd) of nq shell quartets packed in input order,
 * primitive and component loops of compute_quartet_block
 * (src/derivatives.cpp:556-640): ncomp = 12 centre derivatives (slot-major)
 * or 3 magnetic derivatives. */
static int derivative_blocks(BASIS_ARGS, const uint32_t* quartets, long nq, const double* B, const double* O,
                             double* out_, int mode) {
    const int magnetic = mode == 1;
    const int ncomp = mode == 2 ? 36 : (magnetic ? 3 : 12);
    basis_t bs;
    int rc = basis_init(&bs, ns, centers, ls, nprims, ncontrs, exps, coefs);
    cplx* out = (cplx*)out_;
    field_t f;
    memcpy(f.B, B, sizeof f.B);
    memcpy(f.O, O, sizeof f.O);
    const int real_zero = B[0] == 0.0 && B[1] == 0.0 && B[2] == 0.0;
    ws_t w;
    memset(&w, 0, sizeof w);
    size_t off = 0;
    static int comps[4][153][3];
    for (long qi = 0; qi < nq && !rc; ++qi) {
        int sh[4], nc[4];
        size_t shape[4];
        for (int k = 0; k < 4; ++k) {
            sh[k] = (int)quartets[4 * qi + k];
            if (sh[k] < 0 || sh[k] >= ns) {
                rc = set_err(-2, "derivative shell quartet index is out of range");
                break;
            }
            nc[k] = cart_components(ls[sh[k]], comps[k]);
            shape[k] = shell_ao(&bs, sh[k]);
        }
        if (rc) break;
        const size_t block = shape[0] * shape[1] * shape[2] * shape[3];
        cplx* o = out + off;
        for (size_t i = 0; i < (size_t)ncomp * block; ++i) o[i] = 0.0;
        w.boys_valid = 0;
        for (int pa = 0; pa < nprims[sh[0]] && !rc; ++pa)
            for (int pb = 0; pb < nprims[sh[1]] && !rc; ++pb) {
                pair_t ab;
                gaussian_product(exps[bs.eoff[sh[0]] + pa], centers + 3 * sh[0], exps[bs.eoff[sh[1]] + pb],
                                 centers + 3 * sh[1], &f, &ab);
                for (int pc = 0; pc < nprims[sh[2]] && !rc; ++pc)
                    for (int pd = 0; pd < nprims[sh[3]] && !rc; ++pd) {
                        pair_t cd;
                        gaussian_product(exps[bs.eoff[sh[2]] + pc], centers + 3 * sh[2], exps[bs.eoff[sh[3]] + pd],
                                         centers + 3 * sh[3], &f, &cd);
                        const int pidx[4] = {pa, pb, pc, pd};
                        for (int ca = 0; ca < nc[0] && !rc; ++ca)
                            for (int cb = 0; cb < nc[1] && !rc; ++cb)
                                for (int cc = 0; cc < nc[2] && !rc; ++cc)
                                    for (int cdd = 0; cdd < nc[3] && !rc; ++cdd) {
                                        const int cix[4] = {ca, cb, cc, cdd};
                                        prim_t pr[4];
                                        double norm = 1.0;
                                        for (int k = 0; k < 4; ++k) {
                                            pr[k].alpha = exps[bs.eoff[sh[k]] + pidx[k]];
                                            for (int x = 0; x < 3; ++x) {
                                                pr[k].center[x] = centers[3 * sh[k] + x];
                                                pr[k].ang[x] = comps[k][cix[k]][x];
                                            }
                                            norm *= or_primitive_normalization(pr[k].alpha, pr[k].ang[0],
                                                                               pr[k].ang[1], pr[k].ang[2]);
                                        }
                                        cplx d12[36];
                                        rc = mode == 2 ? primitive_mixed_derivatives(pr, &ab, &cd, &f, real_zero, &w, d12)
                                             : magnetic
                                                 ? primitive_magnetic_derivatives(pr, &ab, &cd, &f, real_zero, &w, d12)
                                                 : primitive_center_derivatives(pr, &ab, &cd, &f, real_zero, &w, d12);
                                        if (rc) break;
                                        for (int xa = 0; xa < ncontrs[sh[0]]; ++xa)
                                            for (int xb = 0; xb < ncontrs[sh[1]]; ++xb)
                                                for (int xc = 0; xc < ncontrs[sh[2]]; ++xc)
                                                    for (int xd = 0; xd < ncontrs[sh[3]]; ++xd) {
                                                        const double kk =
                                                            norm *
                                                            coefs[bs.coff[sh[0]] + (size_t)xa * nprims[sh[0]] + pa] *
                                                            coefs[bs.coff[sh[1]] + (size_t)xb * nprims[sh[1]] + pb] *
                                                            coefs[bs.coff[sh[2]] + (size_t)xc * nprims[sh[2]] + pc] *
                                                            coefs[bs.coff[sh[3]] + (size_t)xd * nprims[sh[3]] + pd];
                                                        const size_t e =
                                                            ((((size_t)xa * nc[0] + ca) * shape[1] +
                                                              (size_t)xb * nc[1] + cb) * shape[2] +
                                                             (size_t)xc * nc[2] + cc) * shape[3] +
                                                            (size_t)xd * nc[3] + cdd;
                                                        for (int dd = 0; dd < ncomp; ++dd)
                                                            o[dd * block + e] += kk * d12[dd];
                                                    }
                                    }
                    }
            }
        off += (size_t)ncomp * block;
    }
    ws_free(&w);
    basis_free(&bs);
    return rc;
}

int or_eri_center_derivatives(BASIS_ARGS, const uint32_t* quartets, long nq, const double* B, const double* O,
                              double* out) {
    return derivative_blocks(ns, centers, ls, nprims, ncontrs, exps, coefs, quartets, nq, B, O, out, 0);
}

int or_eri_magnetic_derivatives(BASIS_ARGS, const uint32_t* quartets, long nq, const double* B, const double* O,
                                double* out) {
    return derivative_blocks(ns, centers, ls, nprims, ncontrs, exps, coefs, quartets, nq, B, O, out, 1);
}

int or_eri_mixed_derivatives(BASIS_ARGS, const uint32_t* quartets, long nq, const double* B, const double* O,
                             double* out) {
    return derivative_blocks(ns, centers, ls, nprims, ncontrs, exps, coefs, quartets, nq, B, O, out, 2);
}

/* Derivative-density Schwarz factors of every ordered shell pair
 * (src/derivatives.cpp:1307-1372): for primitives (a, b) with coefficients
 * N(alpha, component), n(a', b') = sqrt|(b' a'|a' b')|; slot s, axis x:
 * 2 alpha n(+1_x) + l_x n(-1_x) + sum_c |(B x e_x)_c| / 2 (n(+1_c) + |R_c| n),
 * contracted with |w_a w_b|, maximised, padded by (1 + 128 eps) and one ulp. */
static double bound_norm(const prim_t* left, const prim_t* right, double cl, double cr, const field_t* f,
                         int real_zero, ws_t* w, int* rc) {
    prim_t q[4] = {*right, *left, *left, *right};
    pair_t ab, cd;
    gaussian_product(right->alpha, right->center, left->alpha, left->center, f, &ab);
    gaussian_product(left->alpha, left->center, right->alpha, right->center, f, &cd);
    cplx v;
    w->boys_valid = 0;
    *rc = eri_kernel(q, &ab, &cd, real_zero, w, &v);
    return sqrt(cabs(v * (cl * cr) * (cl * cr)));
}

int or_eri_derivative_bounds(BASIS_ARGS, const double* B, const double* O, double* out) {
    basis_t bs;
    int rc = basis_init(&bs, ns, centers, ls, nprims, ncontrs, exps, coefs);
    field_t f;
    memcpy(f.B, B, sizeof f.B);
    memcpy(f.O, O, sizeof f.O);
    const int real_zero = B[0] == 0.0 && B[1] == 0.0 && B[2] == 0.0;
    ws_t w;
    memset(&w, 0, sizeof w);
    static int comps[2][153][3];
    for (int sa = 0; sa < ns && !rc; ++sa)
        for (int sb = 0; sb < ns && !rc; ++sb) {
            const int na = cart_components(ls[sa], comps[0]), nb = cart_components(ls[sb], comps[1]);
            const int xa_n = ncontrs[sa], xb_n = ncontrs[sb];
            double* contracted = (double*)malloc(sizeof(double) * 6 * xa_n * xb_n);
            double maximum = 0.0;
            for (int ca = 0; ca < na && !rc; ++ca)
                for (int cb = 0; cb < nb && !rc; ++cb) {
                    for (int i = 0; i < 6 * xa_n * xb_n; ++i) contracted[i] = 0.0;
                    for (int pa = 0; pa < nprims[sa] && !rc; ++pa)
                        for (int pb = 0; pb < nprims[sb] && !rc; ++pb) {
                            prim_t g[2];
                            const int sh[2] = {sa, sb}, pp[2] = {pa, pb}, cc[2] = {ca, cb};
                            double cf[2];
                            for (int k = 0; k < 2; ++k) {
                                g[k].alpha = exps[bs.eoff[sh[k]] + pp[k]];
                                for (int x = 0; x < 3; ++x) {
                                    g[k].center[x] = centers[3 * sh[k] + x];
                                    g[k].ang[x] = comps[k][cc[k]][x];
                                }
                                cf[k] = or_primitive_normalization(g[k].alpha, g[k].ang[0], g[k].ang[1], g[k].ang[2]);
                            }
                            double pb6[6];
                            for (int slot = 0; slot < 2 && !rc; ++slot) {
                                const prim_t* raw = &g[slot];
                                prim_t base_l = g[0], base_r = g[1];
                                const double n0 = bound_norm(&base_l, &base_r, cf[0], cf[1], &f, real_zero, &w, &rc);
                                for (int axis = 0; axis < 3 && !rc; ++axis) {
                                    prim_t ch[2] = {g[0], g[1]};
                                    ch[slot].ang[axis] += 1;
                                    double bound = 2.0 * raw->alpha *
                                                   bound_norm(&ch[0], &ch[1], cf[0], cf[1], &f, real_zero, &w, &rc);
                                    if (raw->ang[axis] != 0) {
                                        prim_t dn[2] = {g[0], g[1]};
                                        dn[slot].ang[axis] -= 1;
                                        bound += (double)raw->ang[axis] *
                                                 bound_norm(&dn[0], &dn[1], cf[0], cf[1], &f, real_zero, &w, &rc);
                                    }
                                    double e[3] = {0.0, 0.0, 0.0};
                                    e[axis] = 1.0;
                                    const double ph[3] = {B[1] * e[2] - B[2] * e[1], B[2] * e[0] - B[0] * e[2],
                                                          B[0] * e[1] - B[1] * e[0]};
                                    for (int c = 0; c < 3; ++c) {
                                        const double wgt = 0.5 * fabs(ph[c]);
                                        if (wgt == 0.0) continue;
                                        prim_t up[2] = {g[0], g[1]};
                                        up[slot].ang[c] += 1;
                                        bound += wgt * (bound_norm(&up[0], &up[1], cf[0], cf[1], &f, real_zero, &w, &rc) +
                                                        fabs(raw->center[c]) * n0);
                                    }
                                    pb6[slot * 3 + axis] = bound;
                                }
                            }
                            for (int xa = 0; xa < xa_n; ++xa)
                                for (int xb = 0; xb < xb_n; ++xb) {
                                    const double wgt = fabs(coefs[bs.coff[sa] + (size_t)xa * nprims[sa] + pa] *
                                                            coefs[bs.coff[sb] + (size_t)xb * nprims[sb] + pb]);
                                    for (int k = 0; k < 6; ++k) contracted[(xa * xb_n + xb) * 6 + k] += wgt * pb6[k];
                                }
                        }
                    for (int i = 0; i < 6 * xa_n * xb_n; ++i) maximum = fmax(maximum, contracted[i]);
                }
            free(contracted);
            out[(size_t)sa * ns + sb] = nextafter(maximum * (1.0 + 128.0 * 2.220446049250313e-16), INFINITY);
        }
    ws_free(&w);
    basis_free(&bs);
    return rc;
}
