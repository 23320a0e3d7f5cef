/*
 * CPU oracle for the CRMod/CRTomo forward + sensitivity hot path.
 *
 * TEST INFRASTRUCTURE ONLY -- see crt_oracle.h.  This file restates the
 * reference Fortran routines in C, in the reference's loop order and
 * operation order, so that the CUDA product can be checked against it.
 * It is compiled by oracle/Makefile into oracle/_build/libcrt_oracle.so and
 * loaded by tests/, __graft_entry__.smoke() and bench.py's CPU baseline only.
 *
 * Build flags keep floating-point contraction off (-ffp-contract=off) so the
 * oracle gives the same bits on x86_64 and aarch64.
 */
#include "crt_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* complex arithmetic on (re, im) pairs                                */
/* ------------------------------------------------------------------ */
typedef struct { double re, im; } cx;

static inline cx cmk(double r, double i) { cx z; z.re = r; z.im = i; return z; }
static inline cx cadd(cx a, cx b) { return cmk(a.re + b.re, a.im + b.im); }
static inline cx csub(cx a, cx b) { return cmk(a.re - b.re, a.im - b.im); }
static inline cx cmul(cx a, cx b) {
    return cmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
static inline cx cscale(cx a, double s) { return cmk(a.re * s, a.im * s); }
/* textbook quotient (the reference is built with -ffast-math, which selects
 * the limited-range formula) */
static inline cx cdiv(cx a, cx b) {
    double d = b.re * b.re + b.im * b.im;
    return cmk((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}
static inline double cabs_(cx a) { return sqrt(a.re * a.re + a.im * a.im); }
/* principal branch square root (cdsqrt) */
static inline cx csqrt_(cx z) {
    double r = cabs_(z);
    if (r == 0.0) return cmk(0.0, 0.0);
    if (z.re >= 0.0) {
        double t = sqrt(0.5 * (r + z.re));
        return cmk(t, z.im / (2.0 * t));
    } else {
        double t = sqrt(0.5 * (r - z.re));
        return cmk(fabs(z.im) / (2.0 * t), copysign(t, z.im));
    }
}
static inline cx clog_(cx z) { return cmk(log(cabs_(z)), atan2(z.im, z.re)); }
static inline cx cexp_(cx z) {
    double e = exp(z.re);
    return cmk(e * cos(z.im), e * sin(z.im));
}
static inline cx cconj(cx a) { return cmk(a.re, -a.im); }

#define CX(p, i) (((cx *)(p))[(i)])

static const double PI_ = 3.14159265358979323846264338327950288;

/* ------------------------------------------------------------------ */
/* modified Bessel functions: Abramowitz & Stegun 9.8.1 - 9.8.8        */
/* polynomial approximations with the branch points of                  */
/* src/bessi0.f90, src/bessi1.f90, src/bessk0.f90, src/bessk1.f90      */
/* ------------------------------------------------------------------ */
static double as_i0(double x) {
    double ax = fabs(x);
    if (ax < 3.75) { /* A&S 9.8.1 */
        double t = (x / 3.75) * (x / 3.75);
        return 1.0 + t * (3.5156229 + t * (3.0899424 + t * (1.2067492 +
               t * (0.2659732 + t * (0.0360768 + t * 0.0045813)))));
    }
    double u = 3.75 / ax; /* A&S 9.8.2 */
    return (exp(ax) / sqrt(ax)) * (0.39894228 + u * (0.01328592 + u * (0.00225319 +
           u * (-0.00157565 + u * (0.00916281 + u * (-0.02057706 + u * (0.02635537 +
           u * (-0.01647633 + u * 0.00392377))))))));
}

static double as_i1(double x) {
    double ax = fabs(x);
    if (ax < 3.75) { /* A&S 9.8.3 */
        double t = (x / 3.75) * (x / 3.75);
        return x * (0.5 + t * (0.87890594 + t * (0.51498869 + t * (0.15084934 +
               t * (0.02658733 + t * (0.00301532 + t * 0.00032411))))));
    }
    double u = 3.75 / ax; /* A&S 9.8.4 */
    return (exp(ax) / sqrt(ax)) * (0.39894228 + u * (-0.03988024 + u * (-0.00362018 +
           u * (0.00163801 + u * (-0.01031555 + u * (0.02282967 + u * (-0.02895312 +
           u * (0.01787654 + u * -0.00420059))))))));
}

double or_bessk0(double x) {
    if (x <= 2.0) { /* A&S 9.8.5 */
        double t = x * x / 4.0;
        return (-log(x / 2.0) * as_i0(x)) + (-0.57721566 + t * (0.42278420 +
               t * (0.23069756 + t * (0.03488590 + t * (0.00262698 +
               t * (0.00010750 + t * 0.0000074))))));
    } else if (x > 500.0) {
        return 0.0;
    }
    double u = 2.0 / x; /* A&S 9.8.6 */
    return (exp(-x) / sqrt(x)) * (1.25331414 + u * (-0.07832358 + u * (0.02189568 +
           u * (-0.01062446 + u * (0.00587872 + u * (-0.00251540 + u * 0.00053208))))));
}

double or_bessk1(double x) {
    if (x <= 2.0) { /* A&S 9.8.7 */
        double t = x * x / 4.0;
        return (log(x / 2.0) * as_i1(x)) + (1.0 / x) * (1.0 + t * (0.15443144 +
               t * (-0.67278579 + t * (-0.18156897 + t * (-0.01919402 +
               t * (-0.00110404 + t * -0.00004686))))));
    } else if (x > 500.0) {
        return 0.0;
    }
    double u = 2.0 / x; /* A&S 9.8.8 */
    return (exp(-x) / sqrt(x)) * (1.25331414 + u * (0.23498619 + u * (-0.03655620 +
           u * (0.01504268 + u * (-0.00780353 + u * (0.00325614 + u * -0.00068245))))));
}

/* ------------------------------------------------------------------ */
/* Gauss rules (written from the mathematics: Newton iteration on the   */
/* three-term recurrences)                                              */
/* ------------------------------------------------------------------ */

/* Legendre nodes/weights on (x1, x2); nodes ascending.  Used by
 * src/rwaven.f90:129 through src/gauleg.f90. */
static void gauss_legendre(double x1, double x2, double *x, double *w, int n) {
    double xm = 0.5 * (x2 + x1), xl = 0.5 * (x2 - x1);
    for (int i = 1; i <= (n + 1) / 2; i++) {
        /* Tricomi's asymptotic guess for the i-th largest root */
        double z = cos(PI_ * (i - 0.25) / (n + 0.5)), dp = 1.0;
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = z;
            for (int j = 2; j <= n; j++) {
                double p2 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p0) / j;
                p0 = p1; p1 = p2;
            }
            if (n == 1) { p1 = z; p0 = 1.0; }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            double dz = p1 / dp;
            z -= dz;
            if (fabs(dz) <= 3e-14) break;
        }
        /* derivative at the converged root */
        {
            double p0 = 1.0, p1 = z;
            for (int j = 2; j <= n; j++) {
                double p2 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p0) / j;
                p0 = p1; p1 = p2;
            }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
        }
        x[i - 1] = xm - xl * z;
        x[n - i] = xm + xl * z;
        w[i - 1] = 2.0 * xl / ((1.0 - z * z) * dp * dp);
        w[n - i] = w[i - 1];
    }
}

/* Laguerre polynomial L_n and derivative at z */
static void laguerre_eval(int n, double z, double *ln, double *dln) {
    double p0 = 1.0, p1 = 1.0 - z;
    if (n == 0) { *ln = 1.0; *dln = 0.0; return; }
    for (int j = 2; j <= n; j++) {
        double p2 = ((2.0 * j - 1.0 - z) * p1 - (j - 1.0) * p0) / j;
        p0 = p1; p1 = p2;
    }
    *ln = p1;
    *dln = n * (p1 - p0) / z;
}

/* Gauss-Laguerre (alpha = 0) nodes ascending and weights.  The roots are
 * bracketed by a sign scan on (0, 4n+2) and polished by Newton.  Used by
 * src/rwaven.f90:146 through src/gaulag.f90. */
static void gauss_laguerre(double *x, double *w, int n) {
    double hi = 4.0 * n + 2.0;
    int nscan = 4000 * n, found = 0;
    double zprev = 1e-12, fprev, d;
    laguerre_eval(n, zprev, &fprev, &d);
    for (int s = 1; s <= nscan && found < n; s++) {
        double z = hi * s / nscan, f;
        laguerre_eval(n, z, &f, &d);
        if ((f < 0.0) != (fprev < 0.0)) {
            double a = zprev, b = z, r = 0.5 * (a + b);
            for (int it = 0; it < 200; it++) { /* safeguarded Newton */
                double fr, dr;
                laguerre_eval(n, r, &fr, &dr);
                double rn = r - fr / dr;
                if (!(rn > a && rn < b)) rn = 0.5 * (a + b);
                double fa, da;
                laguerre_eval(n, a, &fa, &da);
                if ((fr < 0.0) == (fa < 0.0)) a = r; else b = r;
                if (fabs(rn - r) <= 3e-14 * (1.0 + fabs(r))) { r = rn; break; }
                r = rn;
            }
            double fr, dr;
            laguerre_eval(n, r, &fr, &dr);
            x[found] = r;
            w[found] = 1.0 / (r * dr * dr);
            found++;
        }
        zprev = z; fprev = f;
    }
}

/* ------------------------------------------------------------------ */
/* mesh helpers                                                         */
/* ------------------------------------------------------------------ */
#define NREL(m, iel, k) ((m)->nrel[((k) - 1) * (m)->ld_nrel + ((iel) - 1)])
#define SX(m, node) ((m)->sx[(m)->snr[(node) - 1] - 1])
#define SY(m, node) ((m)->sy[(m)->snr[(node) - 1] - 1])

int or_counts(const or_mesh *m, int *elanz, int *relanz, int *maxnk) {
    int e = 0, r = 0, mx = 0;
    for (int i = 0; i < m->typanz; i++) {
        if (m->typ[i] > 10) r += m->nelanz[i]; else e += m->nelanz[i];
        if (m->selanz[i] > mx) mx = m->selanz[i];
    }
    *elanz = e; *relanz = r; *maxnk = mx;
    return 0;
}

static void decode(int code, int *a, int *b) {
    /* src/bvolt.f90:44-49: elec1 = mod(code, 10000), elec2 = code / 10000 */
    *a = code % 10000;
    *b = (code - *a) / 10000;
}

/* src/rwaven.f90:22-171 */
int or_rwaven(const or_mesh *m, double *kwn, double *kwnwi) {
    double amin = 1e9, amax = 0.0;
    double xke[4] = {0, 0, 0, 0}, yke[4] = {0, 0, 0, 0};
    for (int i = 0; i < m->nanz; i++) {
        int el[4];
        decode(m->strnr[i], &el[0], &el[1]);
        decode(m->vnr[i], &el[2], &el[3]);
        for (int j = 0; j < 4; j++)
            if (el[j] > 0) {
                xke[j] = SX(m, m->enr[el[j] - 1]);
                yke[j] = SY(m, m->enr[el[j] - 1]);
            }
        for (int r = 2; r < 4; r++) {
            if (el[r] <= 0) continue;
            for (int j = 0; j < 2; j++) {
                if (el[j] <= 0) continue;
                double dx = xke[r] - xke[j], dy = yke[r] - yke[j];
                double d = sqrt(dx * dx + dy * dy);
                amin = fmin(d, amin);
                amax = fmax(d, amax);
            }
        }
    }
    if (amin < 1e-12 || amax < 1e-12) return -73;
    int lanz = 4;
    int ganz = (int)(float)(6.0 * log10(amax / amin));
    if (ganz < 2) ganz = 2;
    if (ganz > 30 - lanz) ganz = 30 - lanz;
    double kwn0 = 1.0 / (2.0 * amin);
    gauss_legendre(0.0, 1.0, kwn, kwnwi, ganz);
    for (int i = 0; i < ganz; i++) {
        kwnwi[i] = 2.0 * kwn0 * kwnwi[i] * kwn[i];
        kwn[i] = kwn0 * kwn[i] * kwn[i];
    }
    gauss_laguerre(kwn + ganz, kwnwi + ganz, lanz);
    for (int i = ganz; i < ganz + lanz; i++) {
        kwnwi[i] = kwn0 * kwnwi[i] * exp(kwn[i]);
        kwn[i] = kwn0 * (kwn[i] + 1.0);
    }
    return ganz + lanz;
}

/* src/refsig.f90:7-73 */
void or_refsig(const or_mesh *m, const double *sigma, double *sigma0) {
    int iel = 0;
    double area = 0.0;
    cx s0 = cmk(0, 0);
    for (int i = 0; i < m->typanz; i++) {
        for (int j = 0; j < m->nelanz[i]; j++) {
            iel++;
            if (m->typ[i] > 10) continue;
            double xk = SX(m, NREL(m, iel, 1)), yk = SY(m, NREL(m, iel, 1));
            double ax = SX(m, NREL(m, iel, 2)) - xk, ay = SY(m, NREL(m, iel, 2)) - yk;
            double bx = SX(m, NREL(m, iel, 3)) - xk, by = SY(m, NREL(m, iel, 3)) - yk;
            double dum = 0.0;
            if (m->typ[i] == 3) {
                dum = fabs(ax * by - ay * bx) / 2.0;
            } else if (m->typ[i] == 5 || m->typ[i] == 8) {
                double cx_ = SX(m, NREL(m, iel, 4)) - xk, cy = SY(m, NREL(m, iel, 4)) - yk;
                dum = (fabs(ax * by - ay * bx) + fabs(bx * cy - by * cx_)) / 2.0;
            }
            s0 = cadd(s0, cscale(clog_(CX(sigma, iel - 1)), dum));
            area += dum;
        }
    }
    cx r = cexp_(cmk(s0.re / area, s0.im / area));
    sigma0[0] = r.re; sigma0[1] = r.im;
}

/* src/bsytop.f90:7-71 */
double or_bsytop(const or_mesh *m) {
    double sytop = 0.0;
    int iel = 0;
    for (int i = 0; i < m->typanz; i++) {
        if (m->typ[i] == 12) {
            int nkel = m->selanz[i];
            sytop = 0.0;
            for (int j = 1; j <= m->nelanz[i]; j++) {
                iel++;
                double sp = 0.0;
                for (int ik = 1; ik <= nkel; ik++) sp += SY(m, NREL(m, iel, ik));
                sp = sp / nkel;
                if (j == 1) sytop = sp;
                else sytop = (sytop * (j - 1) + sp) / j;
            }
        } else {
            iel += m->nelanz[i];
        }
    }
    return sytop;
}

/* ------------------------------------------------------------------ */
/* element matrices                                                     */
/* ------------------------------------------------------------------ */
static const int S1T[3][3] = {{1, -1, 0}, {-1, 1, 0}, {0, 0, 0}};
static const int S2T[3][3] = {{2, -1, -1}, {-1, 0, 1}, {-1, 1, 0}};
static const int S3T[3][3] = {{1, 0, -1}, {0, 0, 0}, {-1, 0, 1}};
static const int S4T[3][3] = {{2, 1, 1}, {1, 2, 1}, {1, 1, 2}};

/* src/elem1.f90:17-67 (2-node boundary line, mass matrix only) */
static void elem1(const double *xk, const double *yk, double elmam[4][4]) {
    static const int s4[2][2] = {{2, 1}, {1, 2}};
    double x21 = xk[1] - xk[0], y21 = yk[1] - yk[0];
    double l = sqrt(x21 * x21 + y21 * y21);
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) elmam[i][j] = l * (double)s4[i][j] / 6.0;
}

/* src/elem3.f90:27-99 (linear triangle) */
static int elem3(const double *xk, const double *yk, double elmas[4][4], double elmam[4][4]) {
    double x21 = xk[1] - xk[0], x31 = xk[2] - xk[0];
    double y21 = yk[1] - yk[0], y31 = yk[2] - yk[0];
    double det = x21 * y31 - x31 * y21;
    if (det <= 0.0) return 26;
    double a = (x31 * x31 + y31 * y31) / det;
    double b = -(x31 * x21 + y31 * y21) / det;
    double c = (x21 * x21 + y21 * y21) / det;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            elmas[i][j] = (a * S1T[i][j] + b * S2T[i][j] + c * S3T[i][j]) / 2.0;
            elmam[i][j] = det * S4T[i][j] / 24.0;
        }
    return 0;
}

/* src/elem5.f90 (bilinear parallelogram) */
static int elem5(const double *xk, const double *yk, double elmas[4][4], double elmam[4][4]) {
    static const int s1[4][4] = {{2, -2, -1, 1}, {-2, 2, 1, -1}, {-1, 1, 2, -2}, {1, -1, -2, 2}};
    static const int s2[4][4] = {{1, 0, -1, 0}, {0, -1, 0, 1}, {-1, 0, 1, 0}, {0, 1, 0, -1}};
    static const int s3[4][4] = {{2, 1, -1, -2}, {1, 2, -2, -1}, {-1, -2, 2, 1}, {-2, -1, 1, 2}};
    static const int s4[4][4] = {{4, 2, 1, 2}, {2, 4, 2, 1}, {1, 2, 4, 2}, {2, 1, 2, 4}};
    double x21 = xk[1] - xk[0], x31 = xk[3] - xk[0];
    double y21 = yk[1] - yk[0], y31 = yk[3] - yk[0];
    double det = x21 * y31 - x31 * y21;
    if (det <= 0.0) return 26;
    double a = (x31 * x31 + y31 * y31) / det;
    double b = -(x31 * x21 + y31 * y21) / det;
    double c = (x21 * x21 + y21 * y21) / det;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            elmas[i][j] = (a * s1[i][j] + 3.0 * b * s2[i][j] + c * s3[i][j]) / 6.0;
            elmam[i][j] = det * s4[i][j] / 36.0;
        }
    return 0;
}

/* src/elem8.f90:18-205 (quadrilateral from 4 sub-triangles around the
 * diagonal intersection; centre node condensed; depends on k) */
static int elem8(const double *xk, const double *yk, double kwert, double kelmas[4][4]) {
    double xd[5], yd[5], elmas[5][5], elmam[5][5];
    memset(elmas, 0, sizeof elmas);
    memset(elmam, 0, sizeof elmam);
    double a1 = xk[2] - xk[0], a2 = xk[3] - xk[1];
    if (fabs(a1) <= 1e-12 || fabs(a2) <= 1e-12) return 26;
    a1 = (yk[2] - yk[0]) / a1;
    a2 = (yk[3] - yk[1]) / a2;
    if (fabs(a1 - a2) <= 1e-12) return 26;
    xd[4] = (a1 * xk[0] - yk[0] - a2 * xk[1] + yk[1]) / (a1 - a2);
    yd[4] = yk[0] + a1 * (xd[4] - xk[0]);
    for (int i = 0; i < 4; i++) { xd[i] = xk[i]; yd[i] = yk[i]; }
    static const int IK[4][3] = {{0, 1, 4}, {1, 2, 4}, {4, 2, 3}, {0, 4, 3}};
    for (int t = 0; t < 4; t++) {
        const int *ik = IK[t];
        double x21 = xd[ik[1]] - xd[ik[0]], x31 = xd[ik[2]] - xd[ik[0]];
        double y21 = yd[ik[1]] - yd[ik[0]], y31 = yd[ik[2]] - yd[ik[0]];
        double det = x21 * y31 - x31 * y21;
        if (det <= 1e-12) return 26;
        double a = (x31 * x31 + y31 * y31) / det;
        double b = -(x31 * x21 + y31 * y21) / det;
        double c = (x21 * x21 + y21 * y21) / det;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                elmas[ik[i]][ik[j]] += (a * S1T[i][j] + b * S2T[i][j] + c * S3T[i][j]) / 2.0;
                elmam[ik[i]][ik[j]] += det * S4T[i][j] / 24.0;
            }
    }
    for (int i = 0; i < 5; i++)
        for (int j = 0; j < 5; j++) elmas[i][j] = elmas[i][j] + kwert * kwert * elmam[i][j];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            kelmas[i][j] = elmas[i][j] - elmas[i][4] * elmas[4][j] / elmas[4][4];
    return 0;
}

/* src/beta.f90:38-135: mixed boundary factor for boundary line (xk, yk),
 * source electrode at (xs, ys), wavenumber kw */
static int beta_(const double *xk, const double *yk, double xs, double ys, double kw,
                 double sytop, double *out) {
    double xr = (xk[0] + xk[1]) / 2.0, yr = (yk[0] + yk[1]) / 2.0;
    double x3 = xr - xs;
    double y3m = (yr - sytop) - (ys - sytop);
    double y3p = (yr - sytop) + (ys - sytop);
    double r1m = sqrt(x3 * x3 + y3m * y3m), r1p = sqrt(x3 * x3 + y3p * y3p);
    double x4 = yk[0] - yk[1], y4 = xk[1] - xk[0];
    double r2 = sqrt(x4 * x4 + y4 * y4);
    if (r1m < 1e-12 || r1p < 1e-12 || r2 < 1e-12) { *out = 0.0; return 35; }
    double cthetm = (x3 * x4 + y3m * y4) / r1m / r2;
    double cthetp = (x3 * x4 + y3p * y4) / r1p / r2;
    double bk0m = or_bessk0(r1m * kw), bk0p = or_bessk0(r1p * kw);
    double bk1m = or_bessk1(r1m * kw), bk1p = or_bessk1(r1p * kw);
    double b;
    if (bk0m + bk0p == 0.0) b = (cthetm + cthetp) / 2.0;
    else b = (cthetm * bk1m + cthetp * bk1p) / (bk0m + bk0p);
    *out = kw * b;
    return 0;
}

static void element_coords(const or_mesh *m, int iel, int nkel, double *xk, double *yk) {
    for (int q = 1; q <= nkel; q++) {
        xk[q - 1] = SX(m, NREL(m, iel, q));
        yk[q - 1] = SY(m, NREL(m, iel, q));
    }
}

/* src/precal.f90:13-222 */
int or_precal(const or_mesh *m, int kwnanz, const double *kwn, double sytop,
              double *elbg, double *relbg, double *kg, int *lbeta_out, int *lrandb_out) {
    int elanz, relanz, maxnk;
    or_counts(m, &elanz, &relanz, &maxnk);
    int lbeta = 0, lrandb = 0, iel = 0;
    double xk[8], yk[8], elmas[4][4], elmam[4][4];
    for (int i = 0; i < m->typanz; i++) {
        int ntyp = m->typ[i], nkel = m->selanz[i];
        for (int j = 0; j < m->nelanz[i]; j++) {
            iel++;
            element_coords(m, iel, nkel, xk, yk);
            if (ntyp == 11) {
                if (lrandb) return 101;
                lbeta = 1;
                elem1(xk, yk, elmam);
                int rel = iel - elanz;
                if (rel <= 0) return 36;
                int imn = 0;
                for (int a = 0; a < nkel; a++)
                    for (int b = 0; b <= a; b++) {
                        imn++;
                        relbg[(imn - 1) * relanz + rel - 1] = elmam[a][b];
                    }
                for (int l = 1; l <= m->eanz; l++) {
                    int en = m->enr[l - 1];
                    double xs = SX(m, en), ys = SY(m, en);
                    for (int k = 0; k < kwnanz; k++) {
                        double bv;
                        int e = beta_(xk, yk, xs, ys, kwn[k], sytop, &bv);
                        if (e) return e;
                        kg[((size_t)k * m->eanz + (l - 1)) * relanz + rel - 1] = bv;
                    }
                }
            } else if (ntyp == 12) {
                continue;
            } else if (ntyp == 13) {
                if (lbeta) return 101;
                lrandb = 1;
                continue;
            } else if (ntyp == 8) {
                for (int k = 0; k < kwnanz; k++) {
                    double ke[4][4];
                    int e = elem8(xk, yk, kwn[k], ke);
                    if (e) return e;
                    int imn = 0;
                    for (int a = 0; a < nkel; a++)
                        for (int b = 0; b <= a; b++) {
                            imn++;
                            elbg[((size_t)k * 10 + imn - 1) * elanz + iel - 1] = ke[a][b];
                        }
                }
            } else {
                int e;
                if (ntyp == 3) e = elem3(xk, yk, elmas, elmam);
                else if (ntyp == 5) e = elem5(xk, yk, elmas, elmam);
                else return 18;
                if (e) return e;
                for (int k = 0; k < kwnanz; k++) {
                    int imn = 0;
                    for (int a = 0; a < nkel; a++)
                        for (int b = 0; b <= a; b++) {
                            imn++;
                            elbg[((size_t)k * 10 + imn - 1) * elanz + iel - 1] =
                                elmas[a][b] + elmam[a][b] * kwn[k] * kwn[k];
                        }
                }
            }
        }
    }
    *lbeta_out = lbeta;
    *lrandb_out = lrandb;
    return 0;
}

/* src/potana.f90:7-99 */
void or_potana(const or_mesh *m, int l, double kw, const double *sigma0, double *pota) {
    int idum = m->enr[l - 1];
    double xk1 = SX(m, idum), yk1 = SY(m, idum), potmax = 0.0;
    for (int j = 1; j <= m->sanz; j++) {
        if (j == idum) continue;
        double x21 = SX(m, j) - xk1, y21m = SY(m, j) - yk1, y21p = SY(m, j) + yk1;
        double rm = sqrt(x21 * x21 + y21m * y21m), rp = sqrt(x21 * x21 + y21p * y21p);
        double dum = or_bessk0(rm * kw) + or_bessk0(rp * kw);
        potmax = fmax(potmax, dum);
        pota[2 * (j - 1)] = dum;
        pota[2 * (j - 1) + 1] = 0.0;
    }
    pota[2 * (idum - 1)] = 5.0 * potmax;
    pota[2 * (idum - 1) + 1] = 0.0;
    cx dum2 = cdiv(cmk(0.5 / PI_, 0.0), cmk(sigma0[0], sigma0[1]));
    for (int j = 0; j < m->sanz; j++) CX(pota, j) = cmul(CX(pota, j), dum2);
}

/* ------------------------------------------------------------------ */
/* band system: assembly, Dirichlet rows, scaling, LL^T, solves         */
/* band storage: a[(i-1)*(mb+1) + (j - i + mb)] for j in [i-mb, i]      */
/* (1-based a(i*mb + j) of src/kompab.f90:108-110)                      */
/* ------------------------------------------------------------------ */
typedef struct {
    const or_mesh *m;
    int elanz, relanz, maxnk, kwnanz;
    const double *elbg, *relbg, *kg;
    const cx *sigma;
    cx sigma0;
    int lsr, lsink, nsink, lrandb;
    int rwdanz;
    const int *rwdnr;
    const cx *rwd;
    int ldc;
    cx *sigma_dc; /* owned: the real parts of sigma (DC) */
} fe_ctx;

/* src/kompab.f90:11-194 */
static int kompab(const fe_ctx *c, int nelec, int ki, cx *a, cx *b, const cx *pota) {
    const or_mesh *m = c->m;
    int mb = m->mb, sanz = m->sanz;
    memset(a, 0, sizeof(cx) * (size_t)(mb + 1) * sanz);
    memset(b, 0, sizeof(cx) * (size_t)sanz);
    int iel = 0;
    for (int i = 0; i < m->typanz; i++) {
        int ntyp = m->typ[i], nkel = m->selanz[i];
        for (int j = 0; j < m->nelanz[i]; j++) {
            iel++;
            int ikl = 0;
            if (ntyp > 11) continue;
            for (int k = 1; k <= nkel; k++) {
                int nzp = NREL(m, iel, k);
                for (int l = 1; l <= k; l++) {
                    int nnp = NREL(m, iel, l);
                    int idif = abs(nzp - nnp);
                    if (idif > mb) return 19;
                    ikl++;
                    int imax = nzp > nnp ? nzp : nnp, imin = nzp < nnp ? nzp : nnp;
                    size_t im = (size_t)imax * mb + imin; /* 1-based */
                    double dum;
                    cx dum2;
                    if (ntyp == 11) {
                        int rel = iel - c->elanz;
                        dum = c->relbg[(ikl - 1) * c->relanz + rel - 1] *
                              c->kg[((size_t)(ki - 1) * m->eanz + nelec - 1) * c->relanz + rel - 1];
                        dum2 = c->sigma[m->rnr[rel - 1] - 1];
                    } else {
                        dum = c->elbg[((size_t)(ki - 1) * 10 + ikl - 1) * c->elanz + iel - 1];
                        dum2 = c->sigma[iel - 1];
                    }
                    a[im - 1] = cadd(a[im - 1], cmul(cmk(dum, 0.0), dum2));
                    if (c->lsr) {
                        cx d2 = cmul(cmk(dum, 0.0), csub(dum2, c->sigma0));
                        b[nzp - 1] = cadd(b[nzp - 1], cmul(d2, pota[nnp - 1]));
                        if (nnp != nzp) b[nnp - 1] = cadd(b[nnp - 1], cmul(d2, pota[nzp - 1]));
                    }
                }
            }
        }
    }
    if (!c->lsr) b[m->enr[nelec - 1] - 1] = cmk(-1.0, 0.0);
    if (c->lsink) b[c->nsink - 1] = cmk(1.0, 0.0);
    return 0;
}

/* src/kompb.f90:1-69 */
static void kompb(const fe_ctx *c, int nelec, cx *b, const double *fak) {
    const or_mesh *m = c->m;
    memset(b, 0, sizeof(cx) * (size_t)m->sanz);
    int e = m->enr[nelec - 1];
    b[e - 1] = cmk(-fak[e - 1], 0.0);
    if (c->lsink) b[c->nsink - 1] = cmk(fak[c->nsink - 1], 0.0);
}

/* src/randb.f90:1-84 (homogeneous Dirichlet nodes of element type 13) */
static void randb(const or_mesh *m, cx *a, cx *b) {
    int mb = m->mb, sanz = m->sanz, m1 = mb + 1, iel = 0;
    for (int i2 = 0; i2 < m->typanz; i2++) {
        int ntyp = m->typ[i2], nkel = m->selanz[i2];
        for (int j2 = 0; j2 < m->nelanz[i2]; j2++) {
            iel++;
            if (ntyp != 13) continue;
            for (int ir = 1; ir <= nkel; ir++) {
                int k = NREL(m, iel, ir);
                b[k - 1] = cmk(0, 0);
                long idk = (long)k * m1;
                a[idk - 1] = cmk(1, 0);
                if (k != 1) {
                    int ia = 1 > mb + 2 - k ? 1 : mb + 2 - k;
                    for (int i = ia; i <= mb; i++) a[idk + i - m1 - 1] = cmk(0, 0);
                }
                if (k == sanz) continue;
                int ia = 1 > k - sanz + m1 ? 1 : k - sanz + m1;
                for (int i = ia; i <= mb; i++) {
                    int j = k - i + m1;
                    long ji = (long)(j - 1) * m1 + i;
                    a[ji - 1] = cmk(0, 0);
                }
            }
        }
    }
}

/* src/randb2.f90:1-82: node rwdnr(ir) held at the value rwd(ir).  Its row
 * and column are eliminated (diagonal 1, b(k) = -rwd), the eliminated column
 * moved to the right-hand side of the other rows, node by node in file order
 * (a column already eliminated contributes nothing). */
static void randb2(const fe_ctx *c, cx *a, cx *b) {
    const or_mesh *m = c->m;
    int mb = m->mb, sanz = m->sanz, m1 = mb + 1;
    for (int ir = 0; ir < c->rwdanz; ir++) {
        int k = c->rwdnr[ir];
        cx rwert = c->rwd[ir];
        b[k - 1] = cmk(-rwert.re, -rwert.im);
        long idk = (long)k * m1;
        a[idk - 1] = cmk(1, 0);
        if (k != 1) {
            int ia = 1 > mb + 2 - k ? 1 : mb + 2 - k;
            for (int i = ia; i <= mb; i++) {
                int j = k + i - m1;
                long ki = idk + i - m1;
                b[j - 1] = cadd(b[j - 1], cmul(rwert, a[ki - 1]));
                a[ki - 1] = cmk(0, 0);
            }
        }
        if (k == sanz) continue;
        int ia = 1 > k - sanz + m1 ? 1 : k - sanz + m1;
        for (int i = ia; i <= mb; i++) {
            int j = k - i + m1;
            long ji = (long)(j - 1) * m1 + i;
            b[j - 1] = cadd(b[j - 1], cmul(rwert, a[ji - 1]));
            a[ji - 1] = cmk(0, 0);
        }
    }
}

/* src/scalab.f90:14-87 */
static int scalab(int sanz, int mb, cx *a, cx *b, double *fak) {
    for (int i = 1; i <= sanz; i++) {
        long idi = (long)i * (mb + 1);
        double dum = cabs_(a[idi - 1]);
        if (dum <= 0.0) return 27;
        a[idi - 1] = cdiv(a[idi - 1], cmk(dum, 0.0));
        fak[i - 1] = 1.0 / sqrt(dum);
        b[i - 1] = cmul(b[i - 1], cmk(fak[i - 1], 0.0));
        if (i == 1) continue;
        long i0 = (long)i * mb;
        int ja = 1 > i - mb ? 1 : i - mb;
        for (int j = ja; j <= i - 1; j++)
            a[i0 + j - 1] = cmul(a[i0 + j - 1], cmk(fak[i - 1] * fak[j - 1], 0.0));
    }
    return 0;
}

/* src/chol.f90:7-88: in-place complex-symmetric L L^T (no conjugation) */
/* ldc: src/choldc.f90:66-70 stops on a pivot <= 0 (the complex routine only
 * on 0); with real data every other step is the same arithmetic */
static int chol(int sanz, int mb, cx *a, int ldc) {
    int m1 = mb + 1;
    for (int i = 1; i <= sanz; i++) {
        long idi = (long)i * m1;
        int fi = 1 > i - mb ? 1 : i - mb;
        long i0 = idi - i;
        for (int j = fi; j <= i; j++) {
            long ij = i0 + j, j0 = (long)j * mb;
            cx s = a[ij - 1];
            for (int k = fi; k <= j - 1; k++) s = csub(s, cmul(a[i0 + k - 1], a[j0 + k - 1]));
            if (j < i) {
                a[ij - 1] = cdiv(s, a[(long)j * m1 - 1]);
            } else {
                if (cabs_(s) <= 0.0 || (ldc && !(s.re > 0.0))) return 28;
                a[idi - 1] = csqrt_(s);
            }
        }
    }
    return 0;
}

/* src/vre.f90:5-71: pot = -(L L^T)^{-1} b */
static void vre(int sanz, int mb, const cx *a, const cx *b, cx *pot) {
    int m1 = mb + 1;
    long idi = 0;
    for (int i = 1; i <= sanz; i++) {
        idi = (long)i * m1;
        cx s = b[i - 1];
        long i0 = idi - i;
        int jlow = 1 > i - mb ? 1 : i - mb;
        for (int j = jlow; j <= i - 1; j++) s = csub(s, cmul(a[i0 + j - 1], pot[j - 1]));
        pot[i - 1] = cdiv(s, a[idi - 1]);
    }
    for (int i = sanz; i >= 1; i--) {
        pot[i - 1] = cdiv(cmk(-pot[i - 1].re, -pot[i - 1].im), a[idi - 1]);
        int jlow = 1 > i - mb ? 1 : i - mb;
        long i0 = idi - i;
        for (int j = jlow; j <= i - 1; j++) pot[j - 1] = cadd(pot[j - 1], cmul(a[i0 + j - 1], pot[i - 1]));
        idi -= m1;
    }
}

static int setup_ctx(const or_mesh *m, const or_opts *o, int kwnanz, const double *kwn,
                     const double *sigma, fe_ctx *c, double **elbg, double **relbg, double **kg,
                     int *lbeta, int *lsr_eff) {
    or_counts(m, &c->elanz, &c->relanz, &c->maxnk);
    c->m = m;
    c->sigma_dc = NULL;
    c->kwnanz = kwnanz;
    *elbg = (double *)calloc((size_t)c->elanz * 10 * kwnanz + 1, sizeof(double));
    *relbg = (double *)calloc((size_t)c->relanz * 10 + 1, sizeof(double));
    *kg = (double *)calloc((size_t)c->relanz * m->eanz * kwnanz + 1, sizeof(double));
    double sytop = o->lsytop ? or_bsytop(m) : 0.0;
    int lrandb = 0;
    int e = or_precal(m, kwnanz, kwn, sytop, *elbg, *relbg, *kg, lbeta, &lrandb);
    if (e) return e;
    c->elbg = *elbg; c->relbg = *relbg; c->kg = *kg;
    c->sigma = (const cx *)sigma;
    double s0[2];
    or_refsig(m, sigma, s0);
    c->sigma0 = cmk(s0[0], s0[1]);
    int lsr = o->swrtr == 0 ? 0 : o->lsr;  /* lana is decided by the callers */
    if (!*lbeta) lsr = 0; /* src/fem.f90:311 */
    c->lsr = lsr;
    c->lsink = o->lsink;
    c->nsink = o->nsink;
    c->lrandb = lrandb;
    c->rwdanz = o->rwdanz;
    c->rwdnr = o->rwdnr;
    c->rwd = (const cx *)o->rwd;
    c->ldc = o->ldc;
    c->sigma_dc = NULL;
    if (o->ldc) { /* src/kompadc.f90:114-119: DBLE(sigma) */
        c->sigma_dc = (cx *)malloc(sizeof(cx) * (size_t)c->elanz + 1);
        for (int i = 0; i < c->elanz; i++) c->sigma_dc[i] = cmk(((const cx *)sigma)[i].re, 0.0);
        c->sigma = c->sigma_dc;
    }
    for (int ir = 0; ir < c->rwdanz; ir++)  /* src/rrandb.f90 (error 30) */
        if (c->rwdnr[ir] < 1 || c->rwdnr[ir] > m->sanz) return 30;
    *lsr_eff = lsr;
    return 0;
}

/* One wavenumber, all (or a subset of) electrodes: the body of the !$OMP DO
 * loop of src/fem.f90:327-397.  lmask (optional) selects electrodes. */
static int forward_k(const fe_ctx *c, int lbeta, int lana, int k, const double *kwn,
                     const char *lmask, double *kpot) {
    const or_mesh *m = c->m;
    int sanz = m->sanz, mb = m->mb, err = 0;
    cx *a = (cx *)malloc(sizeof(cx) * (size_t)(mb + 1) * sanz);
    cx *b = (cx *)malloc(sizeof(cx) * (size_t)sanz);
    cx *pot = (cx *)malloc(sizeof(cx) * (size_t)sanz);
    cx *pota = (cx *)calloc((size_t)sanz, sizeof(cx));
    double *fak = (double *)malloc(sizeof(double) * (size_t)sanz);
    int have_factor = 0;
    for (int l = 1; l <= m->eanz; l++) {
        int need = lmask ? lmask[l - 1] : 1;
        int refactor = (lbeta || l == 1 || c->lsr) && !lana;
        if (!need && !(refactor && !lbeta && !c->lsr && l == 1)) continue;
        if (c->lsr || lana) {
            double s0[2] = {c->sigma0.re, c->sigma0.im};
            or_potana(m, l, kwn[k - 1], s0, (double *)pota);
        }
        if (refactor) {
            int e = kompab(c, l, k, a, b, pota);
            if (!e && c->lrandb) randb(m, a, b);
            if (!e && c->rwdanz) randb2(c, a, b);
            if (!e) e = scalab(sanz, mb, a, b, fak);
            if (!e) e = chol(sanz, mb, a, c->ldc);
            if (e) { err = e; break; }
            have_factor = 1;
        } else if (!lana) {
            if (!have_factor) { err = 28; break; }
            kompb(c, l, b, fak);
        }
        if (!lana) vre(sanz, mb, a, b, pot);
        if (!need) continue;
        cx *kp = ((cx *)kpot) + ((size_t)(k - 1) * m->eanz + (l - 1)) * sanz;
        for (int j = 0; j < sanz; j++) {
            if (lana) {
                kp[j] = pota[j];
            } else {
                kp[j] = cmul(pot[j], cmk(fak[j], 0.0));
                if (c->lsr) kp[j] = cadd(kp[j], pota[j]);
            }
        }
    }
    free(a); free(b); free(pot); free(pota); free(fak);
    return err;
}

int or_forward(const or_mesh *m, const or_opts *o, int kwnanz, const double *kwn,
               const double *kwnwi, const double *sigma, double *kpot) {
    (void)kwnwi;
    fe_ctx c;
    double *elbg, *relbg, *kg;
    int lbeta, lsr;
    int e = setup_ctx(m, o, kwnanz, kwn, sigma, &c, &elbg, &relbg, &kg, &lbeta, &lsr);
    int lana = (o->swrtr != 0 && o->lana && !lsr) ? 1 : 0;
    if (!e) {
        int err = 0;
#ifdef _OPENMP
        if (o->nthreads > 0) omp_set_num_threads(o->nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
        for (int k = 1; k <= kwnanz; k++) {
            int ek = forward_k(&c, lbeta, lana, k, kwn, NULL, kpot);
            if (ek) {
#ifdef _OPENMP
#pragma omp critical
#endif
                err = ek;
            }
        }
        e = err;
    }
    free(elbg); free(relbg); free(kg); free(c.sigma_dc);
    return e;
}

int or_forward_pairs(const or_mesh *m, const or_opts *o, int kwnanz, const double *kwn,
                     const double *kwnwi, const double *sigma, int npairs, const int *pairs,
                     double *kpot) {
    (void)kwnwi;
    fe_ctx c;
    double *elbg, *relbg, *kg;
    int lbeta, lsr;
    int e = setup_ctx(m, o, kwnanz, kwn, sigma, &c, &elbg, &relbg, &kg, &lbeta, &lsr);
    int lana = (o->swrtr != 0 && o->lana && !lsr) ? 1 : 0;
    if (!e) {
        int err = 0;
#ifdef _OPENMP
        if (o->nthreads > 0) omp_set_num_threads(o->nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
        for (int p = 0; p < npairs; p++) {
            int k = pairs[2 * p], l = pairs[2 * p + 1];
            char *mask = (char *)calloc((size_t)m->eanz, 1);
            mask[l - 1] = 1;
            int ek = forward_k(&c, lbeta, lana, k, kwn, mask, kpot);
            free(mask);
            if (ek) {
#ifdef _OPENMP
#pragma omp critical
#endif
                err = ek;
            }
        }
        e = err;
    }
    free(elbg); free(relbg); free(kg); free(c.sigma_dc);
    return e;
}

/* src/rtrafo.f90:13-92 (complex branch); 2D: hpot = kpot(:, :, 1) */
void or_rtrafo(const or_mesh *m, int swrtr, int kwnanz, const double *kwnwi,
               const double *kpot, double *hpot) {
    int sanz = m->sanz, eanz = m->eanz;
    const cx *kp = (const cx *)kpot;
    cx *hp = (cx *)hpot;
    for (int l = 0; l < eanz; l++)
        for (int j = 0; j < sanz; j++) {
            if (swrtr == 0) { hp[(size_t)l * sanz + j] = kp[(size_t)l * sanz + j]; continue; }
            cx s = cmk(0, 0);
            for (int k = 0; k < kwnanz; k++)
                s = cadd(s, cscale(kp[((size_t)k * eanz + l) * sanz + j], kwnwi[k]));
            hp[(size_t)l * sanz + j] = cmk(s.re / PI_, s.im / PI_);
        }
}

/* src/bkfak.f90:7-149 */
int or_bkfak(const or_mesh *m, double *kfak) {
    double xk[4] = {0, 0, 0, 0}, yk[4] = {0, 0, 0, 0};
    for (int i = 0; i < m->nanz; i++) {
        int e[4];
        decode(m->strnr[i], &e[0], &e[1]);
        decode(m->vnr[i], &e[2], &e[3]);
        for (int q = 0; q < 4; q++)
            if (e[q] > 0) { xk[q] = SX(m, m->enr[e[q] - 1]); yk[q] = SY(m, m->enr[e[q] - 1]); }
        double r[4];
        /* r4: (3,1)  r3: (3,2)  r2: (4,1)  r1: (4,2) */
        static const int P[4][2] = {{3, 1}, {3, 0}, {2, 1}, {2, 0}}; /* r1..r4 */
        for (int q = 0; q < 4; q++) {
            int pa = P[q][0], pb = P[q][1];
            if (e[pa] > 0 && e[pb] > 0) {
                double dx = xk[pa] - xk[pb], dym = yk[pa] - yk[pb], dyp = yk[pa] + yk[pb];
                dym = 1.0 / sqrt(dx * dx + dym * dym);
                dyp = 1.0 / sqrt(dx * dx + dyp * dyp);
                r[q] = dym + dyp;
            } else {
                r[q] = 0.0;
            }
        }
        double dum = (r[0] - r[1]) - (r[2] - r[3]);
        if (fabs(dum) == 0.0) return 93;
        kfak[i] = 4.0 * PI_ / dum;
    }
    return 0;
}

/* src/bvolt.f90:7-89 (mode 0) and src/bvolti.f90:8-100 (mode 1) */
int or_bvolt(const or_mesh *m, int mode, const double *hpot, const double *kfak,
             double *volt, double *sigmaa) {
    int sanz = m->sanz;
    const cx *hp = (const cx *)hpot;
    for (int i = 0; i < m->nanz; i++) {
        int e1, e2, e3, e4;
        decode(m->strnr[i], &e1, &e2);
        decode(m->vnr[i], &e3, &e4);
#define HP(node_e, src_e) hp[(size_t)((src_e) - 1) * sanz + (m->enr[(node_e) - 1] - 1)]
        cx d1 = (e4 > 0 && e2 > 0) ? HP(e4, e2) : cmk(0, 0);
        cx d2 = (e4 > 0 && e1 > 0) ? HP(e4, e1) : cmk(0, 0);
        cx d3 = (e3 > 0 && e2 > 0) ? HP(e3, e2) : cmk(0, 0);
        cx d4 = (e3 > 0 && e1 > 0) ? HP(e3, e1) : cmk(0, 0);
#undef HP
        cx v = csub(csub(d1, d2), csub(d3, d4));
        if (mode == 2) v.im = 0.0; /* DC: dcmplx of the real voltage, src/bvolti.f90:56-62 */
        CX(volt, i) = v;
        if (mode == 0) {
            CX(sigmaa, i) = cmul(cmk(kfak ? kfak[i] : 1.0, 0.0), v);
        } else {
            if (cabs_(v) == 0.0) return 82;
            cx lv = clog_(v);
            CX(sigmaa, i) = cmk(-lv.re, -lv.im);
        }
    }
    return 0;
}

/* src/bsens.f90:23-197 (mode 0, CRMod) and src/bsensi.f90:23-194 (mode 1,
 * CRTomo), with the element matrices elbg supplied (see or_elbg). */
void or_bsens_elbg(const or_mesh *m, const or_opts *o, int mode, int swrtr, int kwnanz,
                   const double *kwnwi, const double *elbg, const double *kpot,
                   const double *sigma, const double *volt, double *sens) {
    int elanz, relanz, maxnk;
    or_counts(m, &elanz, &relanz, &maxnk);
    int sanz = m->sanz, eanz = m->eanz, nanz = m->nanz;
    const cx *kp = (const cx *)kpot;
    cx *sn = (cx *)sens;
    memset(sens, 0, sizeof(cx) * (size_t)nanz * elanz);
#ifdef _OPENMP
    if (o && o->nthreads > 0) omp_set_num_threads(o->nthreads);
#pragma omp parallel for schedule(guided, 256)
#endif
    for (int i = 0; i < nanz; i++) {
        cx hsens[32];
        int e1, e2, e3, e4;
        decode(m->strnr[i], &e1, &e2);
        decode(m->vnr[i], &e3, &e4);
        cx sup[4] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
        int iel = 0;
        for (int ityp = 0; ityp < m->typanz; ityp++) {
            int ntyp = m->typ[ityp], nkel = m->selanz[ityp];
            if (ntyp > 10) continue;
            for (int jn = 0; jn < m->nelanz[ityp]; jn++) {
                iel++;
                for (int k = 0; k < kwnanz; k++) {
                    hsens[k] = cmk(0, 0);
                    for (int mi = 1; mi <= nkel; mi++) {
                        int nzp = NREL(m, iel, mi);
                        for (int mj = 1; mj <= nkel; mj++) {
                            int nnp = NREL(m, iel, mj);
                            int imax = mi > mj ? mi : mj, imin = mi < mj ? mi : mj;
                            int imn = imax * (imax - 1) / 2 + imin;
                            size_t base = (size_t)k * eanz;
                            if (e1 > 0) sup[0] = kp[(base + e1 - 1) * sanz + nnp - 1];
                            if (e2 > 0) sup[1] = kp[(base + e2 - 1) * sanz + nnp - 1];
                            if (e3 > 0) sup[2] = kp[(base + e3 - 1) * sanz + nzp - 1];
                            if (e4 > 0) sup[3] = kp[(base + e4 - 1) * sanz + nzp - 1];
                            cx dum = cmul(csub(sup[1], sup[0]), csub(sup[3], sup[2]));
                            double eb = elbg[((size_t)k * 10 + imn - 1) * elanz + iel - 1];
                            hsens[k] = cadd(hsens[k], cmul(cmk(eb, 0.0), dum));
                        }
                    }
                }
                cx dum;
                double strom = m->strom ? m->strom[i] : 1.0;
                if (mode == 0) {
                    if (swrtr == 0) {
                        dum = cmul(hsens[0], cmk(strom, 0.0));
                    } else {
                        dum = cmk(0, 0);
                        for (int k = 0; k < kwnanz; k++) dum = cadd(dum, cscale(hsens[k], kwnwi[k]));
                        dum = cmul(dum, cmk(strom / PI_, 0.0));
                    }
                    size_t idx = (size_t)(iel - 1) * nanz + i;
                    sn[idx] = csub(sn[idx], dum);
                } else {
                    if (swrtr == 0) {
                        dum = hsens[0];
                    } else {
                        dum = cmk(0, 0);
                        for (int k = 0; k < kwnanz; k++) dum = cadd(dum, cscale(hsens[k], kwnwi[k]));
                        dum = cmk(dum.re / PI_, dum.im / PI_);
                    }
                    size_t idx = (size_t)(iel - 1) * nanz + i;
                    sn[idx] = cadd(sn[idx], cdiv(cmul(dum, CX(sigma, iel - 1)), CX(volt, i)));
                }
            }
        }
    }
}

/* precal element matrices only (for or_bsens_elbg) */
int or_elbg(const or_mesh *m, int kwnanz, const double *kwn, double sytop, double *elbg) {
    int elanz, relanz, maxnk;
    or_counts(m, &elanz, &relanz, &maxnk);
    double *relbg = (double *)calloc((size_t)relanz * 10 + 1, sizeof(double));
    double *kg = (double *)calloc((size_t)relanz * m->eanz * kwnanz + 1, sizeof(double));
    int lbeta, lrandb;
    int e = or_precal(m, kwnanz, kwn, sytop, elbg, relbg, kg, &lbeta, &lrandb);
    free(relbg); free(kg);
    return e;
}

/* precal outputs for external comparison */
int or_precal_all(const or_mesh *m, int kwnanz, const double *kwn, double sytop,
                  double *elbg, double *relbg, double *kg, int *flags) {
    return or_precal(m, kwnanz, kwn, sytop, elbg, relbg, kg, &flags[0], &flags[1]);
}

/* ------------------------------------------------------------------ */
/* Cuthill-McKee renumbering: cutmckee/cutmck.f:125-337                 */
/* ------------------------------------------------------------------ */
int or_cutmck(int sanz, int typanz, const int *typ, const int *nelanz, const int *selanz,
              int *nrel, int ld_nrel, int *snr, int eanz, int *enr) {
    enum { GRMAX = 500, SPMAX = 100 };
    int elanz = 0;
    for (int i = 0; i < typanz; i++)
        if (typ[i] <= 10) elanz += nelanz[i];
    int *graph = (int *)calloc((size_t)GRMAX * sanz, sizeof(int));
    int *grad = (int *)calloc((size_t)sanz, sizeof(int));
    int *perm = (int *)calloc((size_t)sanz, sizeof(int));
    int *neu = (int *)calloc((size_t)sanz + 1, sizeof(int));
    int *neuin = (int *)calloc((size_t)sanz, sizeof(int));
    int *level = (int *)calloc((size_t)sanz + 2, sizeof(int));
    int *start = (int *)calloc((size_t)sanz + 1, sizeof(int));
    char *num = (char *)calloc((size_t)sanz, 1);
    int ret = 0;
#define G(k, node) graph[(size_t)((node) - 1) * GRMAX + (k) - 1]
    int idum = 0;
    for (int l = 0; l < typanz; l++) {
        for (int mm = 1; mm <= nelanz[l]; mm++) {
            for (int i = 1; i <= selanz[l] - 1; i++) {
                int nzp = nrel[(i - 1) * ld_nrel + idum + mm - 1];
                for (int j = i + 1; j <= selanz[l]; j++) {
                    int nnp = nrel[(j - 1) * ld_nrel + idum + mm - 1];
                    int dup = 0;
                    for (int k = 1; k <= GRMAX; k++) {
                        if (G(k, nzp) == nnp) { dup = 1; break; }
                        if (G(k, nzp) > 0) continue;
                        G(k, nzp) = nnp;
                        grad[nzp - 1]++;
                        break;
                    }
                    if (dup) continue;
                    grad[nnp - 1]++;
                    if (grad[nnp - 1] <= GRMAX) G(grad[nnp - 1], nnp) = nzp;
                }
            }
        }
        idum += nelanz[l];
    }
    int mingd = grad[0], maxgd = grad[0];
    for (int i = 0; i < sanz; i++) {
        if (grad[i] < mingd) mingd = grad[i];
        if (grad[i] > maxgd) maxgd = grad[i];
    }
    if (mingd == 0 || maxgd > GRMAX) { ret = -5; goto done; }
    int spanz = elanz / 10;
    if (spanz < 1000) spanz = 1000;
    if (spanz > SPMAX) spanz = SPMAX;
    int k = 0;
    for (;;) {
        int stop = 0;
        for (int i = 1; i <= sanz; i++) {
            if (grad[i - 1] == mingd) {
                k++;
                start[k] = i;
                if (k >= spanz) { stop = 1; break; }
            }
        }
        if (stop) break;
        if (mingd > elanz / 10) break;
        mingd++;
    }
    spanz = k - 1;
    if (spanz < 1) { ret = -5; goto done; }
    int mmin = sanz, kbdm = 0;
    for (int is = 1; is <= spanz; is++) {
        int nstart = start[is];
        neu[1] = nstart;
        neuin[nstart - 1] = 1;
        memset(num, 0, (size_t)sanz);
        num[nstart - 1] = 1;
        level[1] = 1;
        int levs = 1, leve = 1, nlev = 1, l = 1;
        for (;;) {
            for (int j = levs; j <= leve; j++) {
                int nzp = neu[j], gradzp = grad[nzp - 1];
                for (;;) {
                    int mingr = GRMAX, kk = 0;
                    for (int i = 1; i <= gradzp; i++) {
                        int nnp = G(i, nzp);
                        if (num[nnp - 1] || grad[nnp - 1] > mingr) continue;
                        mingr = grad[nnp - 1];
                        kk = nnp;
                    }
                    if (kk == 0) break;
                    l++;
                    neu[l] = kk;
                    neuin[kk - 1] = l;
                    num[kk - 1] = 1;
                }
            }
            levs = levs + level[nlev];
            nlev++;
            level[nlev] = l - levs + 1;
            leve = leve + level[nlev];
            if (level[nlev] == 0 && leve < sanz) { ret = -5; goto done; } /* disconnected */
            if (!(leve < sanz)) break;
        }
        int mbw = 0;
        for (int i = 1; i <= sanz; i++) {
            int nzp = neuin[i - 1];
            for (int j = 1; j <= grad[i - 1]; j++) {
                int kk = neuin[G(j, i) - 1];
                int d = abs(kk - nzp);
                if (d > mbw) mbw = d;
            }
        }
        if (mbw < mmin) {
            mmin = mbw;
            kbdm = is;
            memcpy(perm, neuin, sizeof(int) * (size_t)sanz);
        }
    }
    (void)kbdm;
    idum = 0;
    for (int i = 0; i < typanz; i++) {
        for (int j = 1; j <= nelanz[i]; j++)
            for (int kk = 1; kk <= selanz[i]; kk++) {
                int *p = &nrel[(kk - 1) * ld_nrel + idum + j - 1];
                *p = perm[*p - 1];
            }
        idum += nelanz[i];
    }
    for (int i = 0; i < sanz; i++) grad[i] = snr[i];
    for (int i = 0; i < sanz; i++) snr[perm[i] - 1] = grad[i];
    for (int i = 0; i < eanz; i++) enr[i] = perm[enr[i] - 1];
    ret = mmin;
#undef G
done:
    free(graph); free(grad); free(perm); free(neu); free(neuin); free(level); free(start); free(num);
    return ret;
}

/* ------------------------------------------------------------------ */
/* regularisation and the model update                                  */
/* ------------------------------------------------------------------ */

/* src/bnachbar.f90:7-93 */
void or_bnachbar(const or_mesh *m, int *nachbar) {
    int elanz, relanz, maxnk;
    or_counts(m, &elanz, &relanz, &maxnk);
    memset(nachbar, 0, sizeof(int) * (size_t)elanz * (maxnk + 1));
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = 1; i <= elanz; i++) {
        for (int ik = 1; ik <= maxnk; ik++) {
            int ik1 = NREL(m, i, ik), ik2 = NREL(m, i, ik % maxnk + 1);
            for (int j = 1; j <= elanz; j++) {
                if (j == i) continue;
                for (int jk = 1; jk <= maxnk; jk++) {
                    int jk1 = NREL(m, j, jk), jk2 = NREL(m, j, jk % maxnk + 1);
                    if ((ik1 == jk1 && ik2 == jk2) || (ik1 == jk2 && ik2 == jk1)) {
                        nachbar[(size_t)(ik - 1) * elanz + i - 1] = j;
                        nachbar[(size_t)maxnk * elanz + i - 1] += 1;
                    }
                }
            }
        }
    }
}

/* src/bsmatm_mod.f90:190-362 (no discontinuities: ndis_x = ndis_z = 0) */
void or_bsmatmreg(const or_mesh *m, int nx, int nz, double alfx, double alfz, double *smatm) {
    int manz = nx * nz;
    memset(smatm, 0, sizeof(double) * (size_t)manz * 3);
#define KK(i, j) (((i) - 1) * nx + (j))
#define SM(r, c) smatm[(size_t)((c) - 1) * manz + (r) - 1]
    for (int i = 1; i <= nz; i++) {
        for (int j = 1; j <= nx; j++) {
            int e = KK(i, j);
            double dzleft = fabs(SY(m, NREL(m, e, 4)) - SY(m, NREL(m, e, 1)));
            double dzright = fabs(SY(m, NREL(m, e, 3)) - SY(m, NREL(m, e, 2)));
            double xmean = 0.0;
            for (int l = 1; l <= 4; l++) xmean += SX(m, NREL(m, e, l));
            xmean /= 4.0;
            if (j > 1) {
                double xleft = 0.0;
                for (int l = 1; l <= 4; l++) xleft += SX(m, NREL(m, KK(i, j - 1), l));
                xleft /= 4.0;
                SM(e, 1) = 1.0 * alfx * dzleft / fabs(xmean - xleft);
            }
            if (j < nx) {
                double xright = 0.0;
                for (int l = 1; l <= 4; l++) xright += SX(m, NREL(m, KK(i, j + 1), l));
                xright /= 4.0;
                double dum = 1.0 * alfx * dzright / fabs(xright - xmean);
                SM(e, 1) += dum;
                SM(e, 2) = -dum;
            }
            double dxup = fabs(SX(m, NREL(m, e, 3)) - SX(m, NREL(m, e, 4)));
            double dxdown = fabs(SX(m, NREL(m, e, 2)) - SX(m, NREL(m, e, 1)));
            double zmean = 0.0;
            for (int l = 1; l <= 4; l++) zmean += SY(m, NREL(m, e, l));
            zmean /= 4.0;
            if (i > 1) {
                double zup = 0.0;
                for (int l = 1; l <= 4; l++) zup += SY(m, NREL(m, KK(i - 1, j), l));
                zup /= 4.0;
                SM(e, 1) += 1.0 * alfz * dxup / fabs(zup - zmean);
            }
            if (i < nz) {
                double zdown = 0.0;
                for (int l = 1; l <= 4; l++) zdown += SY(m, NREL(m, KK(i + 1, j), l));
                zdown /= 4.0;
                double dum = 1.0 * alfz * dxdown / fabs(zmean - zdown);
                SM(e, 1) += dum;
                SM(e, 3) = -dum;
            }
        }
    }
#undef KK
#undef SM
}

/* src/bsmatm_mod.f90:364-460 (no decouplings) */
void or_bsmatmtri(const or_mesh *m, const int *nachbar, double alfx, double alfz, double *smatm) {
    int elanz, relanz, maxnk;
    or_counts(m, &elanz, &relanz, &maxnk);
    memset(smatm, 0, sizeof(double) * (size_t)elanz * (maxnk + 1));
    /* element centroids as in src/relem.f90:107-118 */
    double *espx = (double *)calloc((size_t)elanz, sizeof(double));
    double *espy = (double *)calloc((size_t)elanz, sizeof(double));
    int iel = 0, ifln = 0;
    for (int i = 0; i < m->typanz; i++)
        for (int j = 0; j < m->nelanz[i]; j++) {
            iel++;
            if (m->typ[i] < 10) {
                for (int k = 1; k <= m->selanz[i]; k++) {
                    espx[ifln] += SX(m, NREL(m, iel, k));
                    espy[ifln] += SY(m, NREL(m, iel, k));
                }
                espx[ifln] /= m->selanz[i];
                espy[ifln] /= m->selanz[i];
                ifln++;
            }
        }
    for (int i = 1; i <= elanz; i++) {
        double sp1x = espx[i - 1], sp1y = espy[i - 1];
        for (int k = 1; k <= maxnk; k++) {
            int nxt = k % maxnk + 1;
            double dx = SX(m, NREL(m, i, k)) - SX(m, NREL(m, i, nxt));
            double dy = SY(m, NREL(m, i, k)) - SY(m, NREL(m, i, nxt));
            double edglen = sqrt(dx * dx + dy * dy);
            int nb = nachbar[(size_t)(k - 1) * elanz + i - 1];
            if (nb > 0) {
                double sp2x = espx[nb - 1], sp2y = espy[nb - 1];
                double ddx = sp1x - sp2x, ddy = sp1y - sp2y;
                double dist = sqrt(ddx * ddx + ddy * ddy);
                double ang = atan2(ddy, ddx);
                double ca = alfx * cos(ang), sa = alfz * sin(ang);
                double alfgeo = sqrt(ca * ca + sa * sa);
                double rs = edglen / dist * alfgeo;
                smatm[(size_t)(k - 1) * elanz + i - 1] = -rs;
                smatm[(size_t)maxnk * elanz + i - 1] += rs;
            }
        }
    }
    free(espx); free(espy);
}

/* R * v for ltri = 0 (src/update.f90:63-91 stencil) with optional column
 * weights w (cgfac) applied to v (src/cg_mod.f90:547-577) */
static void rmul_reg(int manz, int nx, const double *smatm, const cx *v, const double *w, cx *out) {
#define SM(r, c) smatm[(size_t)((c) - 1) * manz + (r) - 1]
    for (int i = 1; i <= manz; i++) {
        cx cdum = cmk(0, 0);
        if (w) {
            if (i > 1) cdum = cmul(v[i - 2], cmk(SM(i - 1, 2) * w[i - 2], 0.0));
            if (i < manz) cdum = cadd(cdum, cmul(v[i], cmk(SM(i, 2) * w[i], 0.0)));
            if (i > nx) cdum = cadd(cdum, cmul(v[i - nx - 1], cmk(SM(i - nx, 3) * w[i - nx - 1], 0.0)));
            if (i < manz - nx + 1) cdum = cadd(cdum, cmul(v[i + nx - 1], cmk(SM(i, 3) * w[i + nx - 1], 0.0)));
            out[i - 1] = cadd(cdum, cmul(v[i - 1], cmk(SM(i, 1) * w[i - 1], 0.0)));
        } else {
            if (i > 1) cdum = cmul(cmk(SM(i - 1, 2), 0.0), v[i - 2]);
            if (i < manz) cdum = cadd(cdum, cmul(cmk(SM(i, 2), 0.0), v[i]));
            if (i > nx) cdum = cadd(cdum, cmul(cmk(SM(i - nx, 3), 0.0), v[i - nx - 1]));
            if (i < manz - nx + 1) cdum = cadd(cdum, cmul(cmk(SM(i, 3), 0.0), v[i + nx - 1]));
            out[i - 1] = cadd(cdum, cmul(cmk(SM(i, 1), 0.0), v[i - 1]));
        }
    }
#undef SM
}

/* R * v for ltri = 1, 2 (src/update.f90:99-120, src/cg_mod.f90:579-613) */
static void rmul_tri(int manz, int maxnk, const int *nachbar, const double *smatm, const cx *v,
                     const double *w, cx *out) {
    for (int i = 1; i <= manz; i++) {
        cx cdum = cmk(0, 0);
        for (int j = 1; j <= maxnk; j++) {
            int id = nachbar[(size_t)(j - 1) * manz + i - 1];
            if (id == 0) continue;
            double sm = smatm[(size_t)(j - 1) * manz + i - 1];
            if (w) cdum = cadd(cdum, cscale(cmul(v[id - 1], cmk(sm, 0.0)), w[id - 1]));
            else cdum = cadd(cdum, cmul(cmk(sm, 0.0), v[id - 1]));
        }
        double sd = smatm[(size_t)maxnk * manz + i - 1];
        if (w) out[i - 1] = cadd(cdum, cscale(cmul(v[i - 1], cmk(sd, 0.0)), w[i - 1]));
        else out[i - 1] = cadd(cdum, cmul(cmk(sd, 0.0), v[i - 1]));
    }
}

/* src/update.f90 with lfpi or ldc and cjggdc (src/cg_mod.f90:136-260, bapdc,
 * bpdc, bpdctri, bbdc): Re(J) in the preconditioner, the right-hand side and
 * the products; the real CG runs on Im(bvec) (part 1, lfpi: the update goes
 * into the phases) or Re(bvec) (part 2, ldc: the update is real). */
static int update_real(int part, int nanz, int manz, const cx *sens, const double *wmatd, const int *wdfak,
                       const cx *dat, const cx *sigmaa, int ltri, const double *smatm, int nx,
                       const int *nachbar, int maxnk, double lam, double eps, int ncgmax, double step,
                       cx *par, cx *dpar, double *cgfac, float *cgres) {
    cx *bvec = (cx *)calloc((size_t)manz, sizeof(cx));
    cx *tmp = (cx *)calloc((size_t)manz, sizeof(cx));
    double *bdc = (double *)calloc((size_t)manz, sizeof(double));
    double *rdc = (double *)calloc((size_t)manz, sizeof(double));
    double *pdc = (double *)calloc((size_t)manz, sizeof(double));
    double *dp = (double *)calloc((size_t)manz, sizeof(double));
    double *apdc = (double *)calloc((size_t)nanz, sizeof(double));
#define RS(i, j) sens[(size_t)(j) * nanz + (i)].re
    if (ltri == 0) rmul_reg(manz, nx, smatm, par, NULL, bvec);
    else rmul_tri(manz, maxnk, nachbar, smatm, par, NULL, bvec);
    for (int j = 0; j < manz; j++) {
        double dum = 0.0;
        for (int i = 0; i < nanz; i++) dum += RS(i, j) * RS(i, j) * wmatd[i] * (double)wdfak[i];
        dum += lam * (ltri == 0 ? smatm[j] : smatm[(size_t)maxnk * manz + j]);
        cgfac[j] = 1.0 / sqrt(dum);
    }
    for (int j = 0; j < manz; j++) {
        cx cdum = cmk(0, 0);
        for (int i = 0; i < nanz; i++)
            cdum = cadd(cdum, cmul(cmk(RS(i, j) * wmatd[i] * (double)wdfak[i], 0.0), csub(dat[i], sigmaa[i])));
        bvec[j] = cmul(csub(cdum, cmul(cmk(lam, 0.0), bvec[j])), cmk(cgfac[j], 0.0));
        bdc[j] = part == 1 ? bvec[j].im : bvec[j].re; /* src/cg_mod.f90:160-164 */
        rdc[j] = bdc[j];
    }
    double dr = 0, dr0 = 0, dr1 = 0, beta = 0, alpha;
    int ncg = ncgmax, k;
    for (k = 1; k <= ncgmax; k++) {
        ncg = k - 1;
        dr = 0.0;
        for (int j = 0; j < manz; j++) dr += rdc[j] * rdc[j];
        if (k == 1) {
            dr0 = dr * eps;
            beta = 0.0;
        } else {
            beta = dr / dr1;
        }
        if (dr <= dr0) break;
        for (int j = 0; j < manz; j++) pdc[j] = rdc[j] + beta * pdc[j];
        for (int i = 0; i < nanz; i++) {
            double a = 0.0;
            for (int j = 0; j < manz; j++) a += pdc[j] * RS(i, j) * cgfac[j];
            apdc[i] = a;
        }
        for (int j = 0; j < manz; j++) tmp[j] = cmk(pdc[j], 0.0);
        if (ltri == 0) rmul_reg(manz, nx, smatm, tmp, cgfac, bvec);
        else rmul_tri(manz, maxnk, nachbar, smatm, tmp, cgfac, bvec);
        for (int j = 0; j < manz; j++) {
            double dum = 0.0;
            for (int i = 0; i < nanz; i++) dum += RS(i, j) * wmatd[i] * (double)wdfak[i] * apdc[i];
            bdc[j] = (dum + lam * bvec[j].re) * cgfac[j];
        }
        dr1 = 0.0;
        for (int j = 0; j < manz; j++) dr1 += pdc[j] * bdc[j];
        alpha = dr / dr1;
        for (int j = 0; j < manz; j++) {
            dp[j] += alpha * pdc[j];
            rdc[j] -= alpha * bdc[j];
        }
        dr1 = dr;
        cgres[k] = (float)(eps * dr / dr0);
    }
    if (k > ncgmax) ncg = ncgmax;
    cgres[0] = (float)ncg;
    for (int j = 0; j < manz; j++) {
        dpar[j] = part == 1 ? cmk(0.0, dp[j] * cgfac[j]) : cmk(dp[j] * cgfac[j], 0.0);
        par[j] = cadd(par[j], cmul(cmk(step, 0.0), dpar[j]));
    }
#undef RS
    free(bvec); free(tmp); free(bdc); free(rdc); free(pdc); free(dp); free(apdc);
    return ncg;
}

int or_update_fpi(int nanz, int manz, const double *sens, const double *wmatd, const int *wdfak,
                  const double *dat, const double *sigmaa, int ltri, const double *smatm, int nx,
                  const int *nachbar, int maxnk, double lam, double eps, int ncgmax, double step,
                  double *par, double *dpar, double *cgfac, float *cgres) {
    return update_real(1, nanz, manz, (const cx *)sens, wmatd, wdfak, (const cx *)dat, (const cx *)sigmaa, ltri,
                       smatm, nx, nachbar, maxnk, lam, eps, ncgmax, step, (cx *)par, (cx *)dpar, cgfac, cgres);
}

/* DC inversion (ldc: src/update.f90 with sensdc, cjggdc on Re(bvec)); the
 * real Jacobian is Re(sens) */
int or_update_dc(int nanz, int manz, const double *sens, const double *wmatd, const int *wdfak,
                 const double *dat, const double *sigmaa, int ltri, const double *smatm, int nx,
                 const int *nachbar, int maxnk, double lam, double eps, int ncgmax, double step,
                 double *par, double *dpar, double *cgfac, float *cgres) {
    return update_real(2, nanz, manz, (const cx *)sens, wmatd, wdfak, (const cx *)dat, (const cx *)sigmaa, ltri,
                       smatm, nx, nachbar, maxnk, lam, eps, ncgmax, step, (cx *)par, (cx *)dpar, cgfac, cgres);
}

int or_update(int nanz, int manz, const double *sens_, const double *wmatd, const int *wdfak,
              const double *dat_, const double *sigmaa_, int ltri, const double *smatm, int nx,
              const int *nachbar, int maxnk, double lam, double eps, int ncgmax, double step,
              double *par_, double *dpar_, double *cgfac, float *cgres) {
    const cx *sens = (const cx *)sens_, *dat = (const cx *)dat_, *sigmaa = (const cx *)sigmaa_;
    cx *par = (cx *)par_, *dpar = (cx *)dpar_;
    cx *bvec = (cx *)calloc((size_t)manz, sizeof(cx));
    cx *rvec = (cx *)calloc((size_t)manz, sizeof(cx));
    cx *pvec = (cx *)calloc((size_t)manz, sizeof(cx));
    cx *ap = (cx *)calloc((size_t)nanz, sizeof(cx));
#define SENS(i, j) sens[(size_t)(j) * nanz + (i)]
    /* b = R m */
    if (ltri == 0) rmul_reg(manz, nx, smatm, par, NULL, bvec);
    else rmul_tri(manz, maxnk, nachbar, smatm, par, NULL, bvec);
    /* preconditioner */
    for (int j = 0; j < manz; j++) {
        double dum = 0.0;
        for (int i = 0; i < nanz; i++) {
            cx s = SENS(i, j);
            dum += cmul(cconj(s), s).re * wmatd[i] * (double)wdfak[i];
        }
        if (ltri == 0) dum += lam * smatm[j];
        else dum += lam * smatm[(size_t)maxnk * manz + j];
        cgfac[j] = 1.0 / sqrt(dum);
    }
    /* right-hand side */
    for (int j = 0; j < manz; j++) {
        cx cdum = cmk(0, 0);
        for (int i = 0; i < nanz; i++)
            cdum = cadd(cdum, cmul(cmul(cconj(SENS(i, j)), cmk(wmatd[i] * (double)wdfak[i], 0.0)),
                                   csub(dat[i], sigmaa[i])));
        bvec[j] = csub(cdum, cmul(cmk(lam, 0.0), bvec[j]));
        bvec[j] = cmul(bvec[j], cmk(cgfac[j], 0.0));
    }
    /* src/cg_mod.f90:426-518 cjggra */
    for (int j = 0; j < manz; j++) { dpar[j] = cmk(0, 0); rvec[j] = bvec[j]; pvec[j] = cmk(0, 0); }
    double dr = 0, dr0 = 0, dr1 = 0, beta = 0, alpha;
    int ncg = ncgmax, k;
    for (k = 1; k <= ncgmax; k++) {
        ncg = k - 1;
        dr = 0.0;
        for (int j = 0; j < manz; j++) dr += cmul(cconj(rvec[j]), rvec[j]).re;
        if (k == 1) {
            dr0 = dr * eps;
            beta = 0.0;
        } else {
            if (dr <= dr0) break;
            beta = dr / dr1;
        }
        for (int j = 0; j < manz; j++) pvec[j] = cadd(rvec[j], cmul(cmk(beta, 0.0), pvec[j]));
        /* bap */
        for (int i = 0; i < nanz; i++) {
            cx s = cmk(0, 0);
            for (int j = 0; j < manz; j++) s = cadd(s, cmul(cmul(pvec[j], SENS(i, j)), cmk(cgfac[j], 0.0)));
            ap[i] = s;
        }
        /* bp / bptri */
        if (ltri == 0) rmul_reg(manz, nx, smatm, pvec, cgfac, bvec);
        else rmul_tri(manz, maxnk, nachbar, smatm, pvec, cgfac, bvec);
        /* bb */
        for (int j = 0; j < manz; j++) {
            cx cdum = cmk(0, 0);
            for (int i = 0; i < nanz; i++)
                cdum = cadd(cdum, cmul(cmul(cconj(SENS(i, j)), cmk(wmatd[i] * (double)wdfak[i], 0.0)), ap[i]));
            bvec[j] = cadd(cdum, cmul(cmk(lam, 0.0), bvec[j]));
            bvec[j] = cmul(bvec[j], cmk(cgfac[j], 0.0));
        }
        dr1 = 0.0;
        for (int j = 0; j < manz; j++) dr1 += cmul(cconj(pvec[j]), bvec[j]).re;
        alpha = dr / dr1;
        for (int j = 0; j < manz; j++) {
            dpar[j] = cadd(dpar[j], cmul(cmk(alpha, 0.0), pvec[j]));
            rvec[j] = csub(rvec[j], cmul(cmk(alpha, 0.0), bvec[j]));
        }
        dr1 = dr;
        cgres[k] = (float)(eps * dr / dr0);
    }
    if (k > ncgmax) ncg = ncgmax;
    cgres[0] = (float)ncg;
    for (int j = 0; j < manz; j++) dpar[j] = cmul(dpar[j], cmk(cgfac[j], 0.0));
    for (int j = 0; j < manz; j++) par[j] = cadd(par[j], cmul(cmk(step, 0.0), dpar[j]));
#undef SENS
    free(bvec); free(rvec); free(pvec); free(ap);
    return ncg;
}

/* One system (k, l) (1-based): src/kompab.f90 + src/randb.f90 +
 * src/randb2.f90 + src/scalab.f90 + src/chol.f90, leaving the band factor a((mb+1)*sanz) and
 * fak(sanz).  Returns errnr. */
int or_factor(const or_mesh *m, const or_opts *o, int kwnanz, const double *kwn, const double *sigma,
              int k, int l, double *a_out, double *fak_out) {
    fe_ctx c;
    double *elbg, *relbg, *kg;
    int lbeta, lsr;
    int e = setup_ctx(m, o, kwnanz, kwn, sigma, &c, &elbg, &relbg, &kg, &lbeta, &lsr);
    if (!e) {
        int sanz = m->sanz, mb = m->mb;
        cx *b = (cx *)calloc((size_t)sanz, sizeof(cx));
        cx *pota = (cx *)calloc((size_t)sanz, sizeof(cx));
        e = kompab(&c, l, k, (cx *)a_out, b, pota);
        if (!e && c.lrandb) randb(m, (cx *)a_out, b);
        if (!e && c.rwdanz) randb2(&c, (cx *)a_out, b);
        if (!e) e = scalab(sanz, mb, (cx *)a_out, b, fak_out);
        if (!e) e = chol(sanz, mb, (cx *)a_out, c.ldc);
        free(b);
        free(pota);
    }
    free(elbg); free(relbg); free(kg); free(c.sigma_dc);
    return e;
}

/* src/bmcm_mod.f90 buncert on a host Jacobian (column-major (nanz, manz)):
 * bata (ata = Re(J^H W J)), bata_reg (ltri 1, 2: column by column, the
 * diagonal, then the first nachbar(j, nk+1) slots, mirrored; ltri 0: the
 * 5-point stencil of src/update.f90), bmcm (Cholesky inverse), bres
 * (diag(cov ata)) and bmcm2 (diag(cov ata cov)).  Returns 108 when ata_reg
 * is not positive definite. */
int or_mcm(int nanz, int manz, const double *sens_, const double *wmatd, const int *wdfak, int ltri,
           const double *smatm, int nx, const int *nachbar, int maxnk, double lam, double *d_ata,
           double *d_reg, double *d_cov1, double *d_res, double *d_cov2) {
    const cx *sens = (const cx *)sens_;
    size_t n = (size_t)manz;
    double *ata = (double *)calloc(n * n, sizeof(double));
    double *reg = (double *)calloc(n * n, sizeof(double));
    double *L = (double *)calloc(n * n, sizeof(double));
    double *cov = (double *)calloc(n * n, sizeof(double));
#define M(a, i, j) a[(size_t)(j) * n + (i)]
    for (int k = 0; k < manz; k++)
        for (int j = k; j < manz; j++) {
            double s = 0.0;
            for (int i = 0; i < nanz; i++) {
                cx a = sens[(size_t)k * nanz + i], b = sens[(size_t)j * nanz + i];
                s += (a.re * b.re + a.im * b.im) * wmatd[i] * (double)wdfak[i];
            }
            M(ata, k, j) = s;
            M(ata, j, k) = s;
        }
    for (int k = 0; k < manz; k++) d_ata[k] = M(ata, k, k);
    memcpy(reg, ata, sizeof(double) * n * n);
    if (ltri == 0) {
        for (int i = 0; i < manz; i++) {
            M(reg, i, i) += lam * smatm[i];
            if (i + 1 < manz) {
                M(reg, i, i + 1) += lam * smatm[n + i];
                M(reg, i + 1, i) += lam * smatm[n + i];
            }
            if (i + nx < manz) {
                M(reg, i, i + nx) += lam * smatm[2 * n + i];
                M(reg, i + nx, i) += lam * smatm[2 * n + i];
            }
        }
    } else {
        for (int j = 0; j < manz; j++) {
            M(reg, j, j) = M(ata, j, j) + lam * smatm[(size_t)maxnk * n + j];
            int cnt = nachbar[(size_t)maxnk * n + j];
            for (int k = 0; k < cnt && k < maxnk; k++) {
                int ik = nachbar[(size_t)k * n + j];
                if (ik == 0) continue;
                double v = M(ata, ik - 1, j) + lam * smatm[(size_t)k * n + j];
                M(reg, ik - 1, j) = v;
                M(reg, j, ik - 1) = v;
            }
        }
    }
    for (int k = 0; k < manz; k++) d_reg[k] = M(reg, k, k);
    int err = 0;
    /* Cholesky reg = L L^T */
    for (int j = 0; j < manz && !err; j++) {
        double s = M(reg, j, j);
        for (int k = 0; k < j; k++) s -= M(L, j, k) * M(L, j, k);
        if (!(s > 0.0)) { err = 108; break; }
        double d = sqrt(s);
        M(L, j, j) = d;
        for (int i = j + 1; i < manz; i++) {
            double t = M(reg, i, j);
            for (int k = 0; k < j; k++) t -= M(L, i, k) * M(L, j, k);
            M(L, i, j) = t / d;
        }
    }
    if (!err) {
        /* cov = L^-T L^-1: columns of L^-1 by forward substitution */
        double *Li = (double *)calloc(n * n, sizeof(double));
        for (int c = 0; c < manz; c++)
            for (int i = c; i < manz; i++) {
                double t = (i == c) ? 1.0 : 0.0;
                for (int k = c; k < i; k++) t -= M(L, i, k) * M(Li, k, c);
                M(Li, i, c) = t / M(L, i, i);
            }
        for (int i = 0; i < manz; i++)
            for (int j = 0; j <= i; j++) {
                double t = 0.0;
                for (int k = i; k < manz; k++) t += M(Li, k, i) * M(Li, k, j);
                M(cov, i, j) = t;
                M(cov, j, i) = t;
            }
        free(Li);
        for (int k = 0; k < manz; k++) d_cov1[k] = M(cov, k, k);
        if (d_res || d_cov2) {
            /* res = cov ata (src/bmcm_mod.f90 bres), cov2 = res cov (bmcm2) */
            double *res = (double *)calloc(n * n, sizeof(double));
            for (int j = 0; j < manz; j++)
                for (int k = 0; k < manz; k++) {
                    double a = M(ata, k, j);
                    if (a == 0.0) continue;
                    for (int i = 0; i < manz; i++) M(res, i, j) += M(cov, i, k) * a;
                }
            if (d_res)
                for (int k = 0; k < manz; k++) d_res[k] = M(res, k, k);
            if (d_cov2)
                for (int i = 0; i < manz; i++) {
                    double t = 0.0;
                    for (int k = 0; k < manz; k++) t += M(res, i, k) * M(cov, k, i);
                    d_cov2[i] = t;
                }
            free(res);
        }
    }
#undef M
    free(ata); free(reg); free(L); free(cov);
    return err;
}
