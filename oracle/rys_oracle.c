/*
 * rys_oracle.c -- CPU ORACLE (test infrastructure only).
 *
 * This file is the checker for the GPU Fock builder.  Only tests/, the smoke
 * check in __graft_entry__.py and the cpu_baseline / reference legs of bench.py
 * may load it.  Nothing in the product path (segfault_py_gb300/) links or calls
 * it.
 *
 * It restates, in plain C, the integral engine of lyuhang428/SegFault_py:
 *   - module rys   src/hf/core/core.f90:203-1004   (binom, recur, shift, ix,
 *                                                   eri_3d_rys, eri_rys)
 *   - module mmd   src/hf/core/core.f90:5-200      (boys, hermite_gauss_e,
 *                                                   coulomb_auxiliary_r,
 *                                                   eri_3d, eri)
 *   - one-electron src/hf/mmd.py:13-141 / src/hf/mmd2.py:14-84
 *   - the ERI build of src/hf/hf.py:33-61 (unique quartets i>=j, k>=l,
 *     ij>=kl, 8-fold scatter) and a direct J/K digestion of the same
 *     quartets (the maths of hf.py:300 without the dense tensor).
 *
 * Two things the reference takes from elsewhere are written here from the
 * mathematics:
 *   - Rys roots/weights.  The reference evaluates fixed 5-point fits
 *     (root5, core.f90:232-812).  Here the n-point rule for the weight
 *     exp(-x t^2) on t in [0,1] (variable u = t^2) is computed from first
 *     principles: the measure is discretised by Gauss-Legendre in t, the
 *     Stieltjes procedure gives the three-term recurrence, the nodes come
 *     from Sturm-sequence bisection on the Jacobi matrix plus Newton polish,
 *     and the weights from the Christoffel formula.  Like root5, the routine
 *     returns u = t^2 (core.f90:810-811).  A cheap table (piecewise
 *     polynomials fitted to the exact rule) is used for speed; the exact rule
 *     checks it.  A function pointer lets a transcription of the reference's
 *     own root5 (built from the reference source into oracle/_ref/) replace it.
 *   - Boys function F_m(x) (core.f90:23-28 calls GSL 1F1; utils.py:107-109
 *     calls scipy hyp1f1): power series e^{-x} sum (2x)^i/((2m+1)...(2m+2i+1))
 *     for small x, erf + upward recursion for large x.
 *
 * Build: gcc -O2 -fopenmp -shared -fPIC (no -ffast-math), matching the -O2 of
 * the reference's f2py line (core.f90:1).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846264338
#define ORC_MAXK 16

typedef struct {
    int K;              /* number of primitives                           */
    int shell[3];       /* lx, ly, lz                                     */
    double center[3];   /* bohr                                           */
    double expns[ORC_MAXK];
    double coefs[ORC_MAXK];   /* contraction coefficients (renormalised) */
    double nf[ORC_MAXK];      /* primitive normalisation factors          */
} orc_cgf;

/* ------------------------------------------------------------------------ */
/* Boys function                                                            */
/* ------------------------------------------------------------------------ */
double orc_boys(int m, double x)
{
    if (x < 0.0) return NAN;
    if (x < 1e-300) return 1.0 / (2.0 * m + 1.0);
    if (x < 45.0) {
        long double term = 1.0L / (2.0L * m + 1.0L);
        long double sum = term;
        for (int i = 1; i < 2000; ++i) {
            term *= 2.0L * x / (2.0L * m + 2.0L * i + 1.0L);
            sum += term;
            if (term < 1e-21L * sum) break;
        }
        return (double)(expl(-(long double)x) * sum);
    }
    double f = 0.5 * sqrt(ORC_PI / x) * erf(sqrt(x));
    double ex = exp(-x);
    for (int k = 0; k < m; ++k) f = ((2.0 * k + 1.0) * f - ex) / (2.0 * x);
    return f;
}

/* ------------------------------------------------------------------------ */
/* Rys quadrature, exact (discretised Stieltjes)                            */
/* ------------------------------------------------------------------------ */
#define ORC_GL 192
static double gl_x[ORC_GL], gl_w[ORC_GL];
static int gl_ready = 0;

static void gl_init(void)
{
    /* Gauss-Legendre nodes on [-1,1]: Newton on P_M from the asymptotic guess */
    int M = ORC_GL;
    for (int i = 0; i < (M + 1) / 2; ++i) {
        double z = cos(ORC_PI * (i + 0.75) / (M + 0.5)), pp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = 0.0;
            for (int k = 1; k <= M; ++k) {
                double p2 = p1; p1 = p0;
                p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
            }
            pp = M * (z * p0 - p1) / (z * z - 1.0);
            double dz = p0 / pp;
            z -= dz;
            if (fabs(dz) < 1e-16) break;
        }
        gl_x[i] = -z; gl_x[M - 1 - i] = z;
        gl_w[i] = gl_w[M - 1 - i] = 2.0 / ((1.0 - z * z) * pp * pp);
    }
    gl_ready = 1;
}

/* count eigenvalues of the symmetric tridiagonal (a, b2 = offdiag^2) below lam */
static int sturm_count(int n, const double *a, const double *b2, double lam)
{
    int c = 0;
    double d = a[0] - lam;
    if (d < 0) ++c;
    for (int i = 1; i < n; ++i) {
        if (d == 0.0) d = 1e-300;
        d = a[i] - lam - b2[i] / d;
        if (d < 0) ++c;
    }
    return c;
}

/* n-point Rys rule at x: u[i] = t_i^2 ascending, w[i] weights (n <= 8) */
void orc_rys_roots_exact(int n, double x, double *u, double *w)
{
    if (!gl_ready) gl_init();
    double T = (x <= 100.0) ? 1.0 : 10.0 / sqrt(x);
    double uu[ORC_GL], om[ORC_GL], p0[ORC_GL], p1[ORC_GL];
    for (int k = 0; k < ORC_GL; ++k) {
        double t = 0.5 * T * (gl_x[k] + 1.0);
        uu[k] = t * t;
        om[k] = 0.5 * T * gl_w[k] * exp(-x * t * t);
        p0[k] = 1.0; p1[k] = 0.0;
    }
    double alpha[8], beta[8], hprev = 1.0;
    for (int j = 0; j < n; ++j) {
        double h = 0.0, hu = 0.0;
        for (int k = 0; k < ORC_GL; ++k) { double q = om[k] * p0[k] * p0[k]; h += q; hu += q * uu[k]; }
        alpha[j] = hu / h;
        beta[j] = (j == 0) ? h : h / hprev;
        hprev = h;
        for (int k = 0; k < ORC_GL; ++k) {
            double pn = (uu[k] - alpha[j]) * p0[k] - (j > 0 ? beta[j] : 0.0) * p1[k];
            p1[k] = p0[k]; p0[k] = pn;
        }
    }
    /* nodes: bisection with Sturm counts, then Newton on p_n via recurrence */
    for (int i = 0; i < n; ++i) {
        double lo = 0.0, hi = 1.0;
        for (int it = 0; it < 200; ++it) {
            double mid = 0.5 * (lo + hi);
            if (mid <= lo || mid >= hi) break;
            if (sturm_count(n, alpha, beta, mid) > i) hi = mid; else lo = mid;
        }
        double z = 0.5 * (lo + hi);
        for (int it = 0; it < 3; ++it) {
            double q0 = 1.0, q1 = 0.0, d0 = 0.0, d1 = 0.0;
            for (int j = 0; j < n; ++j) {
                double qn = (z - alpha[j]) * q0 - (j > 0 ? beta[j] : 0.0) * q1;
                double dn = q0 + (z - alpha[j]) * d0 - (j > 0 ? beta[j] : 0.0) * d1;
                q1 = q0; q0 = qn; d1 = d0; d0 = dn;
            }
            if (d0 == 0.0) break;
            double dz = q0 / d0;
            if (fabs(dz) > 1e-10 * (fabs(z) + 1e-300)) break; /* bisection already exact */
            z -= dz;
        }
        u[i] = z;
        /* Christoffel: 1/w = sum_j p_j(z)^2 / h_j, h_j = beta_0 ... beta_j */
        double s = 0.0, q0 = 1.0, q1 = 0.0, hj = 1.0;
        for (int j = 0; j < n; ++j) {
            hj *= beta[j];
            s += q0 * q0 / hj;
            double qn = (z - alpha[j]) * q0 - (j > 0 ? beta[j] : 0.0) * q1;
            q1 = q0; q0 = qn;
        }
        w[i] = 1.0 / s;
    }
}

/* ------------------------------------------------------------------------ */
/* Fast 5-point table for the oracle's own speed (fit to the exact rule)     */
/* ------------------------------------------------------------------------ */
#define OTAB_H 1.0
#define OTAB_NINT 64
#define OTAB_DEG 11
#define OTAB_XMAX (OTAB_H * OTAB_NINT)
static double otab[OTAB_NINT][10][OTAB_DEG + 1];
static double oasym_r[5], oasym_w[5];
static int otab_ready = 0;

static void cheb_to_mono(const double *c, int D, double *m)
{
    /* T_k as monomials, built by T_{k+1} = 2 s T_k - T_{k-1} */
    double Tkm1[32] = {0}, Tk[32] = {0}, Tkp1[32];
    Tkm1[0] = 1.0;              /* T_0 */
    Tk[1] = 1.0;                /* T_1 */
    for (int i = 0; i <= D; ++i) m[i] = 0.0;
    m[0] += c[0];
    if (D >= 1) m[1] += c[1];
    for (int k = 1; k < D; ++k) {
        for (int i = 0; i <= D; ++i) Tkp1[i] = -Tkm1[i] + (i > 0 ? 2.0 * Tk[i - 1] : 0.0);
        for (int i = 0; i <= D; ++i) m[i] += c[k + 1] * Tkp1[i];
        memcpy(Tkm1, Tk, sizeof Tk); memcpy(Tk, Tkp1, sizeof Tk);
    }
}

static void otab_init(void)
{
    const int D = OTAB_DEG;
    for (int j = 0; j < OTAB_NINT; ++j) {
        double vals[OTAB_DEG + 1][10], sk[OTAB_DEG + 1];
        for (int k = 0; k <= D; ++k) {
            sk[k] = cos(ORC_PI * (k + 0.5) / (D + 1));
            double x = (j + 0.5 * (sk[k] + 1.0)) * OTAB_H;
            orc_rys_roots_exact(5, x, vals[k], vals[k] + 5);
        }
        for (int f = 0; f < 10; ++f) {
            double c[OTAB_DEG + 1];
            for (int i = 0; i <= D; ++i) {
                double s = 0.0;
                for (int k = 0; k <= D; ++k) s += vals[k][f] * cos(i * acos(sk[k]));
                c[i] = s * 2.0 / (D + 1) * (i == 0 ? 0.5 : 1.0);
            }
            cheb_to_mono(c, D, otab[j][f]);
        }
    }
    /* x -> infinity: u_i = r_i / x, w_i = W_i / sqrt(x) (half-range Hermite) */
    double u[5], w[5], X = 1e6;
    orc_rys_roots_exact(5, X, u, w);
    for (int i = 0; i < 5; ++i) { oasym_r[i] = u[i] * X; oasym_w[i] = w[i] * sqrt(X); }
    otab_ready = 1;
}

static void orc_root5_table(double x, double *rw)
{
    if (x >= OTAB_XMAX) {
        double isx = 1.0 / sqrt(x);
        for (int i = 0; i < 5; ++i) { rw[i] = oasym_r[i] / x; rw[5 + i] = oasym_w[i] * isx; }
        return;
    }
    int j = (int)(x / OTAB_H);
    double s = 2.0 * (x / OTAB_H - j) - 1.0;
    for (int f = 0; f < 10; ++f) {
        const double *c = otab[j][f];
        double v = c[OTAB_DEG];
        for (int i = OTAB_DEG - 1; i >= 0; --i) v = v * s + c[i];
        rw[f] = v;
    }
}

static void orc_root5_exact(double x, double *rw) { orc_rys_roots_exact(5, x, rw, rw + 5); }

typedef void (*orc_root5_fn)(const double *x, double *rw);
static orc_root5_fn ext_root5 = 0;
static int root_mode = 0;   /* 0 table, 1 exact, 2 external (reference root5) */

void orc_set_root_mode(int mode, orc_root5_fn fn)
{
    if (mode == 2 && !fn) mode = 0;
    root_mode = mode;
    ext_root5 = fn;
}

void orc_init(void)
{
    if (!gl_ready) gl_init();
    if (!otab_ready) otab_init();
}

/* 5 roots (u = t^2) followed by 5 weights, like root5's res(10) */
void orc_root5(double x, double *rw)
{
    if (root_mode == 2 && ext_root5) { ext_root5(&x, rw); return; }
    if (root_mode == 1) { orc_root5_exact(x, rw); return; }
    orc_root5_table(x, rw);
}

/* ------------------------------------------------------------------------ */
/* module rys (core.f90:203-1004)                                            */
/* ------------------------------------------------------------------------ */
static const double orc_fact[13] = {1, 1, 2, 6, 24, 120, 720, 5040, 40320,
                                    362880, 3628800, 39916800, 479001600};
int orc_error = 0;

/* core.f90:222-229 (ERROR STOP when n < k becomes an error flag + NaN) */
double orc_binom(int n, int k)
{
    if (n < k || k < 0 || n > 12) { orc_error = 1; return NAN; }
    return orc_fact[n] / orc_fact[k] / orc_fact[n - k];
}

/* core.f90:815-874; G is row-major (li+lj+1) x (lk+ll+1) */
void orc_recur(int li, int lj, int lk, int ll, double xi, double xj, double xk,
               double xl, double alpha, double beta, double gamma, double delta,
               double t, double *G)
{
    double a_ = alpha + beta, b_ = gamma + delta;
    double xa = (alpha * xi + beta * xj) / (alpha + beta);
    double xb = (gamma * xk + delta * xl) / (gamma + delta);
    double ix0 = ORC_PI / sqrt(a_ * b_) *
                 exp(-alpha * beta / (alpha + beta) * (xi - xj) * (xi - xj) -
                     gamma * delta / (gamma + delta) * (xk - xl) * (xk - xl));
    double b00 = 0.5 / (a_ + b_) * t;
    double b10 = 0.5 / a_ - 0.5 * b_ / a_ / (a_ + b_) * t;
    double b10p = 0.5 / b_ - 0.5 * a_ / b_ / (a_ + b_) * t;
    double c00 = (xa - xi) + b_ / (a_ + b_) * (xb - xa) * t;
    double c00p = (xb - xk) + a_ / (a_ + b_) * (xa - xb) * t;
    int ni = li + lj, nk = lk + ll, W = nk + 1;
#define GG(i, k) G[(i) * W + (k)]
    for (int i = 0; i <= ni; ++i)
        for (int k = 0; k <= nk; ++k) GG(i, k) = 0.0;
    GG(0, 0) = ix0;
    if (ni > 0) GG(1, 0) = c00 * GG(0, 0);
    if (nk > 0) GG(0, 1) = c00p * GG(0, 0);
    for (int i = 1; i <= ni - 1; ++i) GG(i + 1, 0) = i * b10 * GG(i - 1, 0) + c00 * GG(i, 0);
    for (int k = 1; k <= nk - 1; ++k) GG(0, k + 1) = k * b10p * GG(0, k - 1) + c00p * GG(0, k);
    if (ni == 0 || nk == 0) return;
    for (int a = 1; a <= ni; ++a) {
        GG(a, 1) = a * b00 * GG(a - 1, 0) + c00p * GG(a, 0);
        for (int b = 2; b <= nk; ++b)
            GG(a, b) = b10p * (b - 1) * GG(a, b - 2) + a * b00 * GG(a - 1, b - 1) + c00p * GG(a, b - 1);
    }
#undef GG
}

/* core.f90:877-899 */
double orc_shift(const double *G, int li, int lj, int lk, int ll, double xij, double xkl)
{
    int W = lk + ll + 1;
    double res = 0.0;
    for (int m = 0; m <= ll; ++m) {
        double tmp = 0.0;
        for (int n = 0; n <= lj; ++n)
            tmp += orc_binom(lj, n) * pow(xij, lj - n) * G[(n + li) * W + (m + lk)];
        res += orc_binom(ll, m) * pow(xkl, ll - m) * tmp;
    }
    return res;
}

/* core.f90:902-914 */
double orc_ix(int l1, int l2, int l3, int l4, double x1, double x2, double x3,
              double x4, double alpha, double beta, double gamma, double delta, double t)
{
    double G[13 * 13];
    orc_recur(l1, l2, l3, l4, x1, x2, x3, x4, alpha, beta, gamma, delta, t, G);
    return orc_shift(G, l1, l2, l3, l4, x1 - x2, x3 - x4);
}

/* core.f90:917-964 (always 5 roots, like the reference) */
double orc_eri_3d_rys(const int *s1, const int *s2, const int *s3, const int *s4,
                      const double *c1, const double *c2, const double *c3,
                      const double *c4, double alpha, double beta, double gamma,
                      double delta)
{
    double a_ = alpha + beta, b_ = gamma + delta;
    double rho = a_ * b_ / (a_ + b_);
    double P[3], Q[3], rpq2 = 0.0;
    for (int d = 0; d < 3; ++d) {
        P[d] = (alpha * c1[d] + beta * c2[d]) / (alpha + beta);
        Q[d] = (gamma * c3[d] + delta * c4[d]) / (gamma + delta);
        rpq2 += (P[d] - Q[d]) * (P[d] - Q[d]);
    }
    double rw[10];
    orc_root5(rpq2 * rho, rw);
    double res = 0.0;
    for (int r = 0; r < 5; ++r) {
        double ix = orc_ix(s1[0], s2[0], s3[0], s4[0], c1[0], c2[0], c3[0], c4[0], alpha, beta, gamma, delta, rw[r]);
        double iy = orc_ix(s1[1], s2[1], s3[1], s4[1], c1[1], c2[1], c3[1], c4[1], alpha, beta, gamma, delta, rw[r]);
        double iz = orc_ix(s1[2], s2[2], s3[2], s4[2], c1[2], c2[2], c3[2], c4[2], alpha, beta, gamma, delta, rw[r]);
        res += ix * iy * iz * rw[5 + r];
    }
    return res * 2.0 * sqrt(rho / ORC_PI);
}

/* core.f90:967-1002 */
double orc_eri_rys(const orc_cgf *f1, const orc_cgf *f2, const orc_cgf *f3, const orc_cgf *f4)
{
    double res = 0.0;
    for (int i1 = 0; i1 < f1->K; ++i1)
        for (int i2 = 0; i2 < f2->K; ++i2)
            for (int i3 = 0; i3 < f3->K; ++i3)
                for (int i4 = 0; i4 < f4->K; ++i4) {
                    double tmp = orc_eri_3d_rys(f1->shell, f2->shell, f3->shell, f4->shell,
                                                f1->center, f2->center, f3->center, f4->center,
                                                f1->expns[i1], f2->expns[i2], f3->expns[i3], f4->expns[i4]);
                    res += f1->nf[i1] * f2->nf[i2] * f3->nf[i3] * f4->nf[i4] *
                           f1->coefs[i1] * f2->coefs[i2] * f3->coefs[i3] * f4->coefs[i4] * tmp;
                }
    return res;
}

/* ------------------------------------------------------------------------ */
/* module mmd (core.f90:5-200) and mmd.py one-electron integrals             */
/* ------------------------------------------------------------------------ */
/* core.f90:30-61, mmd.py:13-30 */
double orc_hermite_e(int i, int j, int t, double qx, double alpha, double beta)
{
    double p = alpha + beta, q = alpha * beta / p;
    if (t < 0 || t > i + j) return 0.0;
    if (i == 0 && j == 0 && t == 0) return exp(-q * qx * qx);
    if (j == 0)
        return (0.5 / p) * orc_hermite_e(i - 1, j, t - 1, qx, alpha, beta) -
               (q * qx / alpha) * orc_hermite_e(i - 1, j, t, qx, alpha, beta) +
               (t + 1) * orc_hermite_e(i - 1, j, t + 1, qx, alpha, beta);
    return (0.5 / p) * orc_hermite_e(i, j - 1, t - 1, qx, alpha, beta) +
           (q * qx / beta) * orc_hermite_e(i, j - 1, t, qx, alpha, beta) +
           (t + 1) * orc_hermite_e(i, j - 1, t + 1, qx, alpha, beta);
}

/* core.f90:64-97, mmd.py:70-108 */
double orc_coulomb_r(int t, int u, int v, int n, double p, double pcx, double pcy,
                     double pcz, double rpc)
{
    double T = p * rpc * rpc, out = 0.0;
    if (t == 0 && u == 0 && v == 0) {
        out += pow(-2.0 * p, n) * orc_boys(n, T);
    } else if (t == 0 && u == 0) {
        if (v >= 2) out += (v - 1) * orc_coulomb_r(t, u, v - 2, n + 1, p, pcx, pcy, pcz, rpc);
        out += pcz * orc_coulomb_r(t, u, v - 1, n + 1, p, pcx, pcy, pcz, rpc);
    } else if (t == 0) {
        if (u >= 2) out += (u - 1) * orc_coulomb_r(t, u - 2, v, n + 1, p, pcx, pcy, pcz, rpc);
        out += pcy * orc_coulomb_r(t, u - 1, v, n + 1, p, pcx, pcy, pcz, rpc);
    } else {
        if (t >= 2) out += (t - 1) * orc_coulomb_r(t - 2, u, v, n + 1, p, pcx, pcy, pcz, rpc);
        out += pcx * orc_coulomb_r(t - 1, u, v, n + 1, p, pcx, pcy, pcz, rpc);
    }
    return out;
}

/* core.f90:100-165 */
double orc_mmd_eri_3d(double alpha, const int *s1, const double *c1,
                      double beta, const int *s2, const double *c2,
                      double gamma, const int *s3, const double *c3,
                      double delta, const int *s4, const double *c4)
{
    double p = alpha + beta, q = gamma + delta, pq = p * q / (p + q);
    double P[3], Q[3], r2 = 0.0;
    for (int d = 0; d < 3; ++d) {
        P[d] = (alpha * c1[d] + beta * c2[d]) / p;
        Q[d] = (gamma * c3[d] + delta * c4[d]) / q;
        r2 += (P[d] - Q[d]) * (P[d] - Q[d]);
    }
    double rpq = sqrt(r2), out = 0.0;
    for (int t = 0; t <= s1[0] + s2[0]; ++t)
     for (int u = 0; u <= s1[1] + s2[1]; ++u)
      for (int v = 0; v <= s1[2] + s2[2]; ++v) {
        double e1 = orc_hermite_e(s1[0], s2[0], t, c1[0] - c2[0], alpha, beta);
        double e2 = orc_hermite_e(s1[1], s2[1], u, c1[1] - c2[1], alpha, beta);
        double e3 = orc_hermite_e(s1[2], s2[2], v, c1[2] - c2[2], alpha, beta);
        for (int tau = 0; tau <= s3[0] + s4[0]; ++tau)
         for (int nu = 0; nu <= s3[1] + s4[1]; ++nu)
          for (int phi = 0; phi <= s3[2] + s4[2]; ++phi) {
            double e4 = orc_hermite_e(s3[0], s4[0], tau, c3[0] - c4[0], gamma, delta);
            double e5 = orc_hermite_e(s3[1], s4[1], nu, c3[1] - c4[1], gamma, delta);
            double e6 = orc_hermite_e(s3[2], s4[2], phi, c3[2] - c4[2], gamma, delta);
            double r = orc_coulomb_r(t + tau, u + nu, v + phi, 0, pq, P[0] - Q[0], P[1] - Q[1], P[2] - Q[2], rpq);
            double sgn = ((tau + nu + phi) & 1) ? -1.0 : 1.0;
            out += e1 * e2 * e3 * e4 * e5 * e6 * sgn * r;
          }
      }
    return out * 2.0 * pow(ORC_PI, 2.5) / (p * q * sqrt(p + q));
}

/* core.f90:167-198 */
double orc_mmd_eri(const orc_cgf *f1, const orc_cgf *f2, const orc_cgf *f3, const orc_cgf *f4)
{
    double res = 0.0;
    for (int i1 = 0; i1 < f1->K; ++i1)
     for (int i2 = 0; i2 < f2->K; ++i2)
      for (int i3 = 0; i3 < f3->K; ++i3)
       for (int i4 = 0; i4 < f4->K; ++i4) {
        double tmp = orc_mmd_eri_3d(f1->expns[i1], f1->shell, f1->center, f2->expns[i2], f2->shell, f2->center,
                                    f3->expns[i3], f3->shell, f3->center, f4->expns[i4], f4->shell, f4->center);
        res += f1->nf[i1] * f2->nf[i2] * f3->nf[i3] * f4->nf[i4] *
               f1->coefs[i1] * f2->coefs[i2] * f3->coefs[i3] * f4->coefs[i4] * tmp;
       }
    return res;
}

/* mmd.py:32-39 */
static double ov3d(double a, const int *s1, const double *c1, double b, const int *s2, const double *c2)
{
    double sx = orc_hermite_e(s1[0], s2[0], 0, c1[0] - c2[0], a, b);
    double sy = orc_hermite_e(s1[1], s2[1], 0, c1[1] - c2[1], a, b);
    double sz = orc_hermite_e(s1[2], s2[2], 0, c1[2] - c2[2], a, b);
    return sx * sy * sz * pow(ORC_PI / (a + b), 1.5);
}

/* mmd.py:49-60 */
static double kin3d(double a, const int *s1, const double *c1, double b, const int *s2, const double *c2)
{
    int l2 = s2[0], m2 = s2[1], n2 = s2[2];
    int sx2[3] = {l2 + 2, m2, n2}, sy2[3] = {l2, m2 + 2, n2}, sz2[3] = {l2, m2, n2 + 2};
    int sxm[3] = {l2 - 2, m2, n2}, sym[3] = {l2, m2 - 2, n2}, szm[3] = {l2, m2, n2 - 2};
    double t0 = b * (2 * (l2 + m2 + n2) + 3) * ov3d(a, s1, c1, b, s2, c2);
    double t1 = -2.0 * b * b * (ov3d(a, s1, c1, b, sx2, c2) + ov3d(a, s1, c1, b, sy2, c2) + ov3d(a, s1, c1, b, sz2, c2));
    double t2 = -0.5 * ((l2 * (l2 - 1) ? l2 * (l2 - 1) * ov3d(a, s1, c1, b, sxm, c2) : 0.0) +
                        (m2 * (m2 - 1) ? m2 * (m2 - 1) * ov3d(a, s1, c1, b, sym, c2) : 0.0) +
                        (n2 * (n2 - 1) ? n2 * (n2 - 1) * ov3d(a, s1, c1, b, szm, c2) : 0.0));
    return t0 + t1 + t2;
}

/* mmd.py:110-133 */
static double pot3d(double a, const int *s1, const double *c1, double b, const int *s2, const double *c2, const double *C)
{
    double p = a + b, P[3], r2 = 0.0;
    for (int d = 0; d < 3; ++d) { P[d] = (a * c1[d] + b * c2[d]) / p; r2 += (P[d] - C[d]) * (P[d] - C[d]); }
    double rpc = sqrt(r2), res = 0.0;
    for (int t = 0; t <= s1[0] + s2[0]; ++t)
     for (int u = 0; u <= s1[1] + s2[1]; ++u)
      for (int v = 0; v <= s1[2] + s2[2]; ++v)
        res += orc_hermite_e(s1[0], s2[0], t, c1[0] - c2[0], a, b) *
               orc_hermite_e(s1[1], s2[1], u, c1[1] - c2[1], a, b) *
               orc_hermite_e(s1[2], s2[2], v, c1[2] - c2[2], a, b) *
               orc_coulomb_r(t, u, v, 0, p, P[0] - C[0], P[1] - C[1], P[2] - C[2], rpc);
    return res * 2.0 * ORC_PI / p;
}

/* mmd.py:41-47, 62-68, 135-141 and hf.py:266-274 */
void orc_one_electron(const orc_cgf *cg, int n, const double *atom_xyz,
                      const double *Z, int natom, double *S, double *T, double *V,
                      int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic)
#endif
    for (int ij = 0; ij < n * n; ++ij) {
        int i = ij / n, j = ij % n;
        const orc_cgf *f1 = &cg[i], *f2 = &cg[j];
        double s = 0.0, t = 0.0, v = 0.0;
        for (int a = 0; a < f1->K; ++a)
            for (int b = 0; b < f2->K; ++b) {
                double c = f1->nf[a] * f2->nf[b] * f1->coefs[a] * f2->coefs[b];
                s += c * ov3d(f1->expns[a], f1->shell, f1->center, f2->expns[b], f2->shell, f2->center);
                t += c * kin3d(f1->expns[a], f1->shell, f1->center, f2->expns[b], f2->shell, f2->center);
            }
        for (int at = 0; at < natom; ++at) {
            double va = 0.0;
            for (int a = 0; a < f1->K; ++a)
                for (int b = 0; b < f2->K; ++b)
                    va += f1->nf[a] * f2->nf[b] * f1->coefs[a] * f2->coefs[b] *
                          pot3d(f1->expns[a], f1->shell, f1->center, f2->expns[b], f2->shell, f2->center, atom_xyz + 3 * at);
            v += va * (-Z[at]);
        }
        S[ij] = s; T[ij] = t; V[ij] = v;
    }
}

/* ------------------------------------------------------------------------ */
/* drivers                                                                   */
/* ------------------------------------------------------------------------ */
static double eri_any(const orc_cgf *cg, int i, int j, int k, int l, int method)
{
    return method == 1 ? orc_mmd_eri(&cg[i], &cg[j], &cg[k], &cg[l])
                       : orc_eri_rys(&cg[i], &cg[j], &cg[k], &cg[l]);
}

/* ERIs of an explicit AO quartet list idx[4*q] */
void orc_eri_list(const orc_cgf *cg, const int32_t *idx, int64_t nq, double *out,
                  int method, int nthreads)
{
    orc_init();
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t q = 0; q < nq; ++q)
        out[q] = eri_any(cg, idx[4 * q], idx[4 * q + 1], idx[4 * q + 2], idx[4 * q + 3], method);
}

/* number of unique AO quartets enumerated by hf.py:37-43 */
int64_t orc_num_unique(int n)
{
    int64_t np_ = (int64_t)n * (n + 1) / 2;
    return np_ * (np_ + 1) / 2;
}

/* decode the q-th unique quartet in the order of hf.py:37-43 is not needed:
 * a pair-index enumeration (ij >= kl over the packed pair index) visits the
 * same set, which is what the 8-fold scatter needs. */
static void pair_of(int64_t ij, int *i, int *j)
{
    int64_t a = (int64_t)((sqrt(8.0 * (double)ij + 1.0) - 1.0) / 2.0);
    while (a * (a + 1) / 2 > ij) --a;
    while ((a + 1) * (a + 2) / 2 <= ij) ++a;
    *i = (int)a; *j = (int)(ij - a * (a + 1) / 2);
}

/* hf.py:33-61: all unique quartets, 8-fold scatter into dense n^4 */
void orc_build_eri_dense(const orc_cgf *cg, int n, double *out, int method, int nthreads)
{
    orc_init();
    int64_t npair = (int64_t)n * (n + 1) / 2;
    int64_t n2 = (int64_t)n * n, n3 = n2 * n;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t ij = 0; ij < npair; ++ij) {
        int i, j;
        pair_of(ij, &i, &j);
        for (int64_t kl = 0; kl <= ij; ++kl) {
            int k, l;
            pair_of(kl, &k, &l);
            double v = eri_any(cg, i, j, k, l, method);
            int perm[8][4] = {{i, j, k, l}, {j, i, k, l}, {i, j, l, k}, {j, i, l, k},
                              {k, l, i, j}, {l, k, i, j}, {k, l, j, i}, {l, k, j, i}};
            for (int p = 0; p < 8; ++p)
                out[perm[p][0] * n3 + perm[p][1] * n2 + (int64_t)perm[p][2] * n + perm[p][3]] = v;
        }
    }
}

/* Coulomb / exchange from unique quartets without the dense tensor:
 * J_pq = sum_rs (pq|rs) D_rs, K_pq = sum_rs (pr|qs) D_rs (hf.py:300 maths).
 * Optional sampling: only pair rows ij with (ij % stride) == phase are done
 * (used to time a bounded sample); stride 1 = everything. */
void orc_jk_direct(const orc_cgf *cg, int n, const double *D, double *J, double *K,
                   int method, int nthreads, int64_t stride, int64_t phase)
{
    orc_init();
    int64_t npair = (int64_t)n * (n + 1) / 2, nn = (int64_t)n * n;
    memset(J, 0, sizeof(double) * nn);
    memset(K, 0, sizeof(double) * nn);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        double *Jt = calloc(nn, sizeof(double)), *Kt = calloc(nn, sizeof(double));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int64_t ij = 0; ij < npair; ++ij) {
            if (stride > 1 && (ij % stride) != phase) continue;
            int i, j;
            pair_of(ij, &i, &j);
            for (int64_t kl = 0; kl <= ij; ++kl) {
                int k, l;
                pair_of(kl, &k, &l);
                double v = eri_any(cg, i, j, k, l, method);
                /* degeneracy-scaled value, all 8 permutations (each distinct
                 * permutation then counts exactly once) */
                double s = v;
                if (i == j) s *= 0.5;
                if (k == l) s *= 0.5;
                if (ij == kl) s *= 0.5;
                int P[8][4] = {{i, j, k, l}, {j, i, k, l}, {i, j, l, k}, {j, i, l, k},
                               {k, l, i, j}, {l, k, i, j}, {k, l, j, i}, {l, k, j, i}};
                for (int p = 0; p < 8; ++p) {
                    int a = P[p][0], b = P[p][1], c = P[p][2], d = P[p][3];
                    Jt[a * n + b] += s * D[c * n + d];
                    Kt[a * n + c] += s * D[b * n + d];
                }
            }
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        {
            for (int64_t x = 0; x < nn; ++x) { J[x] += Jt[x]; K[x] += Kt[x]; }
        }
        free(Jt); free(Kt);
    }
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
