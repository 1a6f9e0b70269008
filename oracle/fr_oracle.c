/*
 * fr_oracle.c -- CPU FP64 restatement of FluxReconstruction.jl's hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline).  See
 * fr_oracle.h for the layout conventions and the parity status.  Every
 * function cites the reference file:line it restates.
 *
 * Rounding: the reference's dot products (`dot`, `u * ll`, `f * lpdm'`) go
 * through BLAS, whose summation order and use of fused multiply-adds depend on
 * the BLAS build and cannot be pinned.  The oracle fixes one order: every dot
 * product is s = v0 w0, then s = fma(v_q, w_q, s) in ascending q (dotw below),
 * and the few other fused multiply-adds are written out with fma().  It is
 * compiled with -ffp-contract=off so that no other operation is fused; every
 * other expression keeps the reference's operation order.
 */
#include "fr_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static int g_threads = 0;
void fro_set_threads(int n) { g_threads = n; }
int fro_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}
#ifdef _OPENMP
#define OMP_THREADS num_threads(fro_get_threads())
#endif

/* dot product of n values v[q*sv] with weights w[q*sw] in the fixed order
 * s = v0 w0; s = fma(v_q, w_q, s) */
static inline double dotw(const double *v, long sv, const double *w, long sw, int n) {
    double s = v[0] * w[0];
    for (int q = 1; q < n; ++q) s = fma(v[q * sv], w[q * sw], s);
    return s;
}

/* ------------------------------------------------------------------------
 * Setup math
 * ---------------------------------------------------------------------- */

/* Legendre polynomial P_n(x) by the three-term recurrence. */
double fro_legendre_p(int n, double x) {
    if (n == 0) return 1.0;
    double p0 = 1.0, p1 = x;
    for (int k = 1; k < n; ++k) {
        double p2 = ((2.0 * k + 1.0) * x * p1 - k * p0) / (k + 1.0);
        p0 = p1;
        p1 = p2;
    }
    return p1;
}

/* P_n'(x): replaces GSL sf_legendre_Pl_deriv_array used by
 * src/Polynomial/poly_legendre.jl:13 (last element of the derivative array).
 * Recurrence P'_n = P'_{n-2} + (2n-1) P_{n-1}, exact at x = +-1. */
double fro_dlegendre(int n, double x) {
    if (n <= 0) return 0.0;
    double dm2 = 0.0, dm1 = 1.0; /* P'_0, P'_1 */
    if (n == 1) return 1.0;
    for (int k = 2; k <= n; ++k) {
        double d = dm2 + (2.0 * k - 1.0) * fro_legendre_p(k - 1, x);
        dm2 = dm1;
        dm1 = d;
    }
    return dm1;
}

/* Gauss-Legendre nodes (ascending) and weights: the values of
 * FastGaussQuadrature.gausslegendre used at src/Polynomial/poly_legendre.jl:6
 * and src/struct.jl:47.  Newton iteration on P_n from the Chebyshev-like
 * initial guess; weights 2/((1-x^2) P_n'(x)^2). */
void fro_gauss_legendre(int n, double *x, double *w) {
    for (int i = 0; i < n; ++i) {
        double z = cos(M_PI * (i + 0.75) / (n + 0.5));
        for (int it = 0; it < 100; ++it) {
            double p = fro_legendre_p(n, z);
            double dp = fro_dlegendre(n, z);
            double dz = p / dp;
            z -= dz;
            if (fabs(dz) < 1e-16) break;
        }
        double dp = fro_dlegendre(n, z);
        /* ascending order: the guess above is descending */
        x[n - 1 - i] = z;
        w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
    /* symmetrise to remove the last ulp of asymmetry */
    for (int i = 0; i < n / 2; ++i) {
        double a = 0.5 * (x[n - 1 - i] - x[i]);
        x[i] = -a;
        x[n - 1 - i] = a;
        double b = 0.5 * (w[i] + w[n - 1 - i]);
        w[i] = b;
        w[n - 1 - i] = b;
    }
    if (n % 2 == 1) x[n / 2] = 0.0;
}

/* Correction-function derivatives, src/Polynomial/poly_legendre.jl:29-71:
 * kind 0 = dradau (:29-37), 1 = dsd (:44-54), 2 = dhuynh (:61-71). */
void fro_dcorrection(int kind, int p, const double *x, int nx, double *dgl, double *dgr) {
    double sgn = (p % 2 == 0) ? 1.0 : -1.0; /* (-1.0)^p */
    for (int i = 0; i < nx; ++i) {
        double d = fro_dlegendre(p, x[i]);
        double dp = fro_dlegendre(p + 1, x[i]);
        double y;
        if (kind == 0) {
            y = dp;
        } else {
            double dm = fro_dlegendre(p - 1, x[i]);
            if (kind == 1)
                y = (p * dm + (p + 1) * dp) / (2 * p + 1);
            else
                y = ((p + 1) * dm + p * dp) / (2 * p + 1);
        }
        dgl[i] = sgn * 0.5 * (d - y);
        dgr[i] = 0.5 * (d + y);
    }
}

/* lagrange_point, src/Polynomial/poly_lagrange.jl:6-20 */
void fro_lagrange_point(const double *sp, int nsp, double x, double *l) {
    for (int k = 0; k < nsp; ++k) {
        double tmp = 1.0;
        for (int j = 0; j < nsp; ++j)
            if (j != k) tmp *= (x - sp[j]) / (sp[k] - sp[j]);
        l[k] = tmp;
    }
}

/* dlagrange (nodal differentiation matrix lpdm[m,k] = l_k'(r_m)),
 * src/Polynomial/poly_lagrange.jl:38-59; column-major lpdm[m + nsp*k]. */
void fro_dlagrange(const double *sp, int nsp, double *lpdm) {
    for (int k = 0; k < nsp; ++k)
        for (int m = 0; m < nsp; ++m) {
            double lsum = 0.0;
            for (int l = 0; l < nsp; ++l) {
                double tmp = 1.0;
                for (int j = 0; j < nsp; ++j)
                    if (j != k && j != l) tmp *= (sp[m] - sp[j]) / (sp[k] - sp[j]);
                if (l != k) lsum += tmp / (sp[k] - sp[l]);
            }
            lpdm[m + nsp * k] = lsum;
        }
}

/* Orthonormal Jacobi polynomial, src/Polynomial/poly_jacobi.jl:7-42 */
double fro_jacobi_p(double x, double alpha, double beta, int N) {
    double gamma0 = pow(2.0, alpha + beta + 1) / (alpha + beta + 1) * tgamma(alpha + 1) *
                    tgamma(beta + 1) / tgamma(alpha + beta + 1);
    double p0 = 1.0 / sqrt(gamma0);
    if (N == 0) return p0;
    double gamma1 = (alpha + 1) * (beta + 1) / (alpha + beta + 3) * gamma0;
    double p1 = ((alpha + beta + 2) * x / 2 + (alpha - beta) / 2) / sqrt(gamma1);
    if (N == 1) return p1;
    double aold = 2 / (2 + alpha + beta) * sqrt((alpha + 1) * (beta + 1) / (alpha + beta + 3));
    for (int i = 1; i <= N - 1; ++i) {
        double h1 = 2 * i + alpha + beta;
        double anew = 2 / (h1 + 2) *
                      sqrt((i + 1) * (i + 1 + alpha + beta) * (i + 1 + alpha) * (i + 1 + beta) /
                           (h1 + 1) / (h1 + 3));
        double bnew = -(alpha * alpha - beta * beta) / h1 / (h1 + 2);
        double p2 = 1 / anew * (-aold * p0 + (x - bnew) * p1);
        aold = anew;
        p0 = p1;
        p1 = p2;
    }
    return p1;
}

/* dJacobiP, src/Polynomial/poly_jacobi.jl:88-95 */
double fro_djacobi_p(double x, double alpha, double beta, int N) {
    if (N == 0) return 0.0;
    return sqrt(N * (N + alpha + beta + 1)) * fro_jacobi_p(x, alpha + 1, beta + 1, N - 1);
}

/* vandermonde_matrix(N, r), src/Transform/transform.jl:18-26; V[i + nr*j] */
void fro_vandermonde_1d(int N, const double *r, int nr, double *V) {
    for (int j = 0; j <= N; ++j)
        for (int i = 0; i < nr; ++i) V[i + nr * j] = fro_jacobi_p(r[i], 0, 0, j);
}

/* dvandermonde_matrix(N, r), src/Transform/transform.jl:76-84 */
void fro_dvandermonde_1d(int N, const double *r, int nr, double *Vr) {
    for (int j = 0; j <= N; ++j)
        for (int i = 0; i < nr; ++i) Vr[i + nr * j] = fro_djacobi_p(r[i], 0, 0, j);
}

/* vandermonde_matrix(Quad, N, r, s), src/Transform/transform.jl:55-68:
 * mode sk runs over i (outer) and j (inner); V[pt + n*sk]. */
void fro_vandermonde_quad(int N, const double *r, const double *s, int n, double *V) {
    int sk = 0;
    for (int i = 0; i <= N; ++i)
        for (int j = 0; j <= N; ++j) {
            for (int q = 0; q < n; ++q)
                V[q + n * sk] = fro_jacobi_p(r[q], 0, 0, i) * fro_jacobi_p(s[q], 0, 0, j);
            ++sk;
        }
}

/* Gauss-Jordan inverse with partial pivoting (stands in for Julia's inv). */
int fro_inverse(int n, const double *A, double *Ainv) {
    double *M = (double *)malloc(sizeof(double) * n * 2 * n);
    if (!M) return -1;
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < 2 * n; ++c)
            M[r * 2 * n + c] = c < n ? A[r + n * c] : (c - n == r ? 1.0 : 0.0);
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (fabs(M[r * 2 * n + c]) > fabs(M[piv * 2 * n + c])) piv = r;
        if (M[piv * 2 * n + c] == 0.0) {
            free(M);
            return -2;
        }
        if (piv != c)
            for (int k = 0; k < 2 * n; ++k) {
                double t = M[c * 2 * n + k];
                M[c * 2 * n + k] = M[piv * 2 * n + k];
                M[piv * 2 * n + k] = t;
            }
        double d = M[c * 2 * n + c];
        for (int k = 0; k < 2 * n; ++k) M[c * 2 * n + k] /= d;
        for (int r = 0; r < n; ++r)
            if (r != c) {
                double f = M[r * 2 * n + c];
                if (f != 0.0)
                    for (int k = 0; k < 2 * n; ++k) M[r * 2 * n + k] -= f * M[c * 2 * n + k];
            }
    }
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) Ainv[r + n * c] = M[r * 2 * n + n + c];
    free(M);
    return 0;
}

/* shock_detector, src/dissipation.jl:13-23 */
int fro_shock_detector(double Se, int deg, double S0, double kappa) {
    (void)deg;
    double sigma;
    if (Se < S0 - kappa)
        sigma = 1.0;
    else if (S0 - kappa <= Se && Se < S0 + kappa)
        sigma = 0.5 * (1.0 - sin(0.5 * M_PI * (Se - S0) / kappa));
    else
        sigma = 0.0;
    return sigma < 0.99 ? 1 : 0;
}

/* ------------------------------------------------------------------------
 * Physics helpers (KitBase 0.9 restatements; the package is not vendored)
 * ---------------------------------------------------------------------- */

/* prim = [rho, U, V, lambda], lambda = rho / (2 p) (KitBase convention) */
void fro_prim_conserve2d(const double *prim, double gamma, double *w) {
    w[0] = prim[0];
    w[1] = prim[0] * prim[1];
    w[2] = prim[0] * prim[2];
    w[3] = 0.5 * prim[0] / prim[3] / (gamma - 1.0) + 0.5 * prim[0] * (prim[1] * prim[1] + prim[2] * prim[2]);
}

void fro_conserve_prim2d(const double *w, double gamma, double *prim) {
    prim[0] = w[0];
    prim[1] = w[1] / w[0];
    prim[2] = w[2] / w[0];
    prim[3] = 0.5 * w[0] / (gamma - 1.0) / (w[3] - 0.5 * (w[1] * w[1] + w[2] * w[2]) / w[0]);
}

void fro_prim_conserve1d(const double *prim, double gamma, double *w) {
    w[0] = prim[0];
    w[1] = prim[0] * prim[1];
    w[2] = 0.5 * prim[0] / prim[2] / (gamma - 1.0) + 0.5 * prim[0] * prim[1] * prim[1];
}

/* Physical Euler flux in direction dir (0 = x, 1 = y) of the conserved state
 * w, with velocity components and pressure computed once:
 * U = mx/rho, V = my/rho, p = (gamma-1)(E - 0.5 (mx U + my V)). */
static inline void euler_flux_dir(const double *w, double gamma, int dir, double *f, double *un_out,
                                  double *c_out) {
    double rinv = 1.0 / w[0];
    double U = w[1] * rinv, V = w[2] * rinv;
    double p = (gamma - 1.0) * (w[3] - 0.5 * fma(w[1], U, w[2] * V));
    double un = dir == 0 ? U : V;
    f[0] = w[1 + dir];
    f[1] = dir == 0 ? fma(w[1], U, p) : w[1] * V;
    f[2] = dir == 1 ? fma(w[2], V, p) : w[2] * U;
    f[3] = (w[3] + p) * un;
    if (un_out) *un_out = un;
    if (c_out) *c_out = sqrt(gamma * p * rinv);
}

/* HLL flux with Davis wave-speed estimates (Toro, "Riemann Solvers and
 * Numerical Methods for Fluid Dynamics", ch. 10), in direction dir.  Stands
 * in for KitBase.flux_hll!(fw, wL, wR, gamma, 1.0) called at
 * example/shock-vortex.jl:78 (x faces) and :84-87 (y faces through
 * local_frame/global_frame, which this directional form equals exactly). */
void fro_flux_hll2d(const double *wL, const double *wR, double gamma, int dir, double *fw) {
    double fL[4], fR[4], uL, uR, cL, cR;
    euler_flux_dir(wL, gamma, dir, fL, &uL, &cL);
    euler_flux_dir(wR, gamma, dir, fR, &uR, &cR);
    double sl = fmin(uL - cL, uR - cR);
    double sr = fmax(uL + cL, uR + cR);
    if (sl >= 0.0) {
        for (int m = 0; m < 4; ++m) fw[m] = fL[m];
    } else if (sr <= 0.0) {
        for (int m = 0; m < 4; ++m) fw[m] = fR[m];
    } else {
        double factor = 1.0 / (sr - sl);
        for (int m = 0; m < 4; ++m)
            fw[m] = factor * (sr * fL[m] - sl * fR[m] + sl * sr * (wR[m] - wL[m]));
    }
}

/* Local Lax-Friedrichs (Rusanov) flux: 0.5 (FL + FR) - 0.5 lambda (wR - wL),
 * lambda = max(|uL| + cL, |uR| + cR). */
void fro_flux_lf2d(const double *wL, const double *wR, double gamma, int dir, double *fw) {
    double fL[4], fR[4], uL, uR, cL, cR;
    euler_flux_dir(wL, gamma, dir, fL, &uL, &cL);
    euler_flux_dir(wR, gamma, dir, fR, &uR, &cR);
    double lam = fmax(fabs(uL) + cL, fabs(uR) + cR);
    for (int m = 0; m < 4; ++m) fw[m] = 0.5 * (fL[m] + fR[m]) - 0.5 * lam * (wR[m] - wL[m]);
}

/* 1D Euler flux [m, m U + p, (E + p) U] */
static inline void euler_flux_1d(const double *w, double gamma, double *f, double *u_out, double *p_out) {
    double U = w[1] / w[0];
    double p = (gamma - 1.0) * (w[2] - 0.5 * w[1] * U);
    f[0] = w[1];
    f[1] = fma(w[1], U, p);
    f[2] = (w[2] + p) * U;
    if (u_out) *u_out = U;
    if (p_out) *p_out = p;
}

/* 1D HLL, stands in for KitBase.flux_hll! at src/Equation/eq_euler.jl:53 */
void fro_flux_hll1d(const double *wL, const double *wR, double gamma, double *fw) {
    double fL[3], fR[3], uL, uR, pL, pR;
    euler_flux_1d(wL, gamma, fL, &uL, &pL);
    euler_flux_1d(wR, gamma, fR, &uR, &pR);
    double cL = sqrt(gamma * pL / wL[0]);
    double cR = sqrt(gamma * pR / wR[0]);
    double sl = fmin(uL - cL, uR - cR);
    double sr = fmax(uL + cL, uR + cR);
    if (sl >= 0.0) {
        for (int m = 0; m < 3; ++m) fw[m] = fL[m];
    } else if (sr <= 0.0) {
        for (int m = 0; m < 3; ++m) fw[m] = fR[m];
    } else {
        double factor = 1.0 / (sr - sl);
        for (int m = 0; m < 3; ++m)
            fw[m] = factor * (sr * fL[m] - sl * fR[m] + sl * sr * (wR[m] - wL[m]));
    }
}

/* Normal-shock (Rankine-Hugoniot) states for a shock of upstream Mach Ma
 * with upstream rho = 1, p = 1 (so c = sqrt(gamma)).  pre/post = [rho, u, p].
 * Stands in for KitBase.ib_rh used at example/shock-vortex.jl:162. */
void fro_ib_rh(double Ma, double gamma, double *pre, double *post) {
    double c1 = sqrt(gamma);
    pre[0] = 1.0;
    pre[1] = Ma * c1;
    pre[2] = 1.0;
    double M2 = Ma * Ma;
    double rr = (gamma + 1.0) * M2 / ((gamma - 1.0) * M2 + 2.0);
    double pr = 1.0 + 2.0 * gamma / (gamma + 1.0) * (M2 - 1.0);
    post[0] = rr;
    post[1] = pre[1] / rr;
    post[2] = pr;
}

/* ------------------------------------------------------------------------
 * Residuals
 * ---------------------------------------------------------------------- */

long fro_ndof(const fro_cfg *c) {
    switch (c->kind) {
    case FRO_ADVECTION:
    case FRO_BURGERS: return (long)c->nx * c->np;
    case FRO_EULER1D: return (long)c->nx * c->np * 3;
    case FRO_EULER2D: return (long)c->nx * c->ny * c->np * c->np * 4;
    case FRO_BGK1D: return (long)c->nx * c->nvel * c->np;
    }
    return 0;
}

/* Scalar 1D residual: frode_advection! (src/Equation/eq_advection.jl:55-77)
 * with advection_dflux! (:103-111), the face interpolation (:63-64),
 * advection_iflux! (:128-137, epsilon 1e-8), rhs1 = f*lpdm' (:68),
 * scalar_rhs! (src/Equation/eq_scalar.jl:1-12) and period_advection!
 * (eq_advection.jl:158-175, epsilon 1e-6) or dirichlet_advection! (:153-156).
 * Burgers uses the same machinery with the flux u^2/2. */
static void rhs_scalar1d(const fro_cfg *c, double *du, const double *u) {
    int ne = c->nx, np = c->np;
    double *f = (double *)malloc(sizeof(double) * ne * np);
    double *uf = (double *)malloc(sizeof(double) * ne * 2);
    double *ff = (double *)malloc(sizeof(double) * ne * 2);
    double *fi = (double *)malloc(sizeof(double) * (ne + 1));
    for (int k = 0; k < np; ++k)
        for (int i = 0; i < ne; ++i) {
            double x = u[i + ne * k];
            double fl = c->kind == FRO_BURGERS ? 0.5 * x * x : c->a * x;
            f[i + ne * k] = fl / c->J[i];
        }
    for (int i = 0; i < ne; ++i) {
        uf[i] = dotw(u + i, ne, c->ll, 1, np);
        uf[i + ne] = dotw(u + i, ne, c->lr, 1, np);
        ff[i] = dotw(f + i, ne, c->ll, 1, np);
        ff[i + ne] = dotw(f + i, ne, c->lr, 1, np);
    }
    for (int i = 1; i < ne; ++i) {
        double au = (ff[i] - ff[i - 1 + ne]) / (uf[i] - uf[i - 1 + ne] + c->eps_interior);
        fi[i] = 0.5 * (ff[i] + ff[i - 1 + ne]) - 0.5 * fabs(au) * (uf[i] - uf[i - 1 + ne]);
    }
    int periodic = c->bc[0] == FRO_BC_PERIODIC;
    if (periodic) {
        double au = (ff[0] - ff[ne - 1 + ne]) / (uf[0] - uf[ne - 1 + ne] + c->eps_periodic);
        fi[0] = 0.5 * (ff[ne - 1 + ne] + ff[0]) - 0.5 * fabs(au) * (uf[0] - uf[ne - 1 + ne]);
        fi[ne] = fi[0];
    }
    for (int m = 0; m < np; ++m)
        for (int i = 0; i < ne; ++i) {
            int boundary = (i == 0 || i == ne - 1);
            if (boundary && !periodic) {
                du[i + ne * m] = 0.0;
                continue;
            }
            double r = dotw(f + i, ne, c->lpdm + m, np, np);
            du[i + ne * m] = -fma(fi[i + 1] - ff[i + ne], c->dgr[m], fma(fi[i] - ff[i], c->dgl[m], r));
        }
    free(f);
    free(uf);
    free(ff);
    free(fi);
}

/* 1D Euler residual: frode_euler! (src/Equation/eq_euler.jl:29-73) with
 * period_euler! (:80-98) or dirichlet_euler! (:75-78).  The interface flux
 * is scaled by 1/J[i] in the combination (:63-64). */
static void rhs_euler1d(const fro_cfg *c, double *du, const double *u) {
    int ne = c->nx, np = c->np;
    double g = c->gamma;
    double *f = (double *)malloc(sizeof(double) * ne * np * 3);
    double *uf = (double *)malloc(sizeof(double) * ne * 2 * 3);
    double *ff = (double *)malloc(sizeof(double) * ne * 2 * 3);
    double *fi = (double *)malloc(sizeof(double) * (ne + 1) * 3);
#define U1(i, k, m) u[(i) + ne * ((k) + np * (m))]
#define F1(i, k, m) f[(i) + ne * ((k) + np * (m))]
    for (int k = 0; k < np; ++k)
        for (int i = 0; i < ne; ++i) {
            double w[3] = {U1(i, k, 0), U1(i, k, 1), U1(i, k, 2)}, fl[3];
            euler_flux_1d(w, g, fl, NULL, NULL);
            for (int m = 0; m < 3; ++m) F1(i, k, m) = fl[m] / c->J[i];
        }
    /* u_face[i, side, m]: side 0 = left (ll), 1 = right (lr) */
    for (int m = 0; m < 3; ++m)
        for (int i = 0; i < ne; ++i) {
            uf[i + ne * (0 + 2 * m)] = dotw(&U1(i, 0, m), ne, c->ll, 1, np);
            uf[i + ne * (1 + 2 * m)] = dotw(&U1(i, 0, m), ne, c->lr, 1, np);
            ff[i + ne * (0 + 2 * m)] = dotw(&F1(i, 0, m), ne, c->ll, 1, np);
            ff[i + ne * (1 + 2 * m)] = dotw(&F1(i, 0, m), ne, c->lr, 1, np);
        }
    for (int i = 1; i < ne; ++i) {
        double wL[3], wR[3], fw[3];
        for (int m = 0; m < 3; ++m) {
            wL[m] = uf[(i - 1) + ne * (1 + 2 * m)];
            wR[m] = uf[i + ne * (0 + 2 * m)];
        }
        fro_flux_hll1d(wL, wR, g, fw);
        for (int m = 0; m < 3; ++m) fi[i + (ne + 1) * m] = fw[m];
    }
    int periodic = c->bc[0] == FRO_BC_PERIODIC;
    if (periodic) {
        double wL[3], wR[3], fw[3];
        for (int m = 0; m < 3; ++m) {
            wL[m] = uf[(ne - 1) + ne * (1 + 2 * m)];
            wR[m] = uf[0 + ne * (0 + 2 * m)];
        }
        fro_flux_hll1d(wL, wR, g, fw);
        for (int m = 0; m < 3; ++m) {
            fi[0 + (ne + 1) * m] = fw[m];
            fi[ne + (ne + 1) * m] = fw[m];
        }
    }
    for (int m = 0; m < 3; ++m)
        for (int kk = 0; kk < np; ++kk)
            for (int i = 0; i < ne; ++i) {
                int boundary = (i == 0 || i == ne - 1);
                double *d = &du[i + ne * (kk + np * m)];
                if (boundary && !periodic) {
                    *d = 0.0;
                    continue;
                }
                double r = dotw(&F1(i, 0, m), ne, c->lpdm + kk, np, np);
                double aL = fi[i + (ne + 1) * m] / c->J[i] - ff[i + ne * (0 + 2 * m)];
                double aR = fi[i + 1 + (ne + 1) * m] / c->J[i] - ff[i + ne * (1 + 2 * m)];
                *d = -fma(aR, c->dgr[kk], fma(aL, c->dgl[kk], r));
            }
#undef U1
#undef F1
    free(f);
    free(uf);
    free(ff);
    free(fi);
}

/* 2D Euler residual on rectangular elements: the dudt! closure of
 * example/shock-vortex.jl:26-118 (same as example/euler2d_wave.jl:35-107)
 * with a choice of HLL or local Lax-Friedrichs interface flux and with the
 * ghost layer refreshed every stage from the boundary kinds (periodic:
 * euler2d_wave.jl:125-135 without the sign flips; copy and fixed inflow:
 * shock-vortex.jl:323-330).
 * Face numbering follows the reference: 0 = bottom (s=-1), 1 = right
 * (r=+1), 2 = top (s=+1), 3 = left (r=-1).  Internally elements are stored
 * contiguously (64 values for p=3) to keep the CPU loops cache-friendly. */
typedef struct {
    int nxg, nyg, np, E;
    double *ug;  /* ghosted element-contiguous state [jg][ig][m][l][k] */
    double *uface; /* [jg][ig][face][pt][m] */
    double *fface; /* normal flux trace [jg][ig][face][pt][m] (interior only) */
    double *fvol;  /* [j][i][dir][m][l][k] interior only */
    double *fxi;   /* [j][i(0..nx)][pt][m] */
    double *fyi;   /* [j(0..ny)][i][pt][m] */
} e2d_work;

/* element (i, j) (0-based) of a state in the reference layout into an
 * element block of the ghost-extended work array */
static void e2d_copy_elem(const fro_cfg *c, const double *u, int i, int j, double *dst) {
    const int nx = c->nx, np = c->np;
    const long nn = (long)nx * c->ny;
    for (int m = 0; m < 4; ++m)
        for (int l = 0; l < np; ++l)
            for (int k = 0; k < np; ++k)
                dst[(m * np + l) * np + k] = u[i + (long)nx * j + nn * (k + np * (l + (long)np * m))];
}

static void e2d_fill_ghosts(const fro_cfg *c, const double *u, e2d_work *w) {
    int nx = c->nx, ny = c->ny, np = c->np, E = w->E, nxg = w->nxg;
    long nn = (long)nx * ny;
    /* with ghosts refreshed once per step the periodic and copy ghosts come from
     * the step's start state (the scripts' dudt! leaves du = 0 on the ghosts,
     * which they copy after each step) */
    const double *gs = c->ghost_src;
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS
#endif
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            double *dst = w->ug + ((long)(j + 1) * nxg + (i + 1)) * E;
            for (int m = 0; m < 4; ++m)
                for (int l = 0; l < np; ++l)
                    for (int k = 0; k < np; ++k)
                        dst[(m * np + l) * np + k] = u[i + (long)nx * j + nn * (k + np * (l + (long)np * m))];
        }
    /* sides: 0 left (ig=0), 1 right (ig=nx+1), 2 bottom (jg=0), 3 top (jg=ny+1) */
    for (int j = 1; j <= ny; ++j) {
        for (int side = 0; side < 2; ++side) {
            int ig = side == 0 ? 0 : nx + 1;
            double *dst = w->ug + ((long)j * nxg + ig) * E;
            int bc = c->bc[side];
            if (bc == FRO_BC_FIXED) {
                for (int m = 0; m < 4; ++m)
                    for (int q = 0; q < np * np; ++q) dst[m * np * np + q] = c->fixed_state[side][m];
            } else {
                int src_i = bc == FRO_BC_PERIODIC ? (side == 0 ? nx : 1) : (side == 0 ? 1 : nx);
                if (gs)
                    e2d_copy_elem(c, gs, src_i - 1, j - 1, dst);
                else
                    memcpy(dst, w->ug + ((long)j * nxg + src_i) * E, sizeof(double) * E);
            }
        }
    }
    for (int i = 1; i <= nx; ++i) {
        for (int side = 2; side < 4; ++side) {
            int jg = side == 2 ? 0 : ny + 1;
            double *dst = w->ug + ((long)jg * nxg + i) * E;
            int bc = c->bc[side];
            if (bc == FRO_BC_FIXED) {
                for (int m = 0; m < 4; ++m)
                    for (int q = 0; q < np * np; ++q) dst[m * np * np + q] = c->fixed_state[side][m];
            } else {
                int src_j = bc == FRO_BC_PERIODIC ? (side == 2 ? ny : 1) : (side == 2 ? 1 : ny);
                if (gs)
                    e2d_copy_elem(c, gs, i - 1, src_j - 1, dst);
                else
                    memcpy(dst, w->ug + ((long)src_j * nxg + i) * E, sizeof(double) * E);
            }
        }
    }
}

/* Interface flux across a face with unit normal n (example
 * dev/parallelogram.jl:115-133): both states to the face frame (momentum along n
 * and along t = (-ny, nx)), the x-direction flux, back to the global frame. */
/* (inv(J) n)_comp for the face Jacobian J = Ji[i, j][f, pt] (2 x 2, column-major
 * entries of the host array Ji[nx, ny, 4, np, 2, 2]): inv(J) = [j11 -j01; -j10 j00] / det */
static double ji_dot(const fro_cfg *c, long i, long j, int f, long pt, double n0, double n1, int comp) {
    const long nx = c->nx, ny = c->ny, np = c->np;
    const long base = i + nx * (j + ny * (f + 4 * pt)), blk = nx * ny * 4 * np;
    const double j00 = c->Ji[base], j10 = c->Ji[base + blk], j01 = c->Ji[base + 2 * blk],
                 j11 = c->Ji[base + 3 * blk];
    const double det = j00 * j11 - j01 * j10;
    return comp == 0 ? (j11 * n0 - j01 * n1) / det : (j00 * n1 - j10 * n0) / det;
}

static void face_flux_n(const fro_cfg *c, const double *wL, const double *wR, double nx_, double ny_, double *fw) {
    double l[4], r[4], f[4];
    l[0] = wL[0]; l[1] = fma(wL[2], ny_, wL[1] * nx_); l[2] = fma(-wL[1], ny_, wL[2] * nx_); l[3] = wL[3];
    r[0] = wR[0]; r[1] = fma(wR[2], ny_, wR[1] * nx_); r[2] = fma(-wR[1], ny_, wR[2] * nx_); r[3] = wR[3];
    if (c->flux == FRO_FLUX_HLL)
        fro_flux_hll2d(l, r, c->gamma, 0, f);
    else
        fro_flux_lf2d(l, r, c->gamma, 0, f);
    fw[0] = f[0];
    fw[1] = fma(-f[2], ny_, f[1] * nx_);
    fw[2] = fma(f[1], ny_, f[2] * nx_);
    fw[3] = f[3];
}

/* FRO_FLUX_CENTRAL: the transformed-flux traces of the element at ghost-layer
 * coordinates (ig, jg); a ghost across a periodic side is its periodic partner
 * (across a Dirichlet side the trace is never used: zeros). */
static const double *central_fface(const fro_cfg *c, const e2d_work *w, int ig, int jg) {
    const int nx = c->nx, ny = c->ny, FS = 4 * w->np * 4;
    if (ig == 0 && c->bc[0] == FRO_BC_PERIODIC) ig = nx;
    if (ig == nx + 1 && c->bc[1] == FRO_BC_PERIODIC) ig = 1;
    if (jg == 0 && c->bc[2] == FRO_BC_PERIODIC) jg = ny;
    if (jg == ny + 1 && c->bc[3] == FRO_BC_PERIODIC) jg = 1;
    return w->fface + ((long)jg * w->nxg + ig) * FS;
}

static void rhs_euler2d(const fro_cfg *c, double *du, const double *u) {
    int nx = c->nx, ny = c->ny, np = c->np;
    double g = c->gamma;
    e2d_work w;
    w.nxg = nx + 2;
    w.nyg = ny + 2;
    w.np = np;
    w.E = 4 * np * np;
    long ng = (long)w.nxg * w.nyg;
    int FS = 4 * np * 4; /* per element face block: face, pt, m */
    w.ug = (double *)malloc(sizeof(double) * ng * w.E);
    w.uface = (double *)malloc(sizeof(double) * ng * FS);
    w.fface = (double *)calloc((size_t)ng * FS, sizeof(double));
    w.fvol = (double *)malloc(sizeof(double) * (long)nx * ny * 2 * w.E);
    w.fxi = (double *)malloc(sizeof(double) * (long)(nx + 1) * ny * np * 4);
    w.fyi = (double *)malloc(sizeof(double) * (long)nx * (ny + 1) * np * 4);
    e2d_fill_ghosts(c, u, &w);
    const double *ll = c->ll, *lr = c->lr, *lpdm = c->lpdm;
    int E = w.E, nxg = w.nxg;

    /* volume flux f = iJ * [F, G] (shock-vortex.jl:48-55) and face traces
     * of u (all elements incl. ghosts) and of the normal flux (interior),
     * shock-vortex.jl:57-71 */
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS schedule(static)
#endif
    for (long e = 0; e < ng; ++e) {
        int jg = (int)(e / nxg), ig = (int)(e % nxg);
        int interior = ig >= 1 && ig <= nx && jg >= 1 && jg <= ny;
        int needed = interior || ((ig >= 1 && ig <= nx) != (jg >= 1 && jg <= ny));
        if (!needed) continue;
        const double *ue = w.ug + e * E;
        double *uf = w.uface + e * FS;
        /* u traces: faces 0/2 along s at r-index l (points u[l, q]),
         * faces 1/3 along r at s-index l (points u[q, l]) */
        for (int m = 0; m < 4; ++m)
            for (int l = 0; l < np; ++l) {
                const double *us = ue + (m * np + 0) * np + l; /* stride np over q */
                const double *ur = ue + (m * np + l) * np;     /* stride 1 over q */
                uf[(0 * np + l) * 4 + m] = dotw(us, np, ll, 1, np);
                uf[(1 * np + l) * 4 + m] = dotw(ur, 1, lr, 1, np);
                uf[(2 * np + l) * 4 + m] = dotw(us, np, lr, 1, np);
                uf[(3 * np + l) * 4 + m] = dotw(ur, 1, ll, 1, np);
            }
        if (!interior) continue;
        long ei = (long)(jg - 1) * nx + (ig - 1);
        double *fv = w.fvol + ei * 2 * E;
        for (int l = 0; l < np; ++l)
            for (int k = 0; k < np; ++k) {
                double ww[4], F[4], G[4];
                for (int m = 0; m < 4; ++m) ww[m] = ue[(m * np + l) * np + k];
                euler_flux_dir(ww, g, 0, F, NULL, NULL);
                euler_flux_dir(ww, g, 1, G, NULL, NULL);
                if (c->iJ) {
                    /* f = a11 F + a12 G, g = a21 F + a22 G (shock-vortex.jl:52) */
                    const long nn = (long)nx * ny, blk = nn * np * np, at = ei + nn * (k + (long)np * l);
                    const double a11 = c->iJ[at], a21 = c->iJ[at + blk], a12 = c->iJ[at + 2 * blk],
                                 a22 = c->iJ[at + 3 * blk];
                    for (int m = 0; m < 4; ++m) {
                        fv[(0 * 4 + m) * np * np + l * np + k] = fma(G[m], a12, F[m] * a11);
                        fv[(1 * 4 + m) * np * np + l * np + k] = fma(G[m], a22, F[m] * a21);
                    }
                } else {
                    for (int m = 0; m < 4; ++m) {
                        fv[(0 * 4 + m) * np * np + l * np + k] = c->iJx * F[m];
                        fv[(1 * 4 + m) * np * np + l * np + k] = c->iJy * G[m];
                    }
                }
            }
        double *ff = w.fface + e * FS;
        for (int m = 0; m < 4; ++m)
            for (int l = 0; l < np; ++l) {
                const double *gs = fv + (1 * 4 + m) * np * np + l;      /* y flux at (k=l, l'=q), stride np */
                const double *fr = fv + (0 * 4 + m) * np * np + l * np; /* x flux at (k=q, l'=l), stride 1 */
                ff[(0 * np + l) * 4 + m] = dotw(gs, np, ll, 1, np);
                ff[(1 * np + l) * 4 + m] = dotw(fr, 1, lr, 1, np);
                ff[(2 * np + l) * 4 + m] = dotw(gs, np, lr, 1, np);
                ff[(3 * np + l) * 4 + m] = dotw(fr, 1, ll, 1, np);
            }
    }

    /* interface fluxes: x faces shock-vortex.jl:73-80, y faces :81-89 */
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS schedule(static)
#endif
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i <= nx; ++i) {
            const double *L = w.uface + ((long)(j + 1) * nxg + i) * FS;     /* element i-1 (ghost index i) */
            const double *R = w.uface + ((long)(j + 1) * nxg + i + 1) * FS; /* element i */
            for (int k = 0; k < np; ++k) {
                double *fw = w.fxi + (((long)j * (nx + 1) + i) * np + k) * 4;
                if (c->flux == FRO_FLUX_CENTRAL) {
                    /* dev/curve_euler.jl:93-104: 0.5 (f_face[i-1, j, 2] + f_face[i, j, 4]) (first
                     * component) - c (u_face[i, j, 4] - u_face[i-1, j, 2]) */
                    const double *fL = central_fface(c, &w, i, j + 1), *fR = central_fface(c, &w, i + 1, j + 1);
                    for (int m = 0; m < 4; ++m)
                        fw[m] = 0.5 * (fL[(1 * np + k) * 4 + m] + fR[(3 * np + k) * 4 + m]) -
                                c->flux_c * (R[(3 * np + k) * 4 + m] - L[(1 * np + k) * 4 + m]);
                } else if (c->iJ && c->n1) {
                    const long f = i + (long)(nx + 1) * j, nf = (long)(nx + 1) * ny;
                    face_flux_n(c, L + (1 * np + k) * 4, R + (3 * np + k) * 4, c->n1[f], c->n1[f + nf], fw);
                } else if (c->flux == FRO_FLUX_HLL)
                    fro_flux_hll2d(L + (1 * np + k) * 4, R + (3 * np + k) * 4, g, 0, fw);
                else
                    fro_flux_lf2d(L + (1 * np + k) * 4, R + (3 * np + k) * 4, g, 0, fw);
            }
        }
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS schedule(static)
#endif
    for (int j = 0; j <= ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const double *B = w.uface + ((long)j * nxg + i + 1) * FS;       /* element j-1 */
            const double *T = w.uface + ((long)(j + 1) * nxg + i + 1) * FS; /* element j */
            for (int k = 0; k < np; ++k) {
                double *fw = w.fyi + (((long)j * nx + i) * np + k) * 4;
                if (c->flux == FRO_FLUX_CENTRAL) {
                    /* dev/curve_euler.jl:106-117 (second component, faces 3 below and 1 above) */
                    const double *fB = central_fface(c, &w, i + 1, j), *fT = central_fface(c, &w, i + 1, j + 1);
                    for (int m = 0; m < 4; ++m)
                        fw[m] = 0.5 * (fB[(2 * np + k) * 4 + m] + fT[(0 * np + k) * 4 + m]) -
                                c->flux_c * (T[(0 * np + k) * 4 + m] - B[(2 * np + k) * 4 + m]);
                } else if (c->iJ && c->n2) {
                    const long f = i + (long)nx * j, nf = (long)nx * (ny + 1);
                    face_flux_n(c, B + (2 * np + k) * 4, T + (0 * np + k) * 4, c->n2[f], c->n2[f + nf], fw);
                } else if (c->flux == FRO_FLUX_HLL)
                    fro_flux_hll2d(B + (2 * np + k) * 4, T + (0 * np + k) * 4, g, 1, fw);
                else
                    fro_flux_lf2d(B + (2 * np + k) * 4, T + (0 * np + k) * 4, g, 1, fw);
            }
        }

    /* derivative (shock-vortex.jl:91-100) and combination (:102-115) */
    long nn = (long)nx * ny;
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS schedule(static)
#endif
    for (long ei = 0; ei < nn; ++ei) {
        int j = (int)(ei / nx), i = (int)(ei % nx);
        const double *fv = w.fvol + ei * 2 * E;
        const double *ff = w.fface + ((long)(j + 1) * nxg + i + 1) * FS;
        for (int m = 0; m < 4; ++m)
            for (int l = 0; l < np; ++l)
                for (int k = 0; k < np; ++k) {
                    double r1 = dotw(fv + (0 * 4 + m) * np * np + l * np, 1, lpdm + k, np, np);
                    double r2 = dotw(fv + (1 * 4 + m) * np * np + k, np, lpdm + l, np, np);
                    double fxl = w.fxi[(((long)j * (nx + 1) + i) * np + l) * 4 + m];
                    double fxr = w.fxi[(((long)j * (nx + 1) + i + 1) * np + l) * 4 + m];
                    double fyb = w.fyi[(((long)j * nx + i) * np + k) * 4 + m];
                    double fyt = w.fyi[(((long)(j + 1) * nx + i) * np + k) * 4 + m];
                    /* the x and y correction terms added to the two derivatives */
                    /* interface-flux scales: iJx, iJy; per point a11, a22 (shock-vortex.jl:104-111);
                     * with face normals (iJ n)_1 and (iJ n)_2 of each face (dev/parallelogram.jl:149-160) */
                    double sL = c->iJx, sR = c->iJx, sB = c->iJy, sT = c->iJy;
                    if (c->flux == FRO_FLUX_CENTRAL) {
                        /* the traces of the transformed flux enter unscaled; the elements
                         * along a Dirichlet side are not updated (dev/curve_euler.jl:119-149
                         * runs over the interior elements only) */
                        sL = sR = sB = sT = 1.0;
                        if ((i == 0 && c->bc[0] == FRO_BC_DIRICHLET) || (i == nx - 1 && c->bc[1] == FRO_BC_DIRICHLET) ||
                            (j == 0 && c->bc[2] == FRO_BC_DIRICHLET) || (j == ny - 1 && c->bc[3] == FRO_BC_DIRICHLET)) {
                            du[i + (long)nx * j + nn * (k + np * (l + (long)np * m))] = 0.0;
                            continue;
                        }
                    } else if (c->iJ) {
                        const long at = ei + nn * (k + (long)np * l), blk = nn * np * np;
                        const double a11 = c->iJ[at], a21 = c->iJ[at + blk], a12 = c->iJ[at + 2 * blk],
                                     a22 = c->iJ[at + 3 * blk];
                        sL = sR = a11;
                        sB = sT = a22;
                        if (c->n1) {
                            const long fl = i + (long)(nx + 1) * j, nf = (long)(nx + 1) * ny;
                            sL = fma(a12, c->n1[fl + nf], a11 * c->n1[fl]);
                            sR = fma(a12, c->n1[fl + 1 + nf], a11 * c->n1[fl + 1]);
                        }
                        if (c->n2) {
                            const long fb = i + (long)nx * j, nf = (long)nx * (ny + 1);
                            sB = fma(a22, c->n2[fb + nf], a21 * c->n2[fb]);
                            sT = fma(a22, c->n2[fb + nx + nf], a21 * c->n2[fb + nx]);
                        }
                        if (c->Ji && c->n1 && c->n2) {
                            /* dev/cylinder2.jl:147-150: (inv(Ji[i, j][f, pt]) n)_1 on the left (face 4)
                             * and right (face 2) faces at row l, (inv(Ji) n)_2 on the bottom (face 1)
                             * and top (face 3) faces at column k */
                            const long fl = i + (long)(nx + 1) * j, nfx = (long)(nx + 1) * ny;
                            const long fb = i + (long)nx * j, nfy = (long)nx * (ny + 1);
                            sL = ji_dot(c, i, j, 3, l, c->n1[fl], c->n1[fl + nfx], 0);
                            sR = ji_dot(c, i, j, 1, l, c->n1[fl + 1], c->n1[fl + 1 + nfx], 0);
                            sB = ji_dot(c, i, j, 0, k, c->n2[fb], c->n2[fb + nfy], 1);
                            sT = ji_dot(c, i, j, 2, k, c->n2[fb + nx], c->n2[fb + nx + nfy], 1);
                        }
                    }
                    double aL = fxl * sL - ff[(3 * np + l) * 4 + m];
                    double aR = fxr * sR - ff[(1 * np + l) * 4 + m];
                    double bB = fyb * sB - ff[(0 * np + k) * 4 + m];
                    double bT = fyt * sT - ff[(2 * np + k) * 4 + m];
                    double cx = fma(aR, c->dgr[k], fma(aL, c->dgl[k], r1));
                    double v = -fma(bT, c->dgr[l], fma(bB, c->dgl[l], cx + r2));
                    du[i + (long)nx * j + nn * (k + np * (l + (long)np * m))] = v;
                }
    }
    free(w.ug);
    free(w.uface);
    free(w.fface);
    free(w.fvol);
    free(w.fxi);
    free(w.fyi);
}

/* 1D1V BGK residual: mol! of example/bgk_wave.jl:69-129 (moments ->
 * conserve_prim(w, 3.0) -> maxwellian :76-81; f = v u / J :84-88;
 * interp_face! :99-101; kinetic upwind through f2e/e2f :103-107;
 * poly_derivative! :114-116; combination + relaxation (M - u)/tau
 * :122-128).  Periodic faces.  tau comes from the configuration (the
 * example hard-codes 1e-2 at :82). */
static void rhs_bgk1d(const fro_cfg *c, double *du, const double *u) {
    int ne = c->nx, nv = c->nvel, np = c->np;
    double *ffL = (double *)malloc(sizeof(double) * ne * nv); /* left-face trace of f */
    double *ffR = (double *)malloc(sizeof(double) * ne * nv); /* right-face trace */
#define UB(i, v, k) u[(i) + (long)ne * ((v) + (long)nv * (k))]
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS schedule(static)
#endif
    for (int i = 0; i < ne; ++i) {
        double J = c->J[i];
        for (int v = 0; v < nv; ++v) {
            double a = 0, b = 0;
            for (int k = 0; k < np; ++k) {
                double f = c->velo[v] * UB(i, v, k) / J;
                a += f * c->ll[k];
                b += f * c->lr[k];
            }
            ffL[i + ne * v] = a;
            ffR[i + ne * v] = b;
        }
    }
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS schedule(static)
#endif
    for (int i = 0; i < ne; ++i) {
        double J = c->J[i];
        int il = (i + ne - 1) % ne, ir = (i + 1) % ne;
        double *M = (double *)malloc(sizeof(double) * nv * np);
        for (int k = 0; k < np; ++k) {
            double w0 = 0, w1 = 0, w2 = 0;
            for (int v = 0; v < nv; ++v) {
                double x = UB(i, v, k);
                w0 += c->weights[v] * x;
                w1 += c->weights[v] * c->velo[v] * x;
                w2 += c->weights[v] * (c->velo[v] * c->velo[v]) * x;
            }
            w2 *= 0.5;
            /* conserve_prim(w, gamma = 3): lambda = 0.5 rho / (gamma-1) / (E - 0.5 m^2/rho);
             * closure 1, example/advection_kinetic.jl:80-86: rho = sum(u .* weights),
             * prim = [rho, a, 1] */
            double rho = w0, U = c->bgk_closure ? c->a : w1 / w0;
            double lam = c->bgk_closure ? 1.0 : 0.5 * w0 / (3.0 - 1.0) / (w2 - 0.5 * w1 * w1 / w0);
            for (int v = 0; v < nv; ++v) {
                double dv = c->velo[v] - U;
                M[v + nv * k] = rho * sqrt(lam / M_PI) * exp(-lam * dv * dv);
            }
        }
        for (int v = 0; v < nv; ++v) {
            double vel = c->velo[v];
            double delta = vel > 0.0 ? 1.0 : 0.0; /* heaviside */
            /* face left of i: upwind between right trace of il and left trace of i */
            double fl = ffL[i + ne * v] * (1.0 - delta) + ffR[il + ne * v] * delta;
            double fr = ffL[ir + ne * v] * (1.0 - delta) + ffR[i + ne * v] * delta;
            for (int m = 0; m < np; ++m) {
                double r = 0.0;
                for (int k = 0; k < np; ++k) r += (vel * UB(i, v, k) / J) * c->lpdm[m + np * k];
                du[i + (long)ne * (v + (long)nv * m)] =
                    -(r + (fl - ffL[i + ne * v]) * c->dgl[m] + (fr - ffR[i + ne * v]) * c->dgr[m]) +
                    (M[v + nv * m] - UB(i, v, m)) / c->tau;
            }
        }
        free(M);
    }
#undef UB
    free(ffL);
    free(ffR);
}

void fro_rhs(const fro_cfg *c, double *du, const double *u) {
    switch (c->kind) {
    case FRO_ADVECTION:
    case FRO_BURGERS: rhs_scalar1d(c, du, u); break;
    case FRO_EULER1D: rhs_euler1d(c, du, u); break;
    case FRO_EULER2D: rhs_euler2d(c, du, u); break;
    case FRO_BGK1D: rhs_bgk1d(c, du, u); break;
    }
}

/* SSPRK3 in Shu-Osher form (OrdinaryDiffEq SSPRK33; the stepping the
 * reference's examples hand to OrdinaryDiffEq's init/step!):
 *   u1 = u + dt L(u);  u2 = (3u + u1 + dt L(u1))/4;  u' = (u + 2 u2 + 2 dt L(u2))/3 */
void fro_ssprk3(const fro_cfg *c, double *u, double dt, int nsteps, double *work) {
    long n = fro_ndof(c);
    double *s = work, *k = work + n;
    const double third = 1.0 / 3.0;
    fro_cfg cl = *c; /* the later stages: ghosts from u^n when refreshed once per step */
    cl.ghost_src = c->kind == FRO_EULER2D && c->ghosts_per_step ? u : NULL;
    for (int it = 0; it < nsteps; ++it) {
        fro_rhs(c, k, u);
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS schedule(static)
#endif
        for (long q = 0; q < n; ++q) s[q] = fma(dt, k[q], u[q]);
        fro_rhs(&cl, k, s);
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS schedule(static)
#endif
        for (long q = 0; q < n; ++q) s[q] = fma(dt, k[q], fma(3.0, u[q], s[q])) * 0.25;
        fro_rhs(&cl, k, s);
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS schedule(static)
#endif
        for (long q = 0; q < n; ++q) u[q] = fma(2.0 * dt, k[q], fma(2.0, s[q], u[q])) * third;
    }
}

/* The time loop of example/shock-vortex.jl:294-321 with SSPRK3 in place of
 * Midpoint: nsteps of (one SSPRK3 step, then the indicator + :l2 filter of
 * fro_filter2d on every element).  work holds 2 * ndof doubles. */
void fro_ssprk3_filtered(const fro_cfg *c, double *u, double dt, int nsteps, double *work, const double *V,
                         const double *iV, double lam, double S0, double kappa) {
    for (int it = 0; it < nsteps; ++it) {
        fro_ssprk3(c, u, dt, 1, work);
        fro_filter2d(c, u, V, iV, lam, S0, kappa, NULL);
    }
}

/* Explicit Runge-Kutta with a Butcher tableau (OrdinaryDiffEq's fixed-step
 * explicit methods: Midpoint, Heun, RK4, Tsit5, ...): per step and stage i,
 * acc = sum over j < i with a_ij != 0, in ascending j, as the fma chain
 * acc = a_ij0 k_j0; acc = fma(a_ij, k_j, acc); stage = fma(dt, acc, u) (u when
 * no a_ij is nonzero); k_i = rhs(stage); then u = fma(dt, acc_b, u) with the b
 * weights.  A is s x s row-major; work holds (s + 1) * ndof doubles. */
void fro_erk(const fro_cfg *c, double *u, double dt, int nsteps, int s, const double *A, const double *b,
             double *work) {
    long n = fro_ndof(c);
    double *st = work, *k = work + n;
    /* ghosts refreshed once per step: the stages after the first take them from u^n */
    fro_cfg cl = *c;
    cl.ghost_src = c->kind == FRO_EULER2D && c->ghosts_per_step ? u : NULL;
    for (int it = 0; it < nsteps; ++it) {
        for (int i = 0; i < s; ++i) {
            int first = 1;
            for (int j = 0; j < i; ++j) {
                const double a = A[i * s + j];
                if (a == 0.0) continue;
                for (long q = 0; q < n; ++q) st[q] = first ? a * k[j * n + q] : fma(a, k[j * n + q], st[q]);
                first = 0;
            }
            if (first)
                fro_rhs(c, k + i * n, u);
            else {
                for (long q = 0; q < n; ++q) st[q] = fma(dt, st[q], u[q]);
                fro_rhs(&cl, k + i * n, st);
            }
        }
        int first = 1;
        for (int j = 0; j < s; ++j) {
            if (b[j] == 0.0) continue;
            for (long q = 0; q < n; ++q) st[q] = first ? b[j] * k[j * n + q] : fma(b[j], k[j * n + q], st[q]);
            first = 0;
        }
        if (!first)
            for (long q = 0; q < n; ++q) u[q] = fma(dt, st[q], u[q]);
    }
}

/* Stabilised step (the recurrence + finishing structure of OrdinaryDiffEq's
 * ROCK2/ROCK4 and of RKC, as example/advection_kinetic.jl:133-146 steps with
 * ROCK4), restated in increment form: D_0 = 0, Y_j = u + D_j,
 *   D_j = alpha_j D_{j-1} + beta_j D_{j-2} + dt (mu_j f(Y_{j-1}) + delta_j f(u)),
 * with the operations in this order: t = mu F; t = fma(delta, F0, t) if
 * delta != 0; t = dt t; t = fma(beta, D_{j-2}, t) if j >= 3 and beta != 0;
 * t = fma(alpha, D_{j-1}, t) if j >= 2 and alpha != 0.  Finishing stages from
 * Y_m: input u + fma(dt, acc, D_m) (Y_m for a zero row), the step
 * u + fma(dt, acc_b, D_m) (u + D_m without weights).  acc is the chain of erk
 * (first nonzero term a k, then fma).  work: (7 + sf) * ndof doubles. */
void fro_rock(const fro_cfg *c, double *u, double dt, int nsteps, int m, const double *alpha, const double *beta,
              const double *mu, const double *delta, int sf, const double *A, const double *b, double *work) {
    long n = fro_ndof(c);
    double *D[3] = {work, work + n, work + 2 * n};
    double *F0 = work + 3 * n, *F = work + 4 * n, *Y = work + 5 * n, *S = work + 6 * n, *K = work + 7 * n;
    fro_cfg cl = *c; /* stage inputs: ghosts from u^n when refreshed once per step */
    cl.ghost_src = c->kind == FRO_EULER2D && c->ghosts_per_step ? u : NULL;
    for (int it = 0; it < nsteps; ++it) {
        fro_rhs(c, F0, u);
        for (int j = 1; j <= m; ++j) {
            if (j >= 2) fro_rhs(&cl, F, Y);
            const double *Fj = j == 1 ? F0 : F;
            const double al = alpha[j - 1], be = beta[j - 1], mj = mu[j - 1], de = delta[j - 1];
            double *Dj = D[j % 3];
            const double *D1 = D[(j - 1) % 3], *D2 = D[(j + 1) % 3];
            for (long q = 0; q < n; ++q) {
                double t = mj * Fj[q];
                if (de != 0.0) t = fma(de, F0[q], t);
                t = dt * t;
                if (j >= 3 && be != 0.0) t = fma(be, D2[q], t);
                if (j >= 2 && al != 0.0) t = fma(al, D1[q], t);
                Dj[q] = t;
                Y[q] = u[q] + t;
            }
        }
        const double *Dm = D[m % 3];
        for (int i = 0; i < sf; ++i) {
            int first = 1;
            for (int l = 0; l < i; ++l) {
                const double a = A[i * sf + l];
                if (a == 0.0) continue;
                for (long q = 0; q < n; ++q) S[q] = first ? a * K[l * n + q] : fma(a, K[l * n + q], S[q]);
                first = 0;
            }
            if (first)
                fro_rhs(&cl, K + i * n, Y);
            else {
                for (long q = 0; q < n; ++q) S[q] = u[q] + fma(dt, S[q], Dm[q]);
                fro_rhs(&cl, K + i * n, S);
            }
        }
        int first = 1;
        for (int i = 0; i < sf; ++i) {
            if (b[i] == 0.0) continue;
            for (long q = 0; q < n; ++q) S[q] = first ? b[i] * K[i * n + q] : fma(b[i], K[i * n + q], S[q]);
            first = 0;
        }
        for (long q = 0; q < n; ++q) u[q] = u[q] + (first ? Dm[q] : fma(dt, S[q], Dm[q]));
    }
}

static double norm2_diff(const double *x, const double *y, long n) {
    double t = 0.0;
    for (long q = 0; q < n; ++q) {
        double d = y ? x[q] - y[q] : x[q];
        t = fma(d, d, t);
    }
    return sqrt(t);
}

/* Nonlinear power method of the RKC code (Sommeijer, Shampine, Verwer, J.
 * Comput. Appl. Math. 88 (1997) 315-326), the spectral-radius estimate of the
 * ROCK methods: v = u + dynrm d/|d| (dynrm = |u| sqrt(eps)), sigma =
 * |f(v) - f(u)| / dynrm, v <- u + (f(v) - f(u)) dynrm / |f(v) - f(u)| until
 * sigma changes by at most 1 %; rho = 1.2 sigma.  dir (ndof) holds the start
 * direction when *have is set and receives v - u; work: 3 * ndof doubles.
 * Returns the iterations used (negative when not settled). */
int fro_spectral_radius(const fro_cfg *c, const double *u, int maxiter, double *dir, int *have, double *rho,
                        double *work) {
    long n = fro_ndof(c);
    double *v = work, *fu = work + n, *fv = work + 2 * n;
    const double uround = 0x1p-53, sq = sqrt(uround);
    fro_rhs(c, fu, u);
    const double *d0 = *have ? dir : fu;
    double ynrm = norm2_diff(u, NULL, n), vnrm = norm2_diff(d0, NULL, n), dynrm;
    if (ynrm != 0.0 && vnrm != 0.0) {
        dynrm = ynrm * sq;
        for (long q = 0; q < n; ++q) v[q] = u[q] + (dynrm / vnrm) * d0[q];
    } else if (ynrm != 0.0) {
        dynrm = ynrm * sq;
        for (long q = 0; q < n; ++q) v[q] = u[q] + sq * u[q];
    } else if (vnrm != 0.0) {
        dynrm = uround;
        for (long q = 0; q < n; ++q) v[q] = u[q] + (dynrm / vnrm) * d0[q];
    } else {
        dynrm = uround;
        for (long q = 0; q < n; ++q) v[q] = dynrm / sqrt((double)n);
    }
    double sigma = 0.0;
    int it = 1, converged = 0;
    for (; it <= maxiter; ++it) {
        fro_rhs(c, fv, v);
        double dfnrm = norm2_diff(fv, fu, n);
        double sigmal = sigma;
        sigma = dfnrm / dynrm;
        if (it >= 2 && fabs(sigma - sigmal) <= fmax(sigma, 1e-300) * 0.01) {
            converged = 1;
            break;
        }
        if (it == maxiter) break;
        if (dfnrm != 0.0) {
            for (long q = 0; q < n; ++q) v[q] = u[q] + (dynrm / dfnrm) * (fv[q] - fu[q]);
        } else {
            long i = it % n;
            v[i] = u[i] - (v[i] - u[i]);
        }
    }
    for (long q = 0; q < n; ++q) dir[q] = v[q] - u[q];
    *have = 1;
    *rho = 1.2 * sigma;
    return converged ? it : -it;
}

/* ------------------------------------------------------------------------
 * Troubled-cell indicator and modal filter
 * ---------------------------------------------------------------------- */

/* KitBase :l2 modal filter on a flat modal vector (as called on the
 * flattened 2D modes at example/shock-vortex.jl:316):
 * u[q] /= 1 + lam (q+1)^2 q^2, q = 0-based mode index. */
static void filter_l2_flat(double *uh, int n, double lam) {
    for (int q = 0; q < n; ++q) uh[q] = uh[q] / (1.0 + lam * (double)((q + 1) * (q + 1) * q * q));
}

/* y = A x for a column-major n x n matrix, fixed dot order */
static void matvec(const double *A, const double *x, int n, double *y) {
    for (int a = 0; a < n; ++a) y[a] = dotw(A + a, n, x, 1, n);
}

/* the modal-decay detector input su = uh_N^2 / (sum uh^2 + add) */
static double decay_ratio(const double *uh, int n, double add) {
    double tot = 0.0;
    for (int a = 0; a < n; ++a) tot = fma(uh[a], uh[a], tot);
    return uh[n - 1] * uh[n - 1] / (tot + add);
}

/* filter one element's nvar variables (point stride ps, variable stride vs) */
static void filter_element(double *u, long ps, long vs, int nvar, int n, const double *V, const double *iV,
                           double lam) {
    double ue[36], uh[36];
    for (int m = 0; m < nvar; ++m) {
        for (int q = 0; q < n; ++q) ue[q] = u[ps * q + vs * m];
        matvec(iV, ue, n, uh);
        filter_l2_flat(uh, n, lam);
        matvec(V, uh, n, ue);
        for (int q = 0; q < n; ++q) u[ps * q + vs * m] = ue[q];
    }
}

/* Post-step indicator + filter, example/shock-vortex.jl:308-321 (over the
 * full np x np block; the example hard-codes 1:3, i.e. p = 2). */
int fro_filter2d(const fro_cfg *c, double *u, const double *V, const double *iV, double lam, double S0,
                 double kappa, int *flags) {
    int nx = c->nx, ny = c->ny, np = c->np, N = np * np;
    long nn = (long)nx * ny;
    int count = 0;
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS reduction(+ : count) schedule(static)
#endif
    for (long e = 0; e < nn; ++e) {
        double ue[36], uh[36];
        for (int q = 0; q < N; ++q) ue[q] = u[e + nn * q];
        matvec(iV, ue, N, uh);
        double su = decay_ratio(uh, N, 0.0);
        int troubled = fro_shock_detector(log10(su), np - 1, S0, kappa);
        if (flags) flags[e] = troubled;
        if (!troubled) continue;
        ++count;
        filter_element(u + e, nn, nn * N, 4, N, V, iV, lam);
    }
    return count;
}

/* 1D indicator + filter, example/euler_highlevel.jl:37-52:
 * su = u_N^2 / (sum u^2 + 1e-6), shock_detector(log10(su), deg) with the
 * default S0 = -3 log10(deg), kappa = 4. */
int fro_filter1d(const fro_cfg *c, double *u, int nvar, const double *V, const double *iV, double lam,
                 int *flags) {
    int ne = c->nx, np = c->np, deg = np - 1;
    int count = 0;
    for (int i = 0; i < ne; ++i) {
        double ue[8], uh[8];
        for (int q = 0; q < np; ++q) ue[q] = u[i + (long)ne * q];
        matvec(iV, ue, np, uh);
        double su = decay_ratio(uh, np, 1e-6);
        int troubled = fro_shock_detector(log10(su), deg, -3.0 * log10((double)deg), 4.0);
        if (flags) flags[i] = troubled;
        if (!troubled) continue;
        ++count;
        filter_element(u + i, ne, (long)ne * np, nvar, np, V, iV, lam);
    }
    return count;
}

/* ------------------------------------------------------------------------
 * Positivity-preserving limiter, src/dissipation.jl:38-216 (Vandenhoeck & Lani
 * 2019).  Per element: the weighted mean u_mean (weights summing to 1), the
 * face traces, eps = min(1e-13, rho_mean, p_mean), the density scaling
 * t1 = min((rho_mean - eps) / (rho_mean - rho_min + 1e-8), 1) over the solution
 * and face points, applied to the density; then for every face point (from
 * the state before the density scaling, as the reference does) and every
 * solution point whose lambda = rho / (2 p) falls below eps, the t at which
 * p(t (u - u_mean) + u_mean) = eps, and all variables scaled by
 * t2 = min(t_j, t0).  The reference takes min(tj, t0) with a call that throws
 * whenever any t_j exists; this restatement defines it as the minimum, and
 * solves p(t) = eps in closed form (p rho is quadratic in t) instead of the
 * reference's Newton iteration from t = 1: the root in [0, 1] nearest to 1.
 * Every dot product is the fma chain of dotw.  Return value: 1 when the
 * element was scaled with t1 < 1 or t2 < 1, 0 otherwise, -1 when t1 left
 * (0, 1] (the reference's assertion).
 * ---------------------------------------------------------------------- */

/* root in [0, 1] nearest to 1 of a t^2 + b t + c (c >= 0 at t = 0); 1 if none */
static double limiter_root(double a, double b, double c) {
    double r = 1.0;
    if (fabs(a) <= 1e-300) {
        if (b != 0.0) r = -c / b;
    } else {
        const double disc = b * b - 4.0 * a * c;
        if (disc >= 0.0) {
            const double q = -0.5 * (b + copysign(sqrt(disc), b));
            const double r1 = q / a, r2 = q != 0.0 ? c / q : r1;
            const int ok1 = r1 >= 0.0 && r1 <= 1.0, ok2 = r2 >= 0.0 && r2 <= 1.0;
            if (ok1 && ok2) r = r1 > r2 ? r1 : r2;
            else if (ok1) r = r1;
            else if (ok2) r = r2;
        }
    }
    return r < 0.0 ? 0.0 : (r > 1.0 ? 1.0 : r);
}

/* t with p(t) = eps on the segment from the mean um to the state w (nv = 3:
 * 1D, nv = 4: 2D): (g - 1)(2 E rho - |m|^2) - 2 eps rho = a t^2 + b t + c */
static double limiter_t(const double *w, const double *um, int nv, double g, double eps) {
    const double gm1 = g - 1.0;
    const int ie = nv - 1;
    const double dr = w[0] - um[0], de = w[ie] - um[ie];
    double dm2 = 0.0, mdm = 0.0, mm = 0.0;
    for (int v = 1; v < ie; ++v) {
        const double dm = w[v] - um[v];
        dm2 = fma(dm, dm, dm2);
        mdm = fma(um[v], dm, mdm);
        mm = fma(um[v], um[v], mm);
    }
    const double a = gm1 * (2.0 * de * dr - dm2);
    const double b = gm1 * (2.0 * (um[ie] * dr + de * um[0]) - 2.0 * mdm) - 2.0 * eps * dr;
    const double c = gm1 * (2.0 * um[ie] * um[0] - mm) - 2.0 * eps * um[0];
    return limiter_root(a, b, c);
}

/* lambda = rho / (2 p) of a conserved state (nv = 3 or 4), conserve_prim's last entry */
static double limiter_lambda(const double *w, int nv, double g) {
    double kin = 0.0;
    for (int v = 1; v < nv - 1; ++v) kin = fma(w[v], w[v], kin);
    return 0.5 * w[0] / (g - 1.0) / (w[nv - 1] - 0.5 * kin / w[0]);
}

/* One Euler element: value (q, v) at u[q * sq + v * sv], nq points with weights
 * wq; nface face points whose traces are the dot products of the state along
 * the face lines: face point f takes the np values u[fb[f] + r * fs[f]] with
 * weights fw[f][r]. */
static int limit_euler_element(double *u, long sq, long sv, int nq, int nv, const double *wq, int nface,
                               const long *fb, const long *fs, const double *const *fw, int np, double g, double t0) {
    double um[4], wb[24][4];
    for (int v = 0; v < nv; ++v) um[v] = dotw(u + v * sv, sq, wq, 1, nq);
    double lm = limiter_lambda(um, nv, g);
    const double pm = 0.5 * um[0] * (1.0 / lm);
    double eps = 1e-13;
    if (um[0] < eps) eps = um[0];
    if (pm < eps) eps = pm;
    double rmin = INFINITY;
    for (int f = 0; f < nface; ++f) {
        for (int v = 0; v < nv; ++v) wb[f][v] = dotw(u + fb[f] + v * sv, fs[f], fw[f], 1, np);
        if (wb[f][0] < rmin) rmin = wb[f][0];
    }
    for (int q = 0; q < nq; ++q)
        if (u[q * sq] < rmin) rmin = u[q * sq];
    double t1 = (um[0] - eps) / (um[0] - rmin + 1e-8);
    if (t1 > 1.0) t1 = 1.0;
    if (!(t1 > 0.0)) return -1;
    for (int q = 0; q < nq; ++q) u[q * sq] = t1 * (u[q * sq] - um[0]) + um[0];
    double t2 = t0;
    int found = 0;
    for (int f = 0; f < nface; ++f)
        if (limiter_lambda(wb[f], nv, g) < eps) {
            const double t = limiter_t(wb[f], um, nv, g, eps);
            if (t < t2) t2 = t;
            found = 1;
        }
    for (int q = 0; q < nq; ++q) {
        double w[4];
        for (int v = 0; v < nv; ++v) w[v] = u[q * sq + v * sv];
        if (limiter_lambda(w, nv, g) < eps) {
            const double t = limiter_t(w, um, nv, g, eps);
            if (t < t2) t2 = t;
            found = 1;
        }
    }
    if (found)
        for (int v = 0; v < nv; ++v)
            for (int q = 0; q < nq; ++q) u[q * sq + v * sv] = t2 * (u[q * sq + v * sv] - um[v]) + um[v];
    return (t1 < 1.0 || (found && t2 < 1.0)) ? 1 : 0;
}

int fro_positive_limiter2d(const fro_cfg *c, double *u, const double *w, double t0) {
    const int np = c->np, nq = np * np;
    const long nn = (long)c->nx * c->ny;
    int count = 0, bad = 0;
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS reduction(+ : count, bad) schedule(static)
#endif
    for (long e = 0; e < nn; ++e) {
        /* face points, in the reference's order (dissipation.jl:143-161):
         * bottom (column j along s, ll), right (row j along r, lr), top
         * (column j, lr), left (row j, ll) for j = 0..np-1 */
        long fb[24], fs[24];
        const double *fw[24];
        int f = 0;
        for (int j = 0; j < np; ++j) {
            fb[f] = nn * j; fs[f] = nn * np; fw[f++] = c->ll;
            fb[f] = nn * (np * j); fs[f] = nn; fw[f++] = c->lr;
            fb[f] = nn * j; fs[f] = nn * np; fw[f++] = c->lr;
            fb[f] = nn * (np * j); fs[f] = nn; fw[f++] = c->ll;
        }
        const int r = limit_euler_element(u + e, nn, nn * nq, nq, 4, w, f, fb, fs, fw, np, c->gamma, t0);
        if (r < 0) ++bad;
        else count += r;
    }
    return bad ? -bad : count;
}

int fro_positive_limiter1d(const fro_cfg *c, double *u, const double *w, double t0) {
    const int np = c->np, ne = c->nx;
    int count = 0, bad = 0;
    for (int i = 0; i < ne; ++i) {
        long fb[2] = {0, 0}, fs[2] = {ne, ne};
        const double *fw[2] = {c->ll, c->lr};
        const int r = limit_euler_element(u + i, ne, (long)ne * np, np, 3, w, 2, fb, fs, fw, np, c->gamma, t0);
        if (r < 0) ++bad;
        else count += r;
    }
    return bad ? -bad : count;
}

/* scalar form, dissipation.jl:38-58: mean = sum(u w) / sum(w), theta over the
 * two face traces and the solution points */
int fro_positive_limiter_scalar(const fro_cfg *c, double *u, const double *w, double t0) {
    (void)t0; /* the reference's scalar form accepts t0 and does not use it */
    const int np = c->np, ne = c->nx;
    int count = 0, bad = 0;
    double sw = w[0];
    for (int q = 1; q < np; ++q) sw += w[q];
    for (int i = 0; i < ne; ++i) {
        double *ue = u + i;
        const double um = dotw(ue, ne, w, 1, np) / sw;
        const double ub0 = dotw(ue, ne, c->ll, 1, np), ub1 = dotw(ue, ne, c->lr, 1, np);
        double eps = 1e-13;
        if (um < eps) eps = um;
        double th = ub0 < ub1 ? ub0 : ub1;
        for (int q = 0; q < np; ++q)
            if (ue[(long)ne * q] < th) th = ue[(long)ne * q];
        double t = (um - eps) / (um - th + 1e-8);
        if (t > 1.0) t = 1.0;
        if (!(t > 0.0)) {
            ++bad;
            continue;
        }
        for (int q = 0; q < np; ++q) ue[(long)ne * q] = t * (ue[(long)ne * q] - um) + um;
        count += t < 1.0;
    }
    return bad ? -bad : count;
}

/* Learned-indicator inputs: per element the normalised modal energies of
 * density and pressure, x_q = clamp(log10(uh_q^2 / sum uh^2 + 1e-16), -16, 0)/8 + 1. */
void fro_modal_features2d(const fro_cfg *c, const double *u, const double *iV, double *feat) {
    int nx = c->nx, ny = c->ny, np = c->np, N = np * np;
    long nn = (long)nx * ny;
    double g = c->gamma;
    for (long e = 0; e < nn; ++e) {
        double ue[2][36], uh[36];
        for (int q = 0; q < N; ++q) {
            double w[4];
            for (int m = 0; m < 4; ++m) w[m] = u[e + nn * (q + (long)N * m)];
            double rinv = 1.0 / w[0];
            double U = w[1] * rinv, Vv = w[2] * rinv;
            ue[0][q] = w[0];
            ue[1][q] = (g - 1.0) * (w[3] - 0.5 * (w[1] * U + w[2] * Vv));
        }
        for (int v = 0; v < 2; ++v) {
            double tot = 0;
            for (int a = 0; a < N; ++a) {
                double s = 0;
                for (int b = 0; b < N; ++b) s += iV[a + N * b] * ue[v][b];
                uh[a] = s * s;
                tot += uh[a];
            }
            for (int a = 0; a < N; ++a) {
                double x = log10(uh[a] / tot + 1e-16);
                if (x < -16.0) x = -16.0;
                if (x > 0.0) x = 0.0;
                feat[e * 2 * N + v * N + a] = x / 8.0 + 1.0;
            }
        }
    }
}

/* Features of the 1D learned indicator of a scalar state u[ne, np] (32 per
 * element): slots 0..np-1 the normalised modal energies as in the 2D form,
 * slot 8 + deg - 1 a degree one-hot, slot 16 the energy level
 * clamp(log10(sum u_hat^2 + 1e-30) + 6, -8, 8) / 8, other slots 0.  The modes
 * are u_hat = iV u of the indicator of example/euler_highlevel.jl:37-40. */
void fro_modal_features1d(const fro_cfg *c, const double *u, const double *iV, double *feat) {
    int ne = c->nx, np = c->np;
    for (long e = 0; e < ne; ++e) {
        double uh[8], tot = 0.0;
        for (int a = 0; a < np; ++a) {
            double s = 0.0;
            for (int b = 0; b < np; ++b) s += iV[a + np * b] * u[e + (long)ne * b];
            uh[a] = s;
            tot += s * s;
        }
        double *row = feat + e * 32;
        for (int q = 0; q < 32; ++q) row[q] = 0.0;
        for (int a = 0; a < np; ++a) {
            double x = log10(uh[a] * uh[a] / tot + 1e-16);
            if (x < -16.0) x = -16.0;
            if (x > 0.0) x = 0.0;
            row[a] = x / 8.0 + 1.0;
        }
        row[8 + np - 2] = 1.0;
        double lv = log10(tot + 1e-30) + 6.0;
        if (lv < -8.0) lv = -8.0;
        if (lv > 8.0) lv = 8.0;
        row[16] = lv / 8.0;
    }
}

/* ------------------------------------------------------------------------
 * Reductions and norms
 * ---------------------------------------------------------------------- */

void fro_conserved_sums2d(const fro_cfg *c, const double *u, const double *wp, double *sums) {
    int np = c->np, N = np * np;
    long nn = (long)c->nx * c->ny;
    double area = 1.0 / (c->iJx * c->iJy); /* dx dy / 4 per unit reference weight */
    for (int m = 0; m < 4; ++m) {
        double s = 0.0;
        for (int q = 0; q < N; ++q) {
            double t = 0.0;
            for (long e = 0; e < nn; ++e) t += u[e + nn * (q + (long)N * m)];
            s += wp[q] * t;
        }
        sums[m] = s * area;
    }
}

double fro_max_speed2d(const fro_cfg *c, const double *u) {
    long n = (long)c->nx * c->ny * c->np * c->np;
    double g = c->gamma, mx = 0.0;
    for (long q = 0; q < n; ++q) {
        double w[4] = {u[q], u[q + n], u[q + 2 * n], u[q + 3 * n]};
        double U = w[1] / w[0], V = w[2] / w[0];
        double p = (g - 1.0) * (w[3] - 0.5 * (w[1] * U + w[2] * V));
        double cs = sqrt(g * p / w[0]);
        double s = fmax(fabs(U) + cs, fabs(V) + cs);
        if (s > mx) mx = s;
    }
    return mx;
}

/* L1_error / L2_error / Linf_error, src/tools.jl:43-53 (note dx inside the
 * square for L2) */
double fro_L1_error(const double *u, const double *ue, long n, double dx) {
    double s = 0;
    for (long i = 0; i < n; ++i) s += fabs(u[i] - ue[i]) * dx;
    return s;
}
double fro_L2_error(const double *u, const double *ue, long n, double dx) {
    double s = 0;
    for (long i = 0; i < n; ++i) {
        double t = fabs(u[i] - ue[i]) * dx;
        s += t * t;
    }
    return sqrt(s);
}
double fro_Linf_error(const double *u, const double *ue, long n, double dx) {
    double s = 0;
    for (long i = 0; i < n; ++i) {
        double t = fabs(u[i] - ue[i]) * dx;
        if (t > s) s = t;
    }
    return s;
}

/* ------------------------------------------------------------------------
 * Learned indicator, FP64 reference for the GPU kernels' gradients
 * ---------------------------------------------------------------------- */

/* GELU in its tanh form (Hendrycks and Gimpel, arXiv:1606.08415) */
static double gelu(double x) {
    const double c = sqrt(2.0 / M_PI), a = 0.044715;
    return 0.5 * x * (1.0 + tanh(c * (x + a * x * x * x)));
}
static double dgelu(double x) {
    const double c = sqrt(2.0 / M_PI), a = 0.044715;
    const double t = tanh(c * (x + a * x * x * x));
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * c * (1.0 + 3.0 * a * x * x);
}

void fro_mlp_forward(const double *P, const double *x, int n, int nin, int nh, double *y) {
    const double *W1 = P, *b1 = W1 + nh * nin, *W2 = b1 + nh, *b2 = W2 + nh * nh, *W3 = b2 + nh,
                 *b3 = W3 + nh;
    double *h1 = (double *)malloc(sizeof(double) * nh * 2), *h2 = h1 + nh;
    for (int s = 0; s < n; ++s) {
        const double *xs = x + (long)s * nin;
        for (int o = 0; o < nh; ++o) {
            double a = b1[o];
            for (int i = 0; i < nin; ++i) a += W1[o * nin + i] * xs[i];
            h1[o] = gelu(a);
        }
        for (int o = 0; o < nh; ++o) {
            double a = b2[o];
            for (int i = 0; i < nh; ++i) a += W2[o * nh + i] * h1[i];
            h2[o] = gelu(a);
        }
        double a = b3[0];
        for (int i = 0; i < nh; ++i) a += W3[i] * h2[i];
        y[s] = 1.0 / (1.0 + exp(-a));
    }
    free(h1);
}

double fro_mlp_loss_grad(const double *P, const double *x, const double *label, int n, int nin, int nh,
                         double *grad) {
    const double *W1 = P, *b1 = W1 + nh * nin, *W2 = b1 + nh, *b2 = W2 + nh * nh, *W3 = b2 + nh,
                 *b3 = W3 + nh;
    long np_ = (long)nh * nin + nh + (long)nh * nh + nh + nh + 1;
    memset(grad, 0, sizeof(double) * np_);
    double *gW1 = grad, *gb1 = gW1 + nh * nin, *gW2 = gb1 + nh, *gb2 = gW2 + nh * nh, *gW3 = gb2 + nh,
           *gb3 = gW3 + nh;
    double *buf = (double *)malloc(sizeof(double) * nh * 6);
    double *a1 = buf, *h1 = buf + nh, *a2 = buf + 2 * nh, *h2 = buf + 3 * nh, *d2 = buf + 4 * nh,
           *d1 = buf + 5 * nh;
    double loss = 0.0;
    for (int s = 0; s < n; ++s) {
        const double *xs = x + (long)s * nin;
        for (int o = 0; o < nh; ++o) {
            double a = b1[o];
            for (int i = 0; i < nin; ++i) a += W1[o * nin + i] * xs[i];
            a1[o] = a;
            h1[o] = gelu(a);
        }
        for (int o = 0; o < nh; ++o) {
            double a = b2[o];
            for (int i = 0; i < nh; ++i) a += W2[o * nh + i] * h1[i];
            a2[o] = a;
            h2[o] = gelu(a);
        }
        double a3 = b3[0];
        for (int i = 0; i < nh; ++i) a3 += W3[i] * h2[i];
        double y = 1.0 / (1.0 + exp(-a3));
        double t = label[s];
        double ye = fmin(fmax(y, 1e-12), 1.0 - 1e-12);
        loss += -(t * log(ye) + (1.0 - t) * log(1.0 - ye));
        double g3 = (y - t) / n; /* d loss / d a3 for sigmoid + BCE, mean */
        gb3[0] += g3;
        for (int i = 0; i < nh; ++i) {
            gW3[i] += g3 * h2[i];
            d2[i] = g3 * W3[i] * dgelu(a2[i]);
        }
        for (int o = 0; o < nh; ++o) {
            gb2[o] += d2[o];
            for (int i = 0; i < nh; ++i) gW2[o * nh + i] += d2[o] * h1[i];
        }
        for (int i = 0; i < nh; ++i) {
            double s2 = 0.0;
            for (int o = 0; o < nh; ++o) s2 += d2[o] * W2[o * nh + i];
            d1[i] = s2 * dgelu(a1[i]);
        }
        for (int o = 0; o < nh; ++o) {
            gb1[o] += d1[o];
            for (int i = 0; i < nin; ++i) gW1[o * nin + i] += d1[o] * xs[i];
        }
    }
    free(buf);
    return loss / n;
}

/* ------------------------------------------------------------------------
 * Unstructured triangles: the modal basis of TriFRPSpace (src/struct.jl:305-352)
 * and the linear-advection residual of dev/wave_triangle.jl:44-125
 * ---------------------------------------------------------------------- */

/* rs_ab, src/Geometry/geo_transform.jl:102-108 */
static void tri_rs_ab(double r, double s, double *a, double *b) {
    *a = s != 1.0 ? 2.0 * (1.0 + r) / (1.0 - s) - 1.0 : -1.0;
    *b = s;
}

/* simplex_basis, src/Transform/transform_triangle.jl:8-14 */
static double tri_simplex(double a, double b, int i, int j) {
    double h1 = fro_jacobi_p(a, 0, 0, i), h2 = fro_jacobi_p(b, 2 * i + 1, 0, j);
    return sqrt(2.0) * h1 * h2 * pow(1 - b, i);
}

/* dsimplex_basis, src/Transform/transform_triangle.jl:22-56 */
static void tri_dsimplex(double a, double b, int id, int jd, double *dr, double *ds) {
    double fa = fro_jacobi_p(a, 0, 0, id), dfa = fro_djacobi_p(a, 0, 0, id);
    double gb = fro_jacobi_p(b, 2 * id + 1, 0, jd), dgb = fro_djacobi_p(b, 2 * id + 1, 0, jd);
    double r = dfa * gb;
    if (id > 0) r *= pow(0.5 * (1.0 - b), id - 1);
    double s = dfa * (gb * (0.5 * (1.0 + a)));
    if (id > 0) s *= pow(0.5 * (1.0 - b), id - 1);
    double tmp = dgb * pow(0.5 * (1.0 - b), id);
    if (id > 0) tmp -= 0.5 * id * gb * pow(0.5 * (1.0 - b), id - 1);
    s += fa * tmp;
    r *= pow(2.0, id + 0.5);
    s *= pow(2.0, id + 0.5);
    *dr = r;
    *ds = s;
}

/* vandermonde_matrix(Tri, N, r, s), src/Transform/transform.jl:36-50: mode sk
 * over i (outer), j = 0..N-i (inner); V[pt + n*sk] */
void fro_vandermonde_tri(int N, const double *r, const double *s, int n, double *V) {
    int sk = 0;
    for (int i = 0; i <= N; ++i)
        for (int j = 0; j <= N - i; ++j, ++sk)
            for (int q = 0; q < n; ++q) {
                double a, b;
                tri_rs_ab(r[q], s[q], &a, &b);
                V[q + n * sk] = tri_simplex(a, b, i, j);
            }
}

/* dvandermonde_matrix(Tri, N, r, s), src/Transform/transform.jl:106-127 */
void fro_dvandermonde_tri(int N, const double *r, const double *s, int n, double *Vr, double *Vs) {
    int sk = 0;
    for (int i = 0; i <= N; ++i)
        for (int j = 0; j <= N - i; ++j, ++sk)
            for (int q = 0; q < n; ++q) {
                double a, b;
                tri_rs_ab(r[q], s[q], &a, &b);
                tri_dsimplex(a, b, i, j, Vr + q + n * sk, Vs + q + n * sk);
            }
}

/* Unit outward normals of the reference right triangle's faces 1 -> 2, 2 -> 3,
 * 3 -> 1 (dev/wave_triangle.jl:68). */
static const double TRI_N[3][2] = {{0.0, -1.0}, {0.70710678118654752440, 0.70710678118654752440}, {-1.0, 0.0}};

/* The dudt! closure of dev/wave_triangle.jl:44-125 for u_t + a u_x + a u_y = 0.
 * Per cell: f = iJ (a u, a u) at the solution points; face values of u and f
 * through lf; at each flux point the Rusanov-type interaction flux of the two
 * sides' physical fluxes J f (zero on a boundary face), back to the reference
 * frame through iJ; du = -(dl . f) - sum over (face, point) of
 * (n . f_int - n . f_face) phi, on cells of type 0 only (du = 0 elsewhere).
 * Fixed evaluation order (the GPU kernel repeats it): 2-vectors A x as
 * fma(A_12, x_2, A_11 x_1); dot products as ascending fma chains; the
 * correction sum runs over the flux points column-major (face fastest). */
static void tri_cell_flux(const fro_tri *t, const double *u, long c, double *f1, double *f2) {
    const long nc = t->ncell;
    const double i11 = t->iJ[c], i21 = t->iJ[c + nc], i12 = t->iJ[c + 2 * nc], i22 = t->iJ[c + 3 * nc];
    for (int q = 0; q < t->np; ++q) {
        const double fg = t->a * u[c + nc * q], gg = t->a * u[c + nc * q];
        f1[q] = fma(i12, gg, i11 * fg);
        f2[q] = fma(i22, gg, i21 * fg);
    }
}

static void tri_face_values(const fro_tri *t, const double *u, const double *f1, const double *f2, long c, int f,
                            int k, double *uf, double *ff1, double *ff2) {
    const int np = t->np, nfp = t->nfp;
    const double *l = t->lf + f + 3 * k; /* lf[f, k, q] at l[3*nfp*q] */
    const long nc = t->ncell;
    double su = u[c] * l[0], s1 = f1[0] * l[0], s2 = f2[0] * l[0];
    for (int q = 1; q < np; ++q) {
        const double w = l[(long)3 * nfp * q];
        su = fma(u[c + nc * q], w, su);
        s1 = fma(f1[q], w, s1);
        s2 = fma(f2[q], w, s2);
    }
    *uf = su;
    *ff1 = s1;
    *ff2 = s2;
}

void fro_tri_rhs(const fro_tri *t, double *du, const double *u) {
    const long nc = t->ncell;
    const int np = t->np, nfp = t->nfp;
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS schedule(static)
#endif
    for (long c = 0; c < nc; ++c) {
        double f1[64], f2[64], g1[64], g2[64], d[3 * 16];
        if (t->ctype[c] != 0) {
            for (int j = 0; j < np; ++j) du[c + nc * j] = 0.0;
            continue;
        }
        tri_cell_flux(t, u, c, f1, f2);
        const double J11 = t->J[c], J21 = t->J[c + nc], J12 = t->J[c + 2 * nc], J22 = t->J[c + 3 * nc];
        const double i11 = t->iJ[c], i21 = t->iJ[c + nc], i12 = t->iJ[c + 2 * nc], i22 = t->iJ[c + 3 * nc];
        for (int f = 0; f < 3; ++f)
            for (int k = 0; k < nfp; ++k) {
                const long fp = c + nc * (f + 3 * (long)k);
                double uL, a1, a2;
                tri_face_values(t, u, f1, f2, c, f, k, &uL, &a1, &a2);
                const double fn_face = fma(a2, TRI_N[f][1], a1 * TRI_N[f][0]);
                double fi1 = 0.0, fi2 = 0.0;
                const long n = t->nbc[fp];
                if (n >= 0) {
                    const int nf = t->nbf[fp], nk = t->nbk[fp];
                    double uR, b1, b2;
                    tri_cell_flux(t, u, n, g1, g2);
                    tri_face_values(t, u, g1, g2, n, nf, nk, &uR, &b1, &b2);
                    const double K11 = t->J[n], K21 = t->J[n + nc], K12 = t->J[n + 2 * nc], K22 = t->J[n + 3 * nc];
                    const double fL1 = fma(J12, a2, J11 * a1), fL2 = fma(J22, a2, J21 * a1);
                    const double fR1 = fma(K12, b2, K11 * b1), fR2 = fma(K22, b2, K21 * b1);
                    const double jump = uL - uR, den = jump + 1e-6;
                    const double au1 = (fL1 - fR1) / den, au2 = (fL2 - fR2) / den;
                    fi1 = 0.5 * (fL1 + fR1) - 0.5 * fabs(au1) * jump;
                    fi2 = 0.5 * (fL2 + fR2) - 0.5 * fabs(au2) * jump;
                }
                const double h1 = fma(i12, fi2, i11 * fi1), h2 = fma(i22, fi2, i21 * fi1);
                const double fn_int = fma(h2, TRI_N[f][1], h1 * TRI_N[f][0]);
                d[f + 3 * k] = fn_int - fn_face;
            }
        for (int j = 0; j < np; ++j) {
            const double r1 = dotw(f1, 1, t->dl + j, np, np);
            const double r2 = dotw(f2, 1, t->dl + j + (long)np * np, np, np);
            const double r3 = dotw(d, 1, t->phi + (long)3 * nfp * j, 1, 3 * nfp);
            du[c + nc * j] = (-r1 - r2) + (-r3);
        }
    }
}

void fro_tri_erk(const fro_tri *t, double *u, double dt, int nsteps, int s, const double *A, const double *b,
                 double *work) {
    long n = (long)t->ncell * t->np;
    double *st = work, *k = work + n;
    for (int it = 0; it < nsteps; ++it) {
        for (int i = 0; i < s; ++i) {
            int first = 1;
            for (int j = 0; j < i; ++j) {
                const double a = A[i * s + j];
                if (a == 0.0) continue;
                for (long q = 0; q < n; ++q) st[q] = first ? a * k[j * n + q] : fma(a, k[j * n + q], st[q]);
                first = 0;
            }
            if (first)
                fro_tri_rhs(t, k + i * n, u);
            else {
                for (long q = 0; q < n; ++q) st[q] = fma(dt, st[q], u[q]);
                fro_tri_rhs(t, k + i * n, st);
            }
        }
        int first = 1;
        for (int j = 0; j < s; ++j) {
            if (b[j] == 0.0) continue;
            for (long q = 0; q < n; ++q) st[q] = first ? b[j] * k[j * n + q] : fma(b[j], k[j * n + q], st[q]);
            first = 0;
        }
        if (!first)
            for (long q = 0; q < n; ++q) u[q] = fma(dt, st[q], u[q]);
    }
}
