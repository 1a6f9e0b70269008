/*
 * fr_oracle.h -- CPU FP64 oracle for the flux-reconstruction hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, in plain C, the
 * reference's (FluxReconstruction.jl) algorithms for the element residual and
 * explicit time stepping.  It is linked only by tests/, by the smoke check in
 * __graft_entry__.py and by the cpu_baseline / --impl reference legs of
 * bench.py.  The product library (libfrgpu.so) never calls it.
 *
 * Parity status: the setup math (Gauss-Legendre points, Lagrange operators,
 * correction-function derivatives, orthonormal Jacobi / Vandermonde matrices)
 * is pinned against the reference's own identities
 * (example/vandermonde_lagrange.jl:14,15,25) and against numpy's
 * leggauss.  The residual structure follows the cited reference code line by
 * line.  The KitBase 0.9 physics kernels (flux_hll!, euler_flux, the :l2
 * modal filter, conserve_prim, maxwellian) are not vendored in the reference,
 * so they are restated from their published methods; at that boundary parity
 * is unpinned (the reference cannot run here: no Julia).
 * Triangles: the solution points are pinned to golden vectors generated from
 * the reference's own src/Quadrature/qpmin.py; the triangle residual
 * (dev/wave_triangle.jl, a script with no test or recorded output) is parity
 * unpinned beyond its properties (uniform state kept, conservation, order of
 * convergence).  Face normals of straight-sided quadrilaterals
 * (dev/parallelogram.jl) likewise: pinned only by free-stream preservation.
 *
 * Array layouts are the reference's Julia column-major layouts:
 *   1D scalar      u[i, k]            -> u[i + ne*k]
 *   1D Euler       u[i, k, m]         -> u[i + ne*(k + np*m)]
 *   2D Euler       u[i, j, k, l, m]   -> u[i + nx*(j + ny*(k + np*(l + np*m)))]
 *   1D1V BGK       u[i, v, k]         -> u[i + ne*(v + nvel*k)]
 * Matrices (lpdm, V, iV) are column-major: A[r + n*c].
 */
#ifndef FR_ORACLE_H
#define FR_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- setup math ---- */
void fro_gauss_legendre(int n, double *x, double *w);
double fro_legendre_p(int n, double x);
double fro_dlegendre(int n, double x);
/* kind: 0 radau, 1 sd, 2 huynh */
void fro_dcorrection(int kind, int deg, const double *x, int nx, double *dgl, double *dgr);
void fro_lagrange_point(const double *sp, int nsp, double x, double *l);
void fro_dlagrange(const double *sp, int nsp, double *lpdm);
double fro_jacobi_p(double x, double alpha, double beta, int N);
double fro_djacobi_p(double x, double alpha, double beta, int N);
void fro_vandermonde_1d(int N, const double *r, int nr, double *V);
void fro_dvandermonde_1d(int N, const double *r, int nr, double *Vr);
void fro_vandermonde_quad(int N, const double *r, const double *s, int n, double *V);
int fro_inverse(int n, const double *A, double *Ainv);
int fro_shock_detector(double Se, int deg, double S0, double kappa);

/* ---- residual configuration ---- */
enum { FRO_ADVECTION = 0, FRO_BURGERS = 1, FRO_EULER1D = 2, FRO_EULER2D = 3, FRO_BGK1D = 4 };
enum { FRO_FLUX_ROE = 0, FRO_FLUX_LF = 1, FRO_FLUX_HLL = 2, FRO_FLUX_UPWIND = 3, FRO_FLUX_CENTRAL = 4 };
enum { FRO_BC_PERIODIC = 0, FRO_BC_COPY = 1, FRO_BC_FIXED = 2, FRO_BC_DIRICHLET = 3 };

typedef struct {
    int kind, flux;
    int nx, ny, np, nvel;
    double a, gamma, tau;
    int bc[4];                 /* 1D: bc[0] for both ends; 2D: left, right, bottom, top */
    double fixed_state[4][4];  /* conserved ghost state per side for FRO_BC_FIXED */
    double eps_interior, eps_periodic;
    const double *J;           /* 1D: per-element Jacobian dx_i/2 */
    double iJx, iJy;           /* 2D rectangular elements: 2/dx, 2/dy */
    const double *ll, *lr, *lpdm, *dgl, *dgr;
    const double *velo, *weights; /* BGK velocity grid */
    const double *iJ;          /* 2D: per-point inverse Jacobian [nx, ny, np, np, 2, 2]
                                  (column-major) or NULL for diag(iJx, iJy) */
    const double *n1, *n2;     /* 2D with iJ: unit normals of the x faces [nx+1, ny, 2] and
                                  the y faces [nx, ny+1, 2], or NULL for the Cartesian axes */
    const double *Ji;          /* 2D with iJ and normals: face Jacobians [nx, ny, 4, np, 2, 2]
                                  (FRPSpace2D's Ji, src/struct.jl:145-158) for the interface-flux
                                  scales of dev/cylinder2.jl:147-150, or NULL */
    int bgk_closure;           /* BGK Maxwellian: 0 conserve_prim(w, 3) (bgk_wave.jl),
                                  1 prim = [rho, a, 1] (advection_kinetic.jl) */
    double flux_c;             /* FRO_FLUX_CENTRAL: dissipation coefficient c */
    int ghosts_per_step;       /* 2D: periodic and copy ghosts hold the step's start values through
                                  the step (the scripts refresh their ghost layers once per step);
                                  applies in fro_ssprk3, fro_erk and fro_rock */
    const double *ghost_src;   /* internal: the state the ghosts are copied from (NULL: the input) */
} fro_cfg;

long fro_ndof(const fro_cfg *c);
void fro_rhs(const fro_cfg *c, double *du, const double *u);
/* Shu-Osher SSPRK3, nsteps fixed steps of size dt; work must hold 2*ndof doubles */
void fro_ssprk3(const fro_cfg *c, double *u, double dt, int nsteps, double *work);
/* nsteps of (SSPRK3 step, indicator + :l2 filter), example/shock-vortex.jl:294-321 */
void fro_ssprk3_filtered(const fro_cfg *c, double *u, double dt, int nsteps, double *work, const double *V,
                         const double *iV, double lam, double S0, double kappa);
/* explicit Runge-Kutta of s stages (A: s x s row-major, b: s), fixed dt;
 * work must hold (s + 1) * ndof doubles */
void fro_erk(const fro_cfg *c, double *u, double dt, int nsteps, int s, const double *A, const double *b,
             double *work);

/* stabilised step: m-stage three-term recurrence in increment form + explicit
 * finishing tableau (sf stages); work must hold (7 + sf) * ndof doubles */
void fro_rock(const fro_cfg *c, double *u, double dt, int nsteps, int m, const double *alpha, const double *beta,
              const double *mu, const double *delta, int sf, const double *A, const double *b, double *work);
/* spectral radius of the residual's Jacobian by the nonlinear power method;
 * dir (ndof) in/out, work 3 * ndof doubles; returns iterations (negative when
 * not settled) */
int fro_spectral_radius(const fro_cfg *c, const double *u, int maxiter, double *dir, int *have, double *rho,
                        double *work);

/* ---- troubled-cell indicator and modal filter ---- */
/* 2D, per step: detect on rho with iV (np^2 x np^2), filter all 4 variables
 * with the flattened L2 filter of strength lam.  Returns number of troubled
 * elements; flags (may be NULL) receives 0/1 per element (i fastest). */
int fro_filter2d(const fro_cfg *c, double *u, const double *V, const double *iV,
                 double lam, double S0, double kappa, int *flags);
/* 1D Euler form (euler_highlevel.jl): su = u_N^2/(sum u^2 + 1e-6), kappa = 4 */
int fro_filter1d(const fro_cfg *c, double *u, int nvar, const double *V, const double *iV,
                 double lam, int *flags);
/* modal energies for the learned indicator: per element 2*np^2 features */
void fro_modal_features2d(const fro_cfg *c, const double *u, const double *iV, double *feat);
void fro_modal_features1d(const fro_cfg *c, const double *u, const double *iV, double *feat);

/* ---- positivity-preserving limiter (src/dissipation.jl:38-216) ---- */
/* w: the element quadrature weights normalised to sum 1 (2D: np^2 values, the
 * reference passes ps.wp / 4; 1D: np values); t0 caps the energy scaling.
 * Return: the number of elements scaled with a parameter below 1, or minus the
 * number of elements whose density parameter left (0, 1]. */
int fro_positive_limiter2d(const fro_cfg *c, double *u, const double *w, double t0);
int fro_positive_limiter1d(const fro_cfg *c, double *u, const double *w, double t0);
int fro_positive_limiter_scalar(const fro_cfg *c, double *u, const double *w, double t0);

/* ---- reductions and norms ---- */
void fro_conserved_sums2d(const fro_cfg *c, const double *u, const double *wp, double *sums);
double fro_max_speed2d(const fro_cfg *c, const double *u);
double fro_L1_error(const double *u, const double *ue, long n, double dx);
double fro_L2_error(const double *u, const double *ue, long n, double dx);
double fro_Linf_error(const double *u, const double *ue, long n, double dx);

/* ---- physics helpers (KitBase restatements) ---- */
void fro_prim_conserve2d(const double *prim, double gamma, double *w);
void fro_conserve_prim2d(const double *w, double gamma, double *prim);
void fro_prim_conserve1d(const double *prim, double gamma, double *w);
void fro_flux_hll2d(const double *wL, const double *wR, double gamma, int dir, double *fw);
void fro_flux_lf2d(const double *wL, const double *wR, double gamma, int dir, double *fw);
void fro_flux_hll1d(const double *wL, const double *wR, double gamma, double *fw);
void fro_ib_rh(double Ma, double gamma, double *pre, double *post);

/* ---- learned indicator (MLP 32->64->64->1, GELU, sigmoid), FP64 ---- */
/* params layout: W1[64x32] b1[64] W2[64x64] b2[64] W3[1x64] b3[1], row-major W[out][in] */
void fro_mlp_forward(const double *params, const double *x, int n, int nin, int nh, double *y);
/* mean binary cross-entropy loss and its gradient w.r.t. params */
double fro_mlp_loss_grad(const double *params, const double *x, const double *label, int n,
                         int nin, int nh, double *grad);

/* threads used by the OpenMP loops (0 = library default) */
void fro_set_threads(int n);

/* ---- unstructured triangles (TriFRPSpace, src/struct.jl:305-352; the advection
 * dudt! of dev/wave_triangle.jl:44-125).  Column-major arrays, cell index fastest:
 * u[ncell, np]; dl[np, np, 2] (dl[j, q, d] = d l_q / d r_d at point j); lf and phi
 * [3, nfp, np]; J and iJ [ncell, 2, 2]; nbc, nbf, nbk [ncell, 3, nfp] the 0-based
 * neighbour cell (< 0: boundary face), its face and its flux point. ---- */
typedef struct {
    int ncell, deg, np, nfp;
    double a;
    const double *dl, *lf, *phi, *J, *iJ;
    const int *nbc, *nbf, *nbk, *ctype;
} fro_tri;
void fro_vandermonde_tri(int N, const double *r, const double *s, int n, double *V);
void fro_dvandermonde_tri(int N, const double *r, const double *s, int n, double *Vr, double *Vs);
void fro_tri_rhs(const fro_tri *t, double *du, const double *u);
void fro_tri_erk(const fro_tri *t, double *u, double dt, int nsteps, int s, const double *A, const double *b,
                 double *work);
int fro_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
