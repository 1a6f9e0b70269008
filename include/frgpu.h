/*
 * frgpu.h -- C ABI of libfrgpu.so, the GB300 (sm_103a) flux-reconstruction
 * element-residual and explicit time-stepping library.
 *
 * Plain C types only.  Every function returns an int status (FRGPU_OK = 0,
 * negative on error) and never aborts; frgpu_last_error() returns the message
 * of the calling thread's last failure.  Host arrays are borrowed for the
 * duration of a call.  All host state arrays use the reference's Julia
 * column-major layouts, element index fastest:
 *   1D scalar      u[ne, np]                 (src/Equation/eq_advection.jl)
 *   1D Euler       u[ne, np, 3]              (src/Equation/eq_euler.jl)
 *   2D Euler       u[nx, ny, np, np, 4]      (example/shock-vortex.jl:26-118, interior only)
 *   1D1V BGK       u[ne, nvel, np]           (example/bgk_wave.jl:69-129)
 * Matrices are column-major.  Each entry point names the reference interface
 * it replaces (path:line within FluxReconstruction.jl).
 */
#ifndef FRGPU_H
#define FRGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define FRGPU_API __attribute__((visibility("default")))
#else
#define FRGPU_API
#endif

/* ---- status codes ---- */
#define FRGPU_OK 0
#define FRGPU_ERR_ARG (-1)         /* bad argument / shape / null handle */
#define FRGPU_ERR_CUDA (-2)        /* CUDA runtime error or no usable device */
#define FRGPU_ERR_NONFINITE (-3)   /* NaN/Inf met in the state */
#define FRGPU_ERR_UNPHYSICAL (-4)  /* non-positive density or pressure */
#define FRGPU_ERR_DT (-5)          /* non-positive or non-finite time step */
#define FRGPU_ERR_TIMEOUT (-6)     /* a bounded device-side wait ran out */
#define FRGPU_ERR_UNSUPPORTED (-7) /* combination not built (e.g. degree) */

/* ---- enumerations ---- */
enum frgpu_equation {
    FRGPU_ADVECTION = 0, /* u_t + a u_x = 0         eq_advection.jl          */
    FRGPU_BURGERS = 1,   /* u_t + (u^2/2)_x = 0     same scalar machinery    */
    FRGPU_EULER1D = 2,   /* 1D Euler                eq_euler.jl              */
    FRGPU_EULER2D = 3,   /* 2D Euler                shock-vortex.jl:26-118   */
    FRGPU_BGK1D = 4      /* 1D1V BGK                bgk_wave.jl:69-129       */
};
enum frgpu_flux {
    FRGPU_FLUX_ROE = 0,
    FRGPU_FLUX_LF = 1,
    FRGPU_FLUX_HLL = 2,
    FRGPU_FLUX_UPWIND = 3,
    /* 2D Euler with a per-point metric: the interaction flux of the active
     * dudt! of dev/curve_euler.jl:93-117, F* = 0.5 (f_L + f_R) - c (u_R - u_L)
     * on the face traces of the transformed flux (x faces its first, y faces its
     * second component) and of u, with a fixed dissipation coefficient c
     * (frgpu_problem_set_flux_dissipation; the script's 40 dt); the traces
     * enter the corrections unscaled.  Sides are periodic or Dirichlet (the
     * elements along a Dirichlet side keep du = 0, the script's interior-only
     * update).  Residual evaluations only: step with frgpu_step_erk (the script
     * uses Midpoint) or frgpu_step_rock. */
    FRGPU_FLUX_CENTRAL = 4
};
enum frgpu_precision {
    FRGPU_FP64 = 0, /* plain FP64 residual and stage combination            */
    FRGPU_FP32K = 1 /* FP32 residual, compensated (Kahan) stage combination  */
};
enum frgpu_bc {
    FRGPU_BC_PERIODIC = 0,  /* period_advection!/period_euler!, periodic ghosts        */
    FRGPU_BC_COPY = 1,      /* ghost element = copy of the adjacent interior element   */
    FRGPU_BC_FIXED = 2,     /* ghost element = a fixed conserved state                 */
    FRGPU_BC_DIRICHLET = 3  /* dirichlet_advection!/dirichlet_euler!: du = 0 at ends   */
};
enum frgpu_correction { FRGPU_RADAU = 0, FRGPU_SD = 1, FRGPU_HUYNH = 2 };
enum frgpu_indicator { FRGPU_IND_NONE = 0, FRGPU_IND_PLAIN = 1, FRGPU_IND_MLP = 2 };
enum frgpu_option {
    FRGPU_OPT_BGK_TENSOR = 1,
    FRGPU_OPT_FUSED_INDICATOR = 2,
    FRGPU_OPT_FUSED_TWO_STAGE = 3,
    FRGPU_OPT_BGK_CLOSURE = 4,
    FRGPU_OPT_GHOSTS_PER_STEP = 5
};

typedef struct frgpu_space frgpu_space;
typedef struct frgpu_problem frgpu_problem;
typedef struct frgpu_mlp frgpu_mlp;
typedef struct frgpu_tri frgpu_tri;

/* ======================================================================
 * Setup math (host).  Used by the space constructors; exported so a caller
 * can compare against its own FRPSpace fields.
 * ==================================================================== */

/* legendre_point(p) (src/Polynomial/poly_legendre.jl:6): deg+1 Gauss-Legendre
 * nodes, ascending, and the matching weights (src/struct.jl:47).  w may be NULL. */
FRGPU_API int frgpu_legendre_point(int deg, double *r, double *w);
/* lagrange_point(sp, x) (src/Polynomial/poly_lagrange.jl:6-20) */
FRGPU_API int frgpu_lagrange_point(const double *sp, int nsp, double x, double *l);
/* dlagrange(sp) (src/Polynomial/poly_lagrange.jl:38-59): lpdm[m + nsp*k] = l_k'(r_m) */
FRGPU_API int frgpu_dlagrange(const double *sp, int nsp, double *lpdm);
/* dradau / dsd / dhuynh (src/Polynomial/poly_legendre.jl:29-71) */
FRGPU_API int frgpu_dcorrection(int correction, int deg, const double *x, int n, double *dgl, double *dgr);
/* vandermonde_matrix(N, r) (src/Transform/transform.jl:18-26), V[i + n*j] */
FRGPU_API int frgpu_vandermonde(int deg, const double *r, int n, double *V);
/* vandermonde_matrix(Quad, N, r, s) (src/Transform/transform.jl:55-68) */
FRGPU_API int frgpu_vandermonde_quad(int deg, const double *r, const double *s, int n, double *V);

/* ======================================================================
 * Spaces (FRPSpace1D / FRPSpace2D)
 * ==================================================================== */

/* FRPSpace1D(x0, x1, nx, deg, ng=0, correction) (src/struct.jl:40-85) */
FRGPU_API int frgpu_space_create_1d(double x0, double x1, int nx, int deg, int correction, frgpu_space **out);
/* FRPSpace2D(x0, x1, nx, y0, y1, ny, deg) (src/struct.jl:229-242), uniform
 * rectangles, dhl/dhr = dradau as at src/struct.jl:193 */
FRGPU_API int frgpu_space_create_2d(double x0, double x1, int nx, double y0, double y1, int ny, int deg,
                                    frgpu_space **out);
/* Adopt operators built by the caller (e.g. the reference's own FRPSpace1D
 * fields ps.J, ps.ll, ps.lr, ps.dl, ps.dhl, ps.dhr, ps.V, ps.iV; V/iV may be NULL). */
FRGPU_API int frgpu_space_create_1d_ops(int nx, int deg, const double *J, const double *ll, const double *lr,
                                        const double *dl, const double *dhl, const double *dhr, const double *V,
                                        const double *iV, frgpu_space **out);
/* Same for FRPSpace2D on uniform rectangles of size dx x dy (iJ = diag(2/dx, 2/dy)). */
FRGPU_API int frgpu_space_create_2d_ops(int nx, int ny, int deg, double dx, double dy, const double *ll,
                                        const double *lr, const double *dl, const double *dhl, const double *dhr,
                                        const double *V, const double *iV, frgpu_space **out);
/* Query: dim, nx, ny (1 in 1D), deg. */
FRGPU_API int frgpu_space_info(const frgpu_space *s, int *dim, int *nx, int *ny, int *deg);
/* Copy a named field out: "xpl","wp","ll","lr","dl","dhl","dhr","V","iV","J","xpg".
 * n = capacity in doubles; returns the number of doubles written (>0) or an error. */
FRGPU_API int frgpu_space_get(const frgpu_space *s, const char *name, double *out, long n);
FRGPU_API void frgpu_space_destroy(frgpu_space *s);

/* ======================================================================
 * Problems: device-resident state + residual + SSPRK3 stepping
 * ==================================================================== */
typedef struct {
    int equation;           /* frgpu_equation */
    int flux;               /* frgpu_flux */
    int precision;          /* frgpu_precision */
    int bc[4];              /* 1D: bc[0] (both ends); 2D: left, right, bottom, top */
    double fixed_state[4][4]; /* per side, conserved ghost state for FRGPU_BC_FIXED */
    double a;               /* advection speed (FRGPU_ADVECTION) */
    double gamma;           /* ratio of specific heats (Euler) */
    double tau;             /* BGK relaxation time */
    int nvel;               /* BGK velocity points */
    const double *velo;     /* BGK velocity nodes [nvel] */
    const double *weights;  /* BGK quadrature weights [nvel] */
    double eps_interior;    /* scalar Roe epsilon, eq_advection.jl:130 (1e-8) */
    double eps_periodic;    /* scalar Roe epsilon at the periodic face, :163 (1e-6) */
} frgpu_problem_desc;

/* FRAdvectionProblem (eq_advection.jl:1-26) / FREulerProblem (eq_euler.jl:1-27)
 * / the ODEProblem(dudt!, ...) closures of the 2D and BGK examples: binds a
 * space and a physics description, allocates the device state. */
FRGPU_API int frgpu_problem_create(const frgpu_space *s, const frgpu_problem_desc *d, frgpu_problem **out);
FRGPU_API void frgpu_problem_destroy(frgpu_problem *p);
/* number of DOFs (doubles in one state array at the boundary) */
FRGPU_API long frgpu_problem_ndof(const frgpu_problem *p);
/* itg.u <- host u (FP64, Julia layout) / host u <- itg.u */
FRGPU_API int frgpu_state_upload(frgpu_problem *p, const double *u);
FRGPU_API int frgpu_state_download(frgpu_problem *p, double *u);
/* rhs!(du, u, p, t): frode_advection! (eq_advection.jl:55-77), frode_euler!
 * (eq_euler.jl:29-73), dudt! (shock-vortex.jl:26-118), mol! (bgk_wave.jl:69-129).
 * Host arrays in, host array out (one H2D and one D2H copy per call). */
FRGPU_API int frgpu_rhs(frgpu_problem *p, double *du, const double *u, double t);
/* nsteps of step!(itg) with SSPRK33 at fixed dt on the device-resident state
 * (OrdinaryDiffEq init(prob, SSPRK33(); adaptive=false, dt) + step!).  Steps
 * are replayed from a captured CUDA graph; the post-step filter configured by
 * frgpu_set_filter runs after every step. */
FRGPU_API int frgpu_step_ssprk3(frgpu_problem *p, double dt, int nsteps);
/* frgpu_step_ssprk3 without waiting: the steps are queued on the problem's
 * stream and the call returns at once (the same step!(itg) calls; a host loop
 * can do other work, or record events, meanwhile).  The device status of
 * these steps (non-finite or unphysical values) is reported by the next
 * synchronising call: frgpu_synchronize, frgpu_step_ssprk3, frgpu_reduce or a
 * state download. */
FRGPU_API int frgpu_step_ssprk3_async(frgpu_problem *p, double dt, int nsteps);
/* nsteps of a fixed-step explicit Runge-Kutta method given by its Butcher
 * tableau: A (s x s, row-major, strictly lower triangular) and b (s), s <= 16
 * (OrdinaryDiffEq's Midpoint, Heun, RK4, Tsit5, ... with adaptive=false, as
 * example/shock-vortex.jl:294 uses Midpoint).  Stage i evaluates the residual at
 * u + dt sum_j a_ij k_j; the step adds dt sum_j b_j k_j.  The limiter and the
 * filter configured for the problem run before and after every step, as with
 * frgpu_step_ssprk3.  Steps are replayed from a captured CUDA graph. */
FRGPU_API int frgpu_step_erk(frgpu_problem *p, int s, const double *A, const double *b, double dt, int nsteps);
/* nsteps of a stabilised explicit method: a three-term recurrence of m stages
 * followed by an explicit finishing tableau (the structure of OrdinaryDiffEq's
 * ROCK2 / ROCK4, as example/advection_kinetic.jl:133-146 steps with ROCK4 at
 * fixed dt, and of the Runge-Kutta-Chebyshev methods).  With D_0 = 0 and
 * Y_j = u + D_j,
 *   D_j = alpha_j D_{j-1} + beta_j D_{j-2} + dt (mu_j f(Y_{j-1}) + delta_j f(u)),
 * j = 1..m (D_{-1} = 0), which is the recurrence
 *   Y_j = alpha_j Y_{j-1} + beta_j Y_{j-2} + (1 - alpha_j - beta_j) u
 *         + dt (mu_j f(Y_{j-1}) + delta_j f(u))
 * in increments.  ROCK4's stages are alpha_j = 1 + kappa_j, beta_j = -kappa_j,
 * delta_j = 0 with its (mu_j, kappa_j) (alpha_1 = beta_1 = 0); RKC's are its
 * (mu_j, nu_j, mu~_j, gamma~_j) as (alpha, beta, mu, delta).  Then sf finishing
 * stages (sf = 0: none) k_i = f(Y_m + dt sum_{l<i} a_il k_l), and
 * u <- u + D_m + dt sum_i b_i k_i.  The coefficient arrays have m entries; A is
 * sf x sf row-major, strictly lower triangular; m <= 4096, sf <= 16.  The
 * caller chooses m and the coefficients for dt times the spectral radius
 * (frgpu_spectral_radius); ROCK4's tables stay with the caller (OrdinaryDiffEq
 * holds them).  The limiter and filter run around every step as with
 * frgpu_step_erk; steps replay captured graphs (the last 8 coefficient sets). */
FRGPU_API int frgpu_step_rock(frgpu_problem *p, int m, const double *alpha, const double *beta, const double *mu,
                              const double *delta, int sf, const double *A, const double *b, double dt, int nsteps);
/* Spectral radius of the Jacobian of the residual at the current state, by the
 * nonlinear power method of the RKC code (the eigenvalue estimate the ROCK
 * methods take each step): at most maxiter residual evaluations, stopping when
 * the estimate changes by at most 1 %; rho = 1.2 x the estimate.  The direction
 * is kept for the next call.  iters receives the iterations used (negative when
 * the estimate did not settle within maxiter; rho is then the last estimate). */
FRGPU_API int frgpu_spectral_radius(frgpu_problem *p, int maxiter, double *rho, int *iters);
/* Coefficients of the second-order Runge-Kutta-Chebyshev method with s >= 2
 * stages and damping eps (Sommeijer, Shampine, Verwer 1997) in the increment
 * form of frgpu_step_rock (alpha, beta, mu, delta: s entries each), and its real
 * stability bound.  Host arithmetic only. */
FRGPU_API int frgpu_rkc2_coefficients(int s, double eps, double *alpha, double *beta, double *mu, double *delta,
                                      double *bound);
/* nsteps of RKC2 in one call, as the ROCK methods step (example/advection_kinetic.jl:135
 * uses ROCK4): before every step the spectral radius (frgpu_spectral_radius,
 * maxiter), then the fewest stages s >= 2 (s = 2, then max(s + 1, floor(1.1 s)))
 * whose stability bound covers dt rho, at most smax, and the step
 * (frgpu_step_rock with frgpu_rkc2_coefficients(s, eps), cached per s).
 * stages (nsteps entries, may be NULL) receives each step's s.  Fails with
 * FRGPU_ERR_DT when dt rho needs more than smax stages.  A step's device status
 * (non-finite or unphysical values) is read with the next step's spectral
 * radius, or after the last step: the call returns at the first failed step,
 * whose stage count is the last one written to stages. */
FRGPU_API int frgpu_step_rkc2(frgpu_problem *p, double dt, int nsteps, double eps, int smax, int maxiter,
                              int *stages);
/* dt = cfl / max over points of sum_d (|u_d| + c)/dx_d (FP64 max-reduction on the GPU);
 * with a per-point metric (frgpu_problem_set_metric) the rate at a point is
 * (lambda_r + lambda_s)/2 with the contravariant speeds lambda_r = |a11 u + a12 v|
 * + c |(a11, a12)| and lambda_s = |a21 u + a22 v| + c |(a21, a22)|. */
FRGPU_API int frgpu_cfl_dt(frgpu_problem *p, double cfl, double *dt);
/* FP64 conserved sums (quadrature-weighted, per variable) and max wave speed.
 * The device status word comes back in the same synchronisation: the error of
 * steps queued before (frgpu_step_ssprk3_async) is returned here, after the
 * sums are written. */
FRGPU_API int frgpu_reduce(frgpu_problem *p, double *sums, double *maxspeed);
/* nsteps of frgpu_step_ssprk3 followed by frgpu_reduce, with one
 * synchronisation: the step!(itg) of a loop that reads back the conserved sums
 * and the wave speed after every step.  Returns the steps' status. */
FRGPU_API int frgpu_step_ssprk3_reduce(frgpu_problem *p, double dt, int nsteps, double *sums, double *maxspeed);
/* Post-step troubled-cell indicator + :l2 modal filter, example/shock-vortex.jl:308-321
 * (2D, detection on density, S0/kappa as given) and example/euler_highlevel.jl:37-52 (1D).
 * indicator = FRGPU_IND_NONE disables it. */
FRGPU_API int frgpu_set_filter(frgpu_problem *p, int indicator, double lam, double S0, double kappa);
/* Apply the indicator + filter once now; *ntroubled receives the troubled-element count. */
FRGPU_API int frgpu_modal_filter(frgpu_problem *p, int indicator, double lam, double S0, double kappa,
                                 int *ntroubled);
/* positive_limiter(u, γ, weights, ll, lr, t0) (src/dissipation.jl:38-216) on
 * every element of the device state, once now: the scalar form for advection
 * and Burgers, the 1D and 2D Euler forms with the density and energy
 * correctors.  weights: the element quadrature weights (np values in 1D, np^2
 * in 2D, q = k + np l; the Euler forms expect them to sum to 1, as
 * example/shock-vortex.jl:301 passes ps.wp ./ 4), or NULL for the space's
 * Gauss weights so normalised.  t0 in (0, 1] caps the energy scaling.
 * *nlimited receives the number of elements scaled with a parameter below 1.
 * FRGPU_ERR_UNPHYSICAL when an element's density parameter leaves (0, 1] (the
 * reference's assertion).  Closed-form energy parameter and min(t_j, t0):
 * see csrc/limiter.cu. */
FRGPU_API int frgpu_positive_limiter(frgpu_problem *p, const double *weights, double t0, int *nlimited);
/* Per-point metric (FRPSpace2D's inverse Jacobian iJ[i, j][k, l],
 * src/struct.jl:135-158): iJ as a host array [nx, ny, np, np, 2, 2] (column-major,
 * the 2 x 2 matrices last).  The residual then takes f = a11 F + a12 G and
 * g = a21 F + a22 G at every solution point.
 * Without face normals (n1 = n2 = NULL) the interface fluxes are Cartesian and
 * the corrections scale them by a11 (x faces) and a22 (y faces), the dudt!
 * closure of example/shock-vortex.jl:48-55, :102-115: exact for rectangles of
 * different sizes (stretched meshes).
 * With the unit normals of the x faces n1[nx+1, ny, 2] and the y faces
 * n2[nx, ny+1, 2], the interface fluxes are solved in each face's frame and
 * scaled by (iJ n)_1, (iJ n)_2, the formulation of dev/parallelogram.jl:115-160
 * for straight-sided quadrilaterals (a uniform flow stays uniform on affine
 * elements).
 * iJ = NULL returns to the uniform rectangles of the space (iJ = diag(2/dx,
 * 2/dy)); 2D Euler only.  The learned indicator then runs as its own kernel. */
FRGPU_API int frgpu_problem_set_metric(frgpu_problem *p, const double *iJ, const double *n1, const double *n2);
/* The face-Jacobian form of the interface-flux scaling of the reference's
 * quadrilateral cylinder scripts (dev/cylinder2.jl:147-150, dev/cylinder3.jl:
 * 147-150; commented out in dev/curve_euler.jl:130-133): the interface flux of
 * face point q is scaled by (inv(Ji[i, j][f, q]) n)_1 on x faces (f = left 4,
 * right 2) and (inv(Ji[i, j][f, q]) n)_2 on y faces (f = bottom 1, top 3), with
 * the face Jacobians Ji of FRPSpace2D (src/struct.jl:145-158) passed as
 * Ji[nx, ny, 4, np, 2, 2] (column-major) and the unit normals n1, n2 the metric
 * was set with.  Needs frgpu_problem_set_metric with normals first; Ji = NULL
 * returns to the (iJ n) scaling at the solution points. */
FRGPU_API int frgpu_problem_set_face_jacobians(frgpu_problem *p, const double *Ji, const double *n1, const double *n2);
/* Dissipation coefficient c >= 0 of FRGPU_FLUX_CENTRAL (dev/curve_euler.jl uses
 * 40 dt with its dt = 0.002). */
FRGPU_API int frgpu_problem_set_flux_dissipation(frgpu_problem *p, double c);
/* Run the limiter before every step of frgpu_step_ssprk3 (the loop of
 * example/shock-vortex.jl:297-303); on = 0 turns it off. */
FRGPU_API int frgpu_set_limiter(frgpu_problem *p, int on, const double *weights, double t0);
/* Per-element troubled flags of the last filter application (ne ints). */
FRGPU_API int frgpu_troubled_flags(frgpu_problem *p, int *flags, long n);
/* Kernel choices for measurements; no counterpart in the reference.
 * FRGPU_OPT_BGK_TENSOR: 1 (default) runs the FP32 BGK transport as a TF32-split
 * tensor-core product with warp-level mma.sync, 2 the same product on tcgen05
 * (M = 128 velocities per CTA, accumulators in tensor memory; the same bits as
 * 1, slower on small velocity grids), 0 on the CUDA cores.
 * FRGPU_OPT_FUSED_INDICATOR: 1 (default) runs the indicator (learned or plain)
 * + filter of an FP32K deg-3 2D Euler problem inside its third SSPRK3 stage, 0
 * as a kernel of its own after the step.
 * FRGPU_OPT_FUSED_TWO_STAGE: 1 (default) runs two-stage tableaux of
 * frgpu_step_erk (Midpoint, Heun, ...) on a 2D Euler problem fused into the
 * stage kernel, 0 through the generic residual + combination kernels.
 * FRGPU_OPT_BGK_CLOSURE: the Maxwellian of a BGK problem.  0 (default): from
 * the moments through conserve_prim(w, 3) (example/bgk_wave.jl:76-81); 1: the
 * density-only closure prim = [rho, a, 1], M = rho sqrt(1/pi) exp(-(v - a)^2),
 * a the problem's advection speed (example/advection_kinetic.jl:80-87, the
 * problem that script steps with ROCK4).
 * FRGPU_OPT_GHOSTS_PER_STEP: 2D Euler.  0 (default): the periodic and copy
 * neighbours outside the domain follow every stage's input.  1: they keep the
 * values of the step's start through the step, as the reference scripts
 * refresh their ghost layers once per step (example/shock-vortex.jl:323-330,
 * example/euler2d_wave.jl:125-135; dudt! leaves du = 0 on the ghosts).  It
 * applies to every step (frgpu_step_ssprk3, frgpu_step_erk, frgpu_step_rock);
 * a lone residual evaluation (frgpu_rhs) has no step start.
 * The next step re-captures its graph. */
FRGPU_API int frgpu_problem_set_option(frgpu_problem *p, int option, int value);
/* Device pointer to the primary state array and its element type size
 * (8 for FP64, 4 for FP32K), for zero-copy hand-off; the stream the problem's
 * kernels run on; the number of this library's kernel launches so far.
 * The device state keeps the host layout except for 2D Euler, whose device
 * array holds the 4 conserved variables of each solution point together:
 * value (i, j, k, l, m) of the host u[nx, ny, deg+1, deg+1, 4] sits at
 * ((q * nx * ny) + i + nx * j) * 4 + m with q = k + (deg + 1) * l. */
FRGPU_API int frgpu_problem_device_state(frgpu_problem *p, void **dptr, int *elem_bytes);
FRGPU_API int frgpu_problem_stream(frgpu_problem *p, void **stream);
FRGPU_API long frgpu_problem_launches(const frgpu_problem *p);
/* Wait for the problem's stream; returns the status of the work queued since
 * the last check (FRGPU_ERR_NONFINITE, FRGPU_ERR_UNPHYSICAL, ...). */
FRGPU_API int frgpu_synchronize(frgpu_problem *p);
/* Fused multiply-add throughput of the current GPU, measured (FLOP/s, an FMA
 * counted as 2): kind 0 = FP64, 1 = FP32, 2 = FP32 pairs (f32x2).  No
 * counterpart in the reference: it is the ceiling the compute-bound forms (the
 * FP64 residuals) are placed against.  Allocates a little scratch and times a
 * few launches with CUDA events. */
FRGPU_API int frgpu_fma_peak(int kind, double *flops_per_s);

/* ======================================================================
 * Learned troubled-cell indicator.  Stands in for the modal-decay test
 * shock_detector(log10(su), ...) (src/dissipation.jl:13-23) in the post-step
 * filter loop of example/shock-vortex.jl:308-321: a 32 -> 64 -> 64 -> 1
 * perceptron (GELU, GELU, sigmoid) on per-element normalised modal energies
 * of density and pressure (deg = 3), BF16 inputs/weights, FP32 accumulation
 * on the tensor cores.  Parameters (FP32): W1[64][32] b1[64] W2[64][64]
 * b2[64] W3[64] b3[1], row-major [out][in].
 * ==================================================================== */
FRGPU_API int frgpu_mlp_nparams(void);
FRGPU_API int frgpu_mlp_create(int seed, frgpu_mlp **out);
FRGPU_API void frgpu_mlp_destroy(frgpu_mlp *m);
FRGPU_API int frgpu_mlp_get_params(const frgpu_mlp *m, float *params);
FRGPU_API int frgpu_mlp_set_params(frgpu_mlp *m, const float *params);
/* y[i] = network(x[i, 0:32]) for host arrays x[n][32], y[n] */
FRGPU_API int frgpu_mlp_forward(frgpu_mlp *m, const float *x, long n, float *y);
/* mean binary cross-entropy of (x, t) and its gradient (nparams floats) */
FRGPU_API int frgpu_mlp_loss_grad(frgpu_mlp *m, const float *x, const float *t, long n, float *loss, float *grad);
/* mini-batch Adam training; loss_out[epochs] (optional) receives the mean loss per epoch */
FRGPU_API int frgpu_mlp_train(frgpu_mlp *m, const float *x, const float *t, long n, int epochs, int batch, float lr,
                              int seed, float *loss_out);
/* Bind a network to a 2D Euler problem (deg = 3) for FRGPU_IND_MLP: an element
 * is troubled when the network's probability exceeds `threshold`; within
 * `band` of the threshold the plain modal-decay test decides (fallback).  An
 * element whose modal decay lies below the plain test's sigma = 1 region
 * (log10 su < S0 - kappa) is smooth without consulting the network.  The
 * network is borrowed and must outlive its use. */
FRGPU_API int frgpu_problem_set_mlp(frgpu_problem *p, const frgpu_mlp *m, double threshold, double band);
/* The 32 indicator inputs of every element of the current state, feat[ne][32]. */
FRGPU_API int frgpu_modal_features(frgpu_problem *p, float *feat, long n);
/* After an FRGPU_IND_MLP filter: stats[0] troubled elements, stats[1]
 * network-vs-plain disagreements (misfires judged by the plain test),
 * stats[2] elements decided by the plain fallback. */
FRGPU_API int frgpu_indicator_stats(frgpu_problem *p, int *stats);

/* ======================================================================
 * Batched ensembles of 1D Burgers instances of uneven size and degree.  Each
 * instance is the scalar residual of frode_advection!
 * (src/Equation/eq_advection.jl:55-77) with the flux u^2/2 on periodic
 * [x0, x1]; frgpu_ensemble_run advances all of them to t_end in one
 * persistent kernel launch.  No single call in the reference does this: it
 * replaces a host loop over FRAdvectionProblem-style problems.
 * ==================================================================== */
typedef struct frgpu_ensemble frgpu_ensemble;
FRGPU_API int frgpu_ensemble_config4_sizes(int n, unsigned seed, int *ne, int *deg);
FRGPU_API int frgpu_ensemble_create(int n, const int *ne, const int *deg, double x0, double x1, int precision,
                                    frgpu_ensemble **out);
FRGPU_API void frgpu_ensemble_destroy(frgpu_ensemble *e);
FRGPU_API long frgpu_ensemble_ndof(const frgpu_ensemble *e);
FRGPU_API int frgpu_ensemble_set_state(frgpu_ensemble *e, int i, const double *u);
FRGPU_API int frgpu_ensemble_get_state(frgpu_ensemble *e, int i, double *u);
FRGPU_API int frgpu_ensemble_init_fourier(frgpu_ensemble *e, double sigma, unsigned seed);
FRGPU_API int frgpu_ensemble_set_tiles(frgpu_ensemble *e, const int *thr);
FRGPU_API int frgpu_ensemble_get_tiles(const frgpu_ensemble *e, int *thr);
FRGPU_API int frgpu_ensemble_run(frgpu_ensemble *e, double t_end, double cfl, int filter);
FRGPU_API int frgpu_ensemble_stats(const frgpu_ensemble *e, double *dof_stage_updates, int *max_steps, float *ms,
                                   double *dt, int *steps);
FRGPU_API int frgpu_ensemble_tune(frgpu_ensemble *e, double t_probe, double cfl, int filter, int *thr);
FRGPU_API long frgpu_ensemble_launches(const frgpu_ensemble *e);
/* Learned indicator in the ensemble's post-step filter (config-4 form; no
 * counterpart in the reference): network m (NULL = plain modal-decay test of
 * example/euler_highlevel.jl:37-52), probability threshold, fallback band
 * within which the plain test decides.  The network is borrowed. */
FRGPU_API int frgpu_ensemble_set_mlp(frgpu_ensemble *e, const frgpu_mlp *m, double threshold, double band);
/* Last run's learned-indicator counts over all steps and instances:
 * stats[0] troubled, [1] misfires (network != plain test), [2] fallbacks, [3] judged. */
FRGPU_API int frgpu_ensemble_indicator_stats(frgpu_ensemble *e, long long *stats);
/* Instances stopped because their state turned non-finite: flags[i] = the
 * step (1-based) after which instance i stopped, -1 when it was not started
 * because its CFL step count t_end / dt exceeds 2e9 (a state of huge or
 * infinite magnitude), 0 otherwise (flags may be NULL).  Returns their number.
 * frgpu_ensemble_run stops such an instance and carries on with the others; it
 * stays stopped until its state is set again. */
FRGPU_API int frgpu_ensemble_failed(frgpu_ensemble *e, int *flags);
/* Total element count over all instances. */
FRGPU_API long frgpu_ensemble_nelem(const frgpu_ensemble *e);
/* Training rows of the 1D learned indicator: 32 features per element (modal
 * energies, degree one-hot, energy level) and the plain test's label (1 =
 * troubled) for every element of the current state, instance by instance;
 * n = frgpu_ensemble_nelem(e). */
FRGPU_API int frgpu_ensemble_features(frgpu_ensemble *e, float *feat, int *labels, long n);

/* Allocation-free 2D Euler reduction.  No counterpart in the reference: it
 * exists for callers that cannot let this library call cudaMalloc -- hosts
 * whose own pool (a Julia CUDA.jl or PyTorch caching allocator) must own every
 * device byte, and processes that fix their device footprint at start-up.
 * Inputs and outputs are the caller's device memory: the state d_state
 * (u[nx, ny, deg+1, deg+1, 4] in the Julia layout; double for FRGPU_FP64,
 * with d_lo = NULL, or float for FRGPU_FP32K, with d_lo either NULL or the
 * float low part in the same layout, added to the state), the
 * quadrature weights d_wp[(deg+1)^2] (wp[k + (deg+1) l] = w_k w_l), and d_out[6]
 * receiving the FP64 conserved sums (4), the maximum wave speed and the
 * maximum CFL rate max((|u|+c)/dx + (|v|+c)/dy) -- the values frgpu_reduce and
 * frgpu_cfl_dt compute.  The work is queued on `stream` (NULL = legacy
 * default stream) and nothing is synchronised.  Scratch is a fixed 192 KiB
 * device array inside the library, held by every GPU that loads it until the
 * process exits.  A call needs ceil(nx*ny / 16384) * (deg+1)^2 partial blocks
 * of it and at most 4096 fit; meshes that need more are rejected with
 * FRGPU_ERR_ARG (at most 67,108,864 solution points nx*ny*(deg+1)^2, and
 * fewer when nx*ny is not a multiple of 16384).  A non-NULL d_lo with
 * FRGPU_FP64 is rejected too.  No cudaMalloc/cudaFree is called.  The
 * first call on each device looks up the array's device address, so make
 * that first call before any stream capture.  All calls share the one array:
 * calls that overlap on the GPU (different streams, or different host
 * threads) race and must be serialised by the caller. */
FRGPU_API int frgpu_reduce2d_noalloc(const void *d_state, const void *d_lo, int precision, int nx, int ny, int deg,
                                     double dx, double dy, double gamma, const double *d_wp, double *d_out,
                                     void *stream);

/* ======================================================================
 * Stateless operators
 * ==================================================================== */

/* interp_face!(fdelta, f, ll, lr) for a matrix f[n, np]
 * (src/interpolate.jl:6-10): fdelta[i, 1] = f[i,:].ll, fdelta[i, 2] = f[i,:].lr.
 * Host arrays (column-major), computed on the GPU. */
FRGPU_API int frgpu_interp_face(const double *f, long n, int np, const double *ll, const double *lr,
                                double *fdelta);
/* poly_derivative!(df, f, pdm) row-wise for a matrix f[n, np]
 * (src/derivative.jl:1-10): df[i, m] = sum_k f[i, k] pdm[m, k]. */
FRGPU_API int frgpu_poly_derivative(const double *f, long n, int np, const double *pdm, double *df);

/* ======================================================================
 * Unstructured triangles: TriFRPSpace (src/struct.jl:305-352) and the
 * linear-advection dudt! of dev/wave_triangle.jl:44-125.  Column-major
 * arrays, cell index fastest: u[ncell, np] with np = (deg+1)(deg+2)/2.
 * ==================================================================== */

/* vandermonde_matrix(Tri, N, r, s) and dvandermonde_matrix(Tri, N, r, s)
 * (src/Transform/transform.jl:36-50, :106-127): V, Vr, Vs [n, np], mode (i, j)
 * with j fastest; any output may be NULL. */
FRGPU_API int frgpu_vandermonde_tri(int deg, const double *r, const double *s, int n, double *V, double *Vr,
                                    double *Vs);
/* The operators TriFRPSpace builds from its solution points (r, s) (the np
 * points of tri_quadrature(deg), src/Quadrature/quadrature.jl:14-71): V[np, np];
 * dl[np, np, 2] (dlagrange(V, Vr, Vs): dl[j, q, d] = d l_q / d r_d at point j);
 * lf[3, deg+1, np] (l_q at the flux points of triface_quadrature,
 * quadrature.jl:86-106); phi[3, deg+1, np] (correction_field,
 * src/Polynomial/poly_triangle.jl:1-28).  Any output may be NULL. */
FRGPU_API int frgpu_tri_operators(int deg, const double *r, const double *s, double *V, double *dl, double *lf,
                                  double *phi);
/* A triangle problem: ncell cells of degree 1..3, precision FRGPU_FP64 or
 * FRGPU_FP32K, speed a (u_t + a u_x + a u_y = 0); the space's dl, lf, phi as
 * above; J and iJ [ncell, 2, 2] (rs_jacobi, src/Geometry/geo_jacobi.jl:32-43,
 * and its inverse); nb_cell, nb_face, nb_point [ncell, 3, deg+1]: the 0-based
 * neighbour_fpidx of every flux point (src/Geometry/geo_neighbor.jl:8-60;
 * nb_cell < 0 on a boundary face); cell_type[ncell] (only cells of type 0 are
 * updated, as in dev/wave_triangle.jl:117-121).  The state starts at zero. */
FRGPU_API int frgpu_tri_create(int ncell, int deg, int precision, double a, const double *dl, const double *lf,
                               const double *phi, const double *J, const double *iJ, const int *nb_cell,
                               const int *nb_face, const int *nb_point, const int *cell_type, frgpu_tri **out);
FRGPU_API int frgpu_tri_destroy(frgpu_tri *t);
FRGPU_API int frgpu_tri_set_state(frgpu_tri *t, const double *u);
FRGPU_API int frgpu_tri_get_state(frgpu_tri *t, double *u);
/* du = L(u) for host arrays: dudt!(du, u, p, t) of dev/wave_triangle.jl:44 */
FRGPU_API int frgpu_tri_rhs(frgpu_tri *t, double *du, const double *u);
/* L(device state) into device scratch on the object's stream (no host copy) */
FRGPU_API int frgpu_tri_rhs_device(frgpu_tri *t);
/* nsteps fixed steps of the explicit tableau (A row-major s x s, b) on the
 * device state: init(prob, alg; dt, adaptive=false) + step!
 * (dev/wave_triangle.jl:131-135 with Euler()); replayed from a CUDA graph. */
FRGPU_API int frgpu_tri_step_erk(frgpu_tri *t, int s, const double *A, const double *b, double dt, int nsteps);
FRGPU_API int frgpu_tri_stream(frgpu_tri *t, void **stream);
FRGPU_API int frgpu_tri_launches(frgpu_tri *t, long long *n);

/* ======================================================================
 * Diagnostics
 * ==================================================================== */
FRGPU_API int frgpu_last_error(char *buf, unsigned long n);
FRGPU_API int frgpu_version(void);

#ifdef __cplusplus
}
#endif
#endif
