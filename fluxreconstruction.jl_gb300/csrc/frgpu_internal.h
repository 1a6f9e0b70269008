// frgpu_internal.h -- host-side structures shared by the libfrgpu translation units.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>
#include <map>
#include <vector>

#include "../../include/frgpu.h"

struct frgpu_space {
    int dim = 1, nx = 0, ny = 1, deg = 0, np = 0;
    double x0 = 0, x1 = 1, y0 = 0, y1 = 1, dx = 0, dy = 0;
    std::vector<double> J;        // 1D: per-element Jacobian dx_i / 2
    std::vector<double> xpl, w1;  // Gauss-Legendre nodes / weights on [-1, 1]
    std::vector<double> wp;       // 1D: w1; 2D: w1 (x) w1, wp[k + np*l] = w_k w_l
    std::vector<double> ll, lr;   // Lagrange basis at r = -1, +1
    std::vector<double> dl;       // lpdm, column-major dl[m + np*k] = l_k'(r_m)
    std::vector<double> dhl, dhr; // correction-function derivatives at the nodes
    std::vector<double> V, iV;    // Vandermonde matrix and inverse (1D np x np, 2D np^2 x np^2)
    std::vector<double> xc, yc;   // element centres
};

// Device buffers of a problem.  FP64: s0 = u^n, s1/s2 = stage states.
// FP32K: s0 = u^n high part, s1/s2 = stage increments d1/d2, s3 = low part.
// Stage coefficients of the fused step (stages 1..3 of the 2D Euler kernel):
// SSPRK3, or a two-stage explicit method run as stages 1 and 3.
struct fr_method {
    int stages = 3;
    double c1 = 1.0;                                  // stage 1 scale of dt L
    double fa = 1.0, fs = 2.0 / 3.0;                  // FP32K last stage: (fa d + dt L) fs
    double g3 = 2.0, al3 = 2.0, be3 = 1.0, s3 = 1.0 / 3.0; // FP64 last stage: (g3 dt L + al3 u_s + be3 u^n) s3
    bool operator==(const fr_method &o) const {
        return stages == o.stages && c1 == o.c1 && fa == o.fa && fs == o.fs && g3 == o.g3 && al3 == o.al3 &&
               be3 == o.be3 && s3 == o.s3;
    }
};

struct frgpu_problem {
    frgpu_space sp;
    frgpu_problem_desc d{};
    std::vector<double> velo, weights;
    int device = 0;
    cudaStream_t stream = nullptr;
    long ndof = 0;
    size_t esize = 8; // bytes per state value on the device
    void *s0 = nullptr, *s1 = nullptr, *s2 = nullptr, *s3 = nullptr;
    double *d_dt = nullptr;  // device copy of dt (graphs read it from here)
    int *d_status = nullptr; // accumulated status bits
    double *d_red = nullptr; // reduction scratch
    int *d_flags = nullptr;  // troubled flags per element
    int *d_count = nullptr;  // counters: [0..2] indicator (troubled, misfires, fallbacks), [FR_COUNT_LIMITER]
    void *d_velo = nullptr, *d_w = nullptr; // BGK velocity grid (state precision)
    void *d_J = nullptr;                    // 1D per-element Jacobian (state precision)
    void *d_V = nullptr, *d_iV = nullptr;   // Vandermonde matrix / inverse (state precision)
    void *rhs_in = nullptr, *rhs_out = nullptr; // scratch of frgpu_rhs
    void *d_stage = nullptr;                // FP64 staging of state uploads / downloads (+ 8 bytes)
    void *d_met = nullptr;                  // 2D Euler: per-point inverse Jacobian (a11, a12, a21, a22), or null
    void *d_nfx = nullptr, *d_nfy = nullptr; // with d_met: unit normals of the x and y faces, or null
    void *d_fsc = nullptr; // with normals: interface-flux scales (inv(Ji) n) per (point line, element), or null
    int parity = 0;                         // FP32K: which buffer holds u^n (0: s0, 1: s1)
    bool prepare_only = false;              // launchers only set kernel attributes
    // post-step filter
    int indicator = FRGPU_IND_NONE;
    double lam = 0, S0 = 0, kappa = 0;
    const frgpu_mlp *mlp = nullptr; // learned indicator (borrowed)
    float mlp_thr = 0.5f, mlp_band = 0.0f;
    int bgk_tensor = 1;             // FP32 BGK transport on the tensor cores
    int bgk_closure = 0;            // BGK Maxwellian: 0 conserve_prim(w, 3), 1 prim = [rho, a, 1]
    int ghosts_per_step = 0;        // 2D steps: ghost neighbours from u^n in the later stages
    const void *lag_src = nullptr;  // while an explicit / stabilised step is enqueued: its u^n
    // page-locked host words the status and reduction results come back into
    // (one copy engine transfer each, no staging through pageable memory)
    struct host_words {
        double red[6];
        double norm[2]; // power-method norms
        double pm_rho;  // the graph form of the power method: 1.2 x the estimate
        int pm_iters;   // and its iterations (negative: not settled)
        int status;
    } *h_words = nullptr;
    // captured reductions (kernels + copies of the results and the status word),
    // one per state buffer the FP32K high part alternates between
    struct red_graph {
        const void *state;
        cudaGraphExec_t gexec;
    } red_graphs[2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    double flux_c = 0.0;            // FRGPU_FLUX_CENTRAL dissipation coefficient
    void *d_c2 = nullptr;           // FRGPU_FLUX_CENTRAL work: transformed fluxes and face traces
    size_t c2_cap = 0;              // values d_c2 holds
    int fuse_indicator = 1;         // FP32K 2D: learned indicator inside stage 3
    int fuse_erk = 1;               // 2D Euler: two-stage tableaux fused into the stage kernel
    fr_method meth;                 // coefficients of the fused step
    int limiter = 0;                // positivity-preserving limiter before every step
    double lim_t0 = 1.0;            // its t0 (cap of the energy scaling)
    std::vector<double> lim_w;      // its element weights
    // explicit Runge-Kutta stepping (erk.cu): tableau, k buffers + stage buffer, step graph
    int erk_s = 0;
    std::vector<double> erk_A, erk_b;
    void *d_erk = nullptr;
    size_t erk_cap = 0; // stages d_erk holds
    cudaGraphExec_t erk_gexec = nullptr;
    long erk_launches = 0; // kernels per captured ERK step
    bool erk_dirty = true;
    const void *erk_hi = nullptr; // the high part the ERK graph updates
    // stabilised stepping (erk.cu): buffers, captured step graphs per coefficient set
    void *d_rock = nullptr;
    size_t rock_cap = 0; // values d_rock holds
    struct rock_graph {
        std::vector<double> key;
        const void *hi; // the high part it updates
        cudaGraphExec_t gexec;
        long launches;
    };
    std::vector<rock_graph> rock_graphs; // most recently used last
    // nonlinear power method: direction of the last estimate, work vectors, norm partials
    void *d_eig = nullptr; // 4 n values: direction, v, f(u), f(v)
    // the warm-started power method as one graph (a while-loop node over the
    // iterations), per state buffer and iteration limit
    struct pm_graph {
        const void *u;
        int maxiter;
        cudaGraphExec_t gexec;
        long pro, body, epi; // kernels of the prologue, of one iteration, of the epilogue
    };
    std::vector<pm_graph> pm_graphs;
    struct fr_power_ctl *d_pm = nullptr;
    bool have_eig = false;
    double *d_eig_red = nullptr; // FR_RED_BLOCKS partials + the last-block counter
    std::map<int, std::vector<double>> rkc2_cache; // frgpu_step_rkc2: s -> alpha, beta, mu, delta, bound
    double rkc2_eps = -1.0;
    float *d_bgk_prim = nullptr;    // FP32 BGK: (rho, U, lambda) per (element, point), from the moments
    uint32_t *d_bgk_frag = nullptr; // FP32 BGK: TF32 A fragments of the transport operator (both signs, split)
    // captured step graph
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    int graph_ind = -1;
    long graph_launches = 0; // kernels per captured step
    double host_dt = -1.0;
    long launches = 0;
};

constexpr int FR_NCOUNT = 8, FR_COUNT_LIMITER = 4; // d_count entries
constexpr int FR_ERK_MAXS = 16;                     // stages of an explicit Runge-Kutta tableau
constexpr int FR_ROCK_MAXM = 4096;                  // recurrence stages of a stabilised step
constexpr int FR_ROCK_GRAPHS = 8;                   // stabilised-step graphs kept per problem
constexpr int FR_RED_BLOCKS = 608; // reduction partial blocks (4 x 152 SMs)
// d_red layout: [FR_RED_BLOCKS*6 partials][8 final][64 quadrature weights]
constexpr int FR_RED_FINAL = FR_RED_BLOCKS * 6;
constexpr int FR_RED_WP = FR_RED_BLOCKS * 6 + 8;
constexpr int FR_RED_SIZE = FR_RED_BLOCKS * 6 + 8 + 64;

// Devices a process may drive (per-device caches below).
constexpr int FR_MAX_DEVICES = 64;

// Current u^n buffers of a problem (FP32K ping-pongs the high part).
inline void *fr_state_hi(frgpu_problem *p) { return p->parity ? p->s1 : p->s0; }
inline void *fr_state_tmp(frgpu_problem *p) { return p->parity ? p->s0 : p->s1; }

// Thread-local error handling.
void fr_set_error(const std::string &msg);
int fr_cuda_fail(cudaError_t e, const char *what);
#define FR_CUDA(call)                                                                                              \
    do {                                                                                                           \
        cudaError_t _e = (call);                                                                                   \
        if (_e != cudaSuccess) return fr_cuda_fail(_e, #call);                                                     \
    } while (0)

// The dynamic shared-memory opt-in of one kernel, as raised on each device:
// cudaFuncSetAttribute acts on the current device only, so a process that
// launches the kernel on a second GPU must raise it there too.  Static
// instances start at zero.
struct fr_smem_optin {
    std::atomic<size_t> bytes[FR_MAX_DEVICES];
};
template <class Kern> inline int fr_raise_smem(Kern kern, size_t need, fr_smem_optin &st, bool force = false) {
    int dev = 0;
    FR_CUDA(cudaGetDevice(&dev));
    const bool known = dev >= 0 && dev < FR_MAX_DEVICES;
    if (!force && known && st.bytes[dev].load(std::memory_order_acquire) >= need) return 0;
    FR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need));
    if (known) {
        size_t cur = st.bytes[dev].load(std::memory_order_acquire);
        while (cur < need && !st.bytes[dev].compare_exchange_weak(cur, need, std::memory_order_acq_rel)) {
        }
    }
    return 0;
}

// Setup math (setup.cpp)
namespace frsetup {
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w);
double dlegendre(int n, double x);
void lagrange_point(const double *sp, int nsp, double x, double *l);
void dlagrange(const double *sp, int nsp, double *lpdm);
void dcorrection(int kind, int deg, const double *x, int n, double *dgl, double *dgr);
double jacobi_orthonormal(int n, double x);
void vandermonde(int deg, const double *r, int n, double *V);
void vandermonde_quad(int deg, const double *r, const double *s, int n, double *V);
bool invert(int n, const double *A, double *Ainv);
void vandermonde_tri(int deg, const double *r, const double *s, int n, double *V, double *Vr, double *Vs);
void triface_points(int deg, double *pr, double *ps, double *wf);
void tri_operators(int deg, const double *r, const double *s, double *V, double *dl, double *lf, double *phi);
void build_1d(frgpu_space &s, int correction);
void build_2d(frgpu_space &s);
} // namespace frsetup

// Kernel launchers (return FRGPU_OK or an error; stage 0 = residual only)
// euler2d.cu
int fr_launch_euler2d(frgpu_problem *p, int stage, const void *in, const void *din, void *out);
// the sums and speeds; with status non-null the device status word comes back
// in the same synchronisation.  Replayed from a captured graph per state buffer.
void fr_drop_reduce_graphs(frgpu_problem *p);
int fr_launch_euler2d_reduce(frgpu_problem *p, const void *state, const void *lo, double *out_sums,
                             double *out_speed, double cfl_dx, double cfl_dy, int *status = nullptr);
// scalar1d.cu
int fr_launch_scalar1d(frgpu_problem *p, int stage, const void *in, const void *din, void *out);
int fr_launch_euler1d(frgpu_problem *p, int stage, const void *in, const void *din, void *out);
int fr_launch_bgk1d(frgpu_problem *p, int stage, const void *in, const void *din, void *out);
int fr_launch_bgk1d_tc(frgpu_problem *p, int stage, const void *in, const void *din, void *out);
int fr_bgk_tc_setup(frgpu_problem *p); // device buffers of the tensor-core BGK path
// Host FP64 state (reference layout) <-> device state (transfer.cu)
int fr_put_state(frgpu_problem *p, const double *u, void *hi, void *lo);
int fr_get_state(frgpu_problem *p, const void *hi, const void *lo, double *u);
int fr_launch_interp_face(const double *d_f, long n, int np, const double *ll, const double *lr, double *d_out,
                          cudaStream_t st);
int fr_launch_poly_derivative(const double *d_f, long n, int np, const double *pdm, double *d_out,
                              cudaStream_t st);
// filter.cu
int fr_launch_filter2d(frgpu_problem *p, int indicator, double lam, double S0, double kappa);
int fr_launch_filter1d(frgpu_problem *p, int indicator, double lam, double S0, double kappa);
// mlp.cu
int fr_launch_features(frgpu_problem *p, float *d_feat);
// Device pointers of a network (FP32 parameters, BF16 W1 [64][32], W2 and W2^T [64][64],
// and the copy packed for the tcgen05 path).
struct fr_mlp_ptrs {
    const float *P;
    const void *W1, *W2, *W2T;
    const unsigned char *TC; // packed for the tcgen05 path
};
fr_mlp_ptrs fr_mlp_device(const frgpu_mlp *m);
// 1D factor iV1[i][k] (row-major 4 x 4, float) of a deg-3 2D space's tensor inverse Vandermonde matrix
void fr_iv1_from_tensor(const frgpu_space &s, float *iv1);
// Which indicator stage 3 of this problem runs itself (FP32K 2D Euler, deg 3,
// uniform rectangles, fusion not switched off): FRGPU_IND_MLP (a network bound
// and selected), FRGPU_IND_PLAIN, or FRGPU_IND_NONE (the filter, if any, runs
// as its own kernel after the step).
int fr_fused_indicator(const frgpu_problem *p);
int fr_launch_mlp_indicator(frgpu_problem *p, double lam, double S0, double kappa);
// positivity-preserving limiter (limiter.cu)
int fr_launch_limiter(frgpu_problem *p, const std::vector<double> &w, double t0);
int fr_limiter_weights(const frgpu_problem *p, const double *weights, std::vector<double> &w);
// explicit Runge-Kutta step (erk.cu); launch_residual evaluates k = L(in)
int fr_enqueue_erk_step(frgpu_problem *p, int (*launch_residual)(frgpu_problem *, const void *, void *));
// One explicit Runge-Kutta step over raw device buffers (erk.cu).
struct fr_erk_raw {
    cudaStream_t stream;
    int s;                      // stages
    const double *A, *b;        // host tableau, A row-major s x s
    size_t n;                   // values in the state
    bool f32;                   // FP32 state with compensated update into lo
    void *u, *lo;               // state (high part) and FP32 low part (null for FP64)
    char *kbuf;                 // (s + 1) n values: k_0 .. k_{s-1}, stage input
    size_t esize;               // bytes per value
    const double *d_dt;         // device dt
    int *d_status;              // device status flags
    bool prepare_only;          // launch nothing but the residual's preparation
    long *launches;             // incremented per kernel enqueued
};
int fr_erk_enqueue_raw(const fr_erk_raw &r, int (*residual)(void *, const void *, void *), void *ctx);
// One stabilised step (three-term recurrence + finishing tableau) over raw
// device buffers (erk.cu).
struct fr_rock_raw {
    cudaStream_t stream;
    int m;                                       // recurrence stages
    const double *alpha, *beta, *mu, *delta;     // host coefficients [m]
    int sf;                                      // finishing stages (0: none)
    const double *A, *b;                         // host finishing tableau, A row-major sf x sf
    size_t n;                                    // values in the state
    bool f32;                                    // FP32 state with compensated update into lo
    void *u, *lo;                                // state (high part) and FP32 low part (null for FP64)
    char *buf;                                   // (7 + sf) n values: D x 3, F0, F, Y, stage input, k_0..
    const double *d_dt;
    int *d_status;
    bool prepare_only;
    long *launches;
};
int fr_rock_enqueue_raw(const fr_rock_raw &r, int (*residual)(void *, const void *, void *), void *ctx);
// vector helpers of the nonlinear power method (erk.cu)
// residual of a FRGPU_FLUX_CENTRAL 2D problem (central2d.cu)
int fr_launch_central2d(frgpu_problem *p, int stage, const void *in, void *out);
int fr_vec_axpy(cudaStream_t st, bool f32, size_t n, void *out, const void *x, const void *y, double c);
int fr_vec_axpy_diff(cudaStream_t st, bool f32, size_t n, void *out, const void *x, const void *a, const void *b,
                     double c); // out = x + c (a - b)
int fr_vec_fill(cudaStream_t st, bool f32, size_t n, void *v, double c);
int fr_vec_flip(cudaStream_t st, bool f32, void *v, const void *u, size_t i);
// Device state of the graph form of the power method (erk.cu).
struct fr_power_ctl {
    double ynrm, vnrm, dfnrm, dynrm, sigma, coef;
    long flip;
    int it, done, converged, maxiter, mode;
};
int fr_pm_start(cudaStream_t st, fr_power_ctl *ctl, size_t n, double uround, double sq, int maxiter);
int fr_pm_vinit(cudaStream_t st, bool f32, size_t n, void *v, const void *u, const void *d0, const fr_power_ctl *ctl);
int fr_pm_step(cudaStream_t st, fr_power_ctl *ctl, size_t n, cudaGraphConditionalHandle h);
int fr_pm_update(cudaStream_t st, bool f32, size_t n, void *v, const void *u, const void *fv, const void *fu,
                 const fr_power_ctl *ctl);
int fr_pm_finish(cudaStream_t st, const fr_power_ctl *ctl, double *host_rho, int *host_iters);
int fr_vec_norm2(cudaStream_t st, bool f32, size_t n, const void *x, const void *y, double *d_part, unsigned *cnt,
                 double *host_out, const int *d_status, int *host_status);
int fr_vec_norm2_to(cudaStream_t st, bool f32, size_t n, const void *x, const void *y, double *d_part, unsigned *cnt,
                    double *dev_out, const int *d_status, int *host_status);
