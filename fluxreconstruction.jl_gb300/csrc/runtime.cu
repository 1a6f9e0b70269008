// runtime.cu -- the C ABI of libfrgpu.so: spaces, problems, device memory,
// streams, captured SSPRK3 step graphs, error handling.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "frgpu_internal.h"

static thread_local std::string g_err;

void fr_set_error(const std::string &msg) { g_err = msg; }
int fr_cuda_fail(cudaError_t e, const char *what) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return FRGPU_ERR_CUDA;
}

#define FR_TRY try {
#define FR_CATCH                                                                                                   \
    }                                                                                                              \
    catch (const std::exception &ex) {                                                                             \
        fr_set_error(ex.what());                                                                                   \
        return FRGPU_ERR_ARG;                                                                                      \
    }                                                                                                              \
    catch (...) {                                                                                                  \
        fr_set_error("unknown C++ exception");                                                                     \
        return FRGPU_ERR_ARG;                                                                                      \
    }

#define FR_REQ(cond, msg)                                                                                          \
    do {                                                                                                           \
        if (!(cond)) {                                                                                             \
            fr_set_error(msg);                                                                                     \
            return FRGPU_ERR_ARG;                                                                                  \
        }                                                                                                          \
    } while (0)

extern "C" {

FRGPU_API int frgpu_version(void) { return 100; }

FRGPU_API int frgpu_last_error(char *buf, unsigned long n) {
    if (!buf || n == 0) return (int)g_err.size();
    std::snprintf(buf, n, "%s", g_err.c_str());
    return (int)g_err.size();
}

// ------------------------------------------------------------------ setup math
FRGPU_API int frgpu_legendre_point(int deg, double *r, double *w) {
    FR_REQ(deg >= 0 && deg < 64 && r, "legendre_point: bad arguments");
    FR_TRY
    std::vector<double> x, wt;
    frsetup::gauss_legendre(deg + 1, x, wt);
    std::memcpy(r, x.data(), sizeof(double) * (deg + 1));
    if (w) std::memcpy(w, wt.data(), sizeof(double) * (deg + 1));
    return FRGPU_OK;
    FR_CATCH
}

FRGPU_API int frgpu_lagrange_point(const double *sp, int nsp, double x, double *l) {
    FR_REQ(sp && l && nsp > 0, "lagrange_point: bad arguments");
    frsetup::lagrange_point(sp, nsp, x, l);
    return FRGPU_OK;
}

FRGPU_API int frgpu_dlagrange(const double *sp, int nsp, double *lpdm) {
    FR_REQ(sp && lpdm && nsp > 0, "dlagrange: bad arguments");
    frsetup::dlagrange(sp, nsp, lpdm);
    return FRGPU_OK;
}

FRGPU_API int frgpu_dcorrection(int correction, int deg, const double *x, int n, double *dgl, double *dgr) {
    FR_REQ(x && dgl && dgr && n > 0 && deg >= 1, "dcorrection: bad arguments");
    FR_REQ(correction >= FRGPU_RADAU && correction <= FRGPU_HUYNH, "dcorrection: unknown correction");
    frsetup::dcorrection(correction, deg, x, n, dgl, dgr);
    return FRGPU_OK;
}

FRGPU_API int frgpu_vandermonde(int deg, const double *r, int n, double *V) {
    FR_REQ(r && V && n > 0 && deg >= 0, "vandermonde: bad arguments");
    frsetup::vandermonde(deg, r, n, V);
    return FRGPU_OK;
}

FRGPU_API int frgpu_vandermonde_quad(int deg, const double *r, const double *s, int n, double *V) {
    FR_REQ(r && s && V && n > 0 && deg >= 0, "vandermonde_quad: bad arguments");
    frsetup::vandermonde_quad(deg, r, s, n, V);
    return FRGPU_OK;
}

// ------------------------------------------------------------------ spaces
FRGPU_API int frgpu_space_create_1d(double x0, double x1, int nx, int deg, int correction, frgpu_space **out) {
    FR_REQ(out, "space_create_1d: null output");
    *out = nullptr;
    FR_REQ(nx >= 1 && deg >= 1 && deg <= 5, "space_create_1d: need nx >= 1 and 1 <= deg <= 5");
    FR_REQ(x1 > x0, "space_create_1d: need x1 > x0");
    FR_REQ(correction >= FRGPU_RADAU && correction <= FRGPU_HUYNH, "space_create_1d: unknown correction");
    FR_TRY
    auto *s = new frgpu_space();
    s->dim = 1;
    s->nx = nx;
    s->ny = 1;
    s->deg = deg;
    s->np = deg + 1;
    s->x0 = x0;
    s->x1 = x1;
    frsetup::build_1d(*s, correction);
    *out = s;
    return FRGPU_OK;
    FR_CATCH
}

FRGPU_API int frgpu_space_create_2d(double x0, double x1, int nx, double y0, double y1, int ny, int deg,
                                    frgpu_space **out) {
    FR_REQ(out, "space_create_2d: null output");
    *out = nullptr;
    FR_REQ(nx >= 1 && ny >= 1 && deg >= 1 && deg <= 5, "space_create_2d: need nx, ny >= 1 and 1 <= deg <= 5");
    FR_REQ(x1 > x0 && y1 > y0, "space_create_2d: empty domain");
    FR_TRY
    auto *s = new frgpu_space();
    s->dim = 2;
    s->nx = nx;
    s->ny = ny;
    s->deg = deg;
    s->np = deg + 1;
    s->x0 = x0;
    s->x1 = x1;
    s->y0 = y0;
    s->y1 = y1;
    frsetup::build_2d(*s);
    *out = s;
    return FRGPU_OK;
    FR_CATCH
}

static void copy_ops(frgpu_space &s, const double *ll, const double *lr, const double *dl, const double *dhl,
                     const double *dhr, const double *V, const double *iV, int nV) {
    const int np = s.np;
    s.ll.assign(ll, ll + np);
    s.lr.assign(lr, lr + np);
    s.dl.assign(dl, dl + np * np);
    s.dhl.assign(dhl, dhl + np);
    s.dhr.assign(dhr, dhr + np);
    if (V) s.V.assign(V, V + nV * nV);
    if (iV) s.iV.assign(iV, iV + nV * nV);
}

FRGPU_API int frgpu_space_create_1d_ops(int nx, int deg, const double *J, const double *ll, const double *lr,
                                        const double *dl, const double *dhl, const double *dhr, const double *V,
                                        const double *iV, frgpu_space **out) {
    FR_REQ(out, "space_create_1d_ops: null output");
    *out = nullptr;
    FR_REQ(nx >= 1 && deg >= 1 && deg <= 5 && J && ll && lr && dl && dhl && dhr, "space_create_1d_ops: bad arguments");
    FR_TRY
    auto *s = new frgpu_space();
    s->dim = 1;
    s->nx = nx;
    s->deg = deg;
    s->np = deg + 1;
    std::vector<double> w;
    frsetup::gauss_legendre(s->np, s->xpl, s->w1);
    s->wp = s->w1;
    s->J.assign(J, J + nx);
    copy_ops(*s, ll, lr, dl, dhl, dhr, V, iV, s->np);
    double len = 0;
    for (int i = 0; i < nx; ++i) len += 2 * J[i];
    s->x0 = 0;
    s->x1 = len;
    s->dx = len / nx;
    s->xc.resize(nx);
    double x = 0;
    for (int i = 0; i < nx; ++i) {
        s->xc[i] = x + J[i];
        x += 2 * J[i];
    }
    *out = s;
    return FRGPU_OK;
    FR_CATCH
}

FRGPU_API int frgpu_space_create_2d_ops(int nx, int ny, int deg, double dx, double dy, const double *ll,
                                        const double *lr, const double *dl, const double *dhl, const double *dhr,
                                        const double *V, const double *iV, frgpu_space **out) {
    FR_REQ(out, "space_create_2d_ops: null output");
    *out = nullptr;
    FR_REQ(nx >= 1 && ny >= 1 && deg >= 1 && deg <= 5 && dx > 0 && dy > 0 && ll && lr && dl && dhl && dhr,
           "space_create_2d_ops: bad arguments");
    FR_TRY
    auto *s = new frgpu_space();
    s->dim = 2;
    s->nx = nx;
    s->ny = ny;
    s->deg = deg;
    s->np = deg + 1;
    frsetup::gauss_legendre(s->np, s->xpl, s->w1);
    s->wp.resize(s->np * s->np);
    for (int l = 0; l < s->np; ++l)
        for (int k = 0; k < s->np; ++k) s->wp[k + s->np * l] = s->w1[k] * s->w1[l];
    copy_ops(*s, ll, lr, dl, dhl, dhr, V, iV, s->np * s->np);
    s->x0 = 0;
    s->x1 = dx * nx;
    s->y0 = 0;
    s->y1 = dy * ny;
    s->dx = dx;
    s->dy = dy;
    s->xc.resize(nx);
    s->yc.resize(ny);
    for (int i = 0; i < nx; ++i) s->xc[i] = (i + 0.5) * dx;
    for (int j = 0; j < ny; ++j) s->yc[j] = (j + 0.5) * dy;
    *out = s;
    return FRGPU_OK;
    FR_CATCH
}

FRGPU_API int frgpu_space_info(const frgpu_space *s, int *dim, int *nx, int *ny, int *deg) {
    FR_REQ(s, "space_info: null space");
    if (dim) *dim = s->dim;
    if (nx) *nx = s->nx;
    if (ny) *ny = s->ny;
    if (deg) *deg = s->deg;
    return FRGPU_OK;
}

FRGPU_API int frgpu_space_get(const frgpu_space *s, const char *name, double *out, long n) {
    FR_REQ(s && name && out, "space_get: null argument");
    FR_TRY
    std::vector<double> tmp;
    const std::vector<double> *v = nullptr;
    std::string k(name);
    if (k == "xpl") v = &s->xpl;
    else if (k == "wp") v = &s->wp;
    else if (k == "ll") v = &s->ll;
    else if (k == "lr") v = &s->lr;
    else if (k == "dl") v = &s->dl;
    else if (k == "dhl") v = &s->dhl;
    else if (k == "dhr") v = &s->dhr;
    else if (k == "V") v = &s->V;
    else if (k == "iV") v = &s->iV;
    else if (k == "J") v = &s->J;
    else if (k == "xpg") {
        // global solution points, src/Geometry/geo_points.jl:8-15 (1D, xpg[i, k]);
        // 2D: xpg[i, j, k, l, 1:2] of src/struct.jl:161-175 on rectangles
        const int np = s->np;
        if (s->dim == 1) {
            tmp.resize((size_t)s->nx * np);
            for (int kk = 0; kk < np; ++kk)
                for (int i = 0; i < s->nx; ++i) {
                    // r_x (src/Geometry/geo_transform.jl:7): ((1-r)/2) x_l + ((1+r)/2) x_r
                    const double J = s->J.empty() ? 0.5 * s->dx : s->J[i];
                    const double xl = s->xc[i] - J, xr = s->xc[i] + J, r = s->xpl[kk];
                    tmp[i + (size_t)s->nx * kk] = ((1.0 - r) / 2.0) * xl + ((1.0 + r) / 2.0) * xr;
                }
        } else {
            const size_t nn = (size_t)s->nx * s->ny;
            tmp.resize(nn * np * np * 2);
            for (int d = 0; d < 2; ++d)
                for (int l = 0; l < np; ++l)
                    for (int kk = 0; kk < np; ++kk)
                        for (int j = 0; j < s->ny; ++j)
                            for (int i = 0; i < s->nx; ++i) {
                                double val = d == 0 ? s->xc[i] + 0.5 * s->dx * s->xpl[kk]
                                                    : s->yc[j] + 0.5 * s->dy * s->xpl[l];
                                tmp[i + (size_t)s->nx * j + nn * (kk + np * (l + (size_t)np * d))] = val;
                            }
        }
        v = &tmp;
    } else {
        fr_set_error("space_get: unknown field '" + k + "'");
        return FRGPU_ERR_ARG;
    }
    FR_REQ((long)v->size() <= n, "space_get: output too small");
    std::memcpy(out, v->data(), sizeof(double) * v->size());
    return (int)v->size();
    FR_CATCH
}

FRGPU_API void frgpu_space_destroy(frgpu_space *s) { delete s; }

} // extern "C"

// ------------------------------------------------------------------ problems
static void drop_rock_graphs(frgpu_problem *p) {
    for (auto &g : p->rock_graphs)
        if (g.gexec) cudaGraphExecDestroy(g.gexec);
    p->rock_graphs.clear();
    for (auto &g : p->pm_graphs)
        if (g.gexec) cudaGraphExecDestroy(g.gexec);
    p->pm_graphs.clear();
}

static void free_problem(frgpu_problem *p) {
    if (!p) return;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(p->device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    for (auto &g : p->gexec)
        if (g) cudaGraphExecDestroy(g);
    if (p->erk_gexec) cudaGraphExecDestroy(p->erk_gexec);
    drop_rock_graphs(p);
    fr_drop_reduce_graphs(p);
    void *bufs[] = {p->s0,     p->s1,      p->s2,         p->s3,      p->d_dt,      p->d_status, p->d_red,
                    p->d_flags, p->d_count, p->d_velo,     p->d_w,     p->d_J,       p->d_V,      p->d_iV,
                    p->rhs_in, p->rhs_out, p->d_bgk_prim, p->d_bgk_frag, p->d_stage, p->d_erk,   p->d_met,
                    p->d_nfx,  p->d_nfy,   p->d_fsc,      p->d_rock,  p->d_eig,     p->d_eig_red, p->d_c2,
                    p->d_pm};
    for (void *b : bufs)
        if (b) cudaFree(b);
    if (p->stream) cudaStreamDestroy(p->stream);
    if (p->h_words) cudaFreeHost(p->h_words);
    cudaSetDevice(cur);
    delete p;
}

template <class T> static int upload_as(void **dst, const std::vector<double> &src) {
    std::vector<T> tmp(src.begin(), src.end());
    FR_CUDA(cudaMalloc(dst, sizeof(T) * (tmp.empty() ? 1 : tmp.size())));
    if (!tmp.empty()) FR_CUDA(cudaMemcpy(*dst, tmp.data(), sizeof(T) * tmp.size(), cudaMemcpyHostToDevice));
    return FRGPU_OK;
}

static int upload_vec(frgpu_problem *p, void **dst, const std::vector<double> &src) {
    return p->esize == 8 ? upload_as<double>(dst, src) : upload_as<float>(dst, src);
}

// The error a device status word st stands for (0: none); resets the word.
static int status_error(frgpu_problem *p, int st) {
    if (st == 0) return FRGPU_OK;
    FR_CUDA(cudaMemsetAsync(p->d_status, 0, sizeof(int), p->stream));
    if (st & 1) {
        fr_set_error("non-finite value in the state");
        return FRGPU_ERR_NONFINITE;
    }
    if (st & 2) {
        fr_set_error("non-positive density or pressure in the state");
        return FRGPU_ERR_UNPHYSICAL;
    }
    fr_set_error("device-side wait timed out");
    return FRGPU_ERR_TIMEOUT;
}

static int check_status(frgpu_problem *p) {
    FR_CUDA(cudaMemcpyAsync(&p->h_words->status, p->d_status, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
    FR_CUDA(cudaStreamSynchronize(p->stream));
    return status_error(p, p->h_words->status);
}

static int launch_stage(frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    switch (p->d.equation) {
    case FRGPU_ADVECTION:
    case FRGPU_BURGERS: return fr_launch_scalar1d(p, stage, in, din, out);
    case FRGPU_EULER1D: return fr_launch_euler1d(p, stage, in, din, out);
    case FRGPU_EULER2D: return fr_launch_euler2d(p, stage, in, din, out);
    case FRGPU_BGK1D: return fr_launch_bgk1d(p, stage, in, din, out);
    }
    fr_set_error("unknown equation");
    return FRGPU_ERR_ARG;
}

// One SSPRK3 step (limiter before it, filter after it, the order of the loop
// of example/shock-vortex.jl:297-321) on the current buffers.
static int enqueue_step(frgpu_problem *p) {
    int rc;
    if (p->limiter && (rc = fr_launch_limiter(p, p->lim_w, p->lim_t0))) return rc;
    const bool two = p->meth.stages == 2; // stages 1 and 3 only (2D Euler)
    if (p->d.precision == FRGPU_FP64) {
        if ((rc = launch_stage(p, 1, p->s0, nullptr, p->s1))) return rc;
        if (!two && (rc = launch_stage(p, 2, p->s1, nullptr, p->s2))) return rc;
        if ((rc = launch_stage(p, 3, two ? p->s1 : p->s2, nullptr, p->s0))) return rc;
    } else {
        // the last stage reads its increment from s2 and writes the new high
        // part into the other buffer
        void *hi = fr_state_hi(p), *tmp = fr_state_tmp(p);
        if ((rc = launch_stage(p, 1, hi, nullptr, two ? p->s2 : tmp))) return rc;
        if (!two && (rc = launch_stage(p, 2, hi, tmp, p->s2))) return rc;
        if ((rc = launch_stage(p, 3, hi, p->s2, tmp))) return rc;
    }
    if (p->indicator != FRGPU_IND_NONE && !fr_fused_indicator(p)) {
        // the filter runs on the new state: for FP32K that is the buffer the
        // high part moves to, so evaluate with the parity flipped
        if (p->d.precision == FRGPU_FP32K) p->parity ^= 1;
        rc = p->sp.dim == 2 ? fr_launch_filter2d(p, p->indicator, p->lam, p->S0, p->kappa)
                            : fr_launch_filter1d(p, p->indicator, p->lam, p->S0, p->kappa);
        if (p->d.precision == FRGPU_FP32K) p->parity ^= 1;
        if (rc) return rc;
    }
    return FRGPU_OK;
}

// One explicit Runge-Kutta step (limiter before it, filter after it).
static int residual_into(frgpu_problem *p, const void *in, void *out) { return launch_stage(p, 0, in, nullptr, out); }

// u^n of a step, for residual evaluations whose ghosts stay at the step's start
static const void *step_start_state(frgpu_problem *p) {
    return p->ghosts_per_step && p->d.equation == FRGPU_EULER2D ? fr_state_hi(p) : nullptr;
}

static int enqueue_erk(frgpu_problem *p) {
    int rc;
    if (p->limiter && (rc = fr_launch_limiter(p, p->lim_w, p->lim_t0))) return rc;
    p->lag_src = step_start_state(p);
    rc = fr_enqueue_erk_step(p, residual_into);
    p->lag_src = nullptr;
    if (rc) return rc;
    if (p->indicator != FRGPU_IND_NONE) {
        // the high part stays in place (no parity flip); the learned indicator
        // runs as its own kernel (its fused form lives in SSPRK3's stage 3)
        rc = p->sp.dim == 2 ? fr_launch_filter2d(p, p->indicator, p->lam, p->S0, p->kappa)
                            : fr_launch_filter1d(p, p->indicator, p->lam, p->S0, p->kappa);
        if (rc) return rc;
    }
    return FRGPU_OK;
}

static int build_erk_graph(frgpu_problem *p) {
    if (p->erk_gexec) {
        cudaGraphExecDestroy(p->erk_gexec);
        p->erk_gexec = nullptr;
    }
    p->prepare_only = true;
    int rc = enqueue_erk(p);
    p->prepare_only = false;
    if (rc) return rc;
    const long before = p->launches;
    cudaGraph_t g = nullptr;
    FR_CUDA(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
    rc = enqueue_erk(p);
    cudaError_t ce = cudaStreamEndCapture(p->stream, &g);
    p->erk_launches = p->launches - before;
    p->launches = before;
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (ce != cudaSuccess) return fr_cuda_fail(ce, "cudaStreamEndCapture");
    ce = cudaGraphInstantiate(&p->erk_gexec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return fr_cuda_fail(ce, "cudaGraphInstantiate");
    p->erk_dirty = false;
    p->erk_hi = fr_state_hi(p);
    return FRGPU_OK;
}

static int build_graphs(frgpu_problem *p) {
    for (auto &g : p->gexec)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    const int ngraphs = p->d.precision == FRGPU_FP32K ? 2 : 1;
    const int parity0 = p->parity;
    for (int gi = 0; gi < ngraphs; ++gi) {
        p->parity = gi;
        p->prepare_only = true;
        int rc = enqueue_step(p);
        p->prepare_only = false;
        if (rc) {
            p->parity = parity0;
            return rc;
        }
        const long before = p->launches;
        cudaGraph_t g = nullptr;
        FR_CUDA(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
        rc = enqueue_step(p);
        cudaError_t ce = cudaStreamEndCapture(p->stream, &g);
        p->graph_launches = p->launches - before;
        p->launches = before;
        if (rc) {
            if (g) cudaGraphDestroy(g);
            p->parity = parity0;
            return rc;
        }
        if (ce != cudaSuccess) {
            p->parity = parity0;
            return fr_cuda_fail(ce, "cudaStreamEndCapture");
        }
        ce = cudaGraphInstantiate(&p->gexec[gi], g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            p->parity = parity0;
            return fr_cuda_fail(ce, "cudaGraphInstantiate");
        }
    }
    p->parity = parity0;
    p->graph_ind = p->indicator;
    return FRGPU_OK;
}

extern "C" {

FRGPU_API int frgpu_problem_create(const frgpu_space *s, const frgpu_problem_desc *d, frgpu_problem **out) {
    FR_REQ(out, "problem_create: null output");
    *out = nullptr;
    FR_REQ(s && d, "problem_create: null space or description");
    FR_REQ(d->precision == FRGPU_FP64 || d->precision == FRGPU_FP32K, "problem_create: unknown precision");
    const int eq = d->equation;
    FR_REQ(eq >= FRGPU_ADVECTION && eq <= FRGPU_BGK1D, "problem_create: unknown equation");
    FR_REQ((eq == FRGPU_EULER2D) == (s->dim == 2), "problem_create: equation and space dimension disagree");
    FR_REQ(s->np >= 2 && s->np <= 6, "problem_create: polynomial degree must be 1..5");
    if (eq == FRGPU_EULER1D || eq == FRGPU_EULER2D) FR_REQ(d->gamma > 1.0, "problem_create: need gamma > 1");
    if (eq == FRGPU_BGK1D)
        FR_REQ(d->nvel >= 1 && d->velo && d->weights && d->tau > 0, "problem_create: BGK needs nvel, velo, weights, tau");
    if (eq == FRGPU_EULER2D) {
        FR_REQ(d->flux == FRGPU_FLUX_LF || d->flux == FRGPU_FLUX_HLL || d->flux == FRGPU_FLUX_CENTRAL,
               "problem_create: 2D Euler fluxes are LF, HLL or central");
        if (d->flux == FRGPU_FLUX_CENTRAL) {
            for (int side = 0; side < 4; ++side)
                FR_REQ(d->bc[side] == FRGPU_BC_PERIODIC || d->bc[side] == FRGPU_BC_DIRICHLET,
                       "problem_create: with the central flux the boundaries are periodic or Dirichlet");
        } else {
            for (int side = 0; side < 4; ++side)
                FR_REQ(d->bc[side] == FRGPU_BC_PERIODIC || d->bc[side] == FRGPU_BC_COPY ||
                           d->bc[side] == FRGPU_BC_FIXED,
                       "problem_create: 2D boundaries are periodic, copy or fixed");
        }
        FR_REQ((d->bc[0] == FRGPU_BC_PERIODIC) == (d->bc[1] == FRGPU_BC_PERIODIC) &&
                   (d->bc[2] == FRGPU_BC_PERIODIC) == (d->bc[3] == FRGPU_BC_PERIODIC),
               "problem_create: periodic boundaries come in pairs");
        // the 2D kernels address a state array with 32-bit offsets
        FR_REQ((unsigned long long)s->nx * s->ny * s->np * s->np * 4ull < (1ull << 32),
               "problem_create: 2D state exceeds 2^32 values (nx * ny * (deg+1)^2 * 4)");
    } else if (eq == FRGPU_BGK1D) {
        FR_REQ(d->bc[0] == FRGPU_BC_PERIODIC, "problem_create: BGK supports periodic boundaries");
    } else {
        FR_REQ(d->bc[0] == FRGPU_BC_PERIODIC || d->bc[0] == FRGPU_BC_DIRICHLET,
               "problem_create: 1D boundaries are periodic or dirichlet");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        fr_set_error("problem_create: no CUDA device");
        return FRGPU_ERR_CUDA;
    }
    FR_TRY
    auto *p = new frgpu_problem();
    p->sp = *s;
    p->d = *d;
    cudaGetDevice(&p->device);
    p->esize = d->precision == FRGPU_FP64 ? 8 : 4;
    const long np = s->np;
    switch (eq) {
    case FRGPU_ADVECTION:
    case FRGPU_BURGERS: p->ndof = (long)s->nx * np; break;
    case FRGPU_EULER1D: p->ndof = (long)s->nx * np * 3; break;
    case FRGPU_EULER2D: p->ndof = (long)s->nx * s->ny * np * np * 4; break;
    case FRGPU_BGK1D: p->ndof = (long)s->nx * d->nvel * np; break;
    }
    if (eq == FRGPU_BGK1D) {
        p->velo.assign(d->velo, d->velo + d->nvel);
        p->weights.assign(d->weights, d->weights + d->nvel);
        p->d.velo = nullptr;
        p->d.weights = nullptr;
    }
    int rc = FRGPU_OK;
    auto fail = [&](int code) {
        free_problem(p);
        return code;
    };
    if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) {
        fr_set_error("problem_create: cudaStreamCreate failed");
        return fail(FRGPU_ERR_CUDA);
    }
    const size_t bytes = (size_t)p->ndof * p->esize;
    if ((rc = [&]() -> int {
            FR_CUDA(cudaMalloc(&p->s0, bytes));
            FR_CUDA(cudaMalloc(&p->s1, bytes));
            FR_CUDA(cudaMalloc(&p->s2, bytes));
            FR_CUDA(cudaMemset(p->s0, 0, bytes));
            FR_CUDA(cudaMemset(p->s1, 0, bytes));
            FR_CUDA(cudaMemset(p->s2, 0, bytes));
            if (p->d.precision == FRGPU_FP32K) {
                FR_CUDA(cudaMalloc(&p->s3, bytes));
                FR_CUDA(cudaMemset(p->s3, 0, bytes));
            }
            FR_CUDA(cudaMalloc(&p->d_dt, sizeof(double)));
            FR_CUDA(cudaMemset(p->d_dt, 0, sizeof(double)));
            FR_CUDA(cudaMalloc(&p->d_status, sizeof(int)));
            FR_CUDA(cudaMemset(p->d_status, 0, sizeof(int)));
            FR_CUDA(cudaMallocHost((void **)&p->h_words, sizeof(frgpu_problem::host_words)));
            p->h_words->status = 0;
            FR_CUDA(cudaMalloc(&p->d_red, sizeof(double) * FR_RED_SIZE));
            FR_CUDA(cudaMemset(p->d_red, 0, sizeof(double) * FR_RED_SIZE));
            const size_t ne = (size_t)s->nx * s->ny;
            FR_CUDA(cudaMalloc(&p->d_flags, sizeof(int) * ne));
            FR_CUDA(cudaMemset(p->d_flags, 0, sizeof(int) * ne));
            FR_CUDA(cudaMalloc(&p->d_count, sizeof(int) * FR_NCOUNT));
            FR_CUDA(cudaMemset(p->d_count, 0, sizeof(int) * FR_NCOUNT));
            if (!s->wp.empty())
                FR_CUDA(cudaMemcpy(p->d_red + FR_RED_WP, s->wp.data(), sizeof(double) * s->wp.size(),
                                   cudaMemcpyHostToDevice));
            int r2;
            if (s->dim == 1) {
                std::vector<double> J = s->J;
                if (J.empty()) J.assign(s->nx, 0.5 * s->dx);
                if ((r2 = upload_vec(p, &p->d_J, J))) return r2;
            }
            if (!s->V.empty() && (r2 = upload_vec(p, &p->d_V, s->V))) return r2;
            if (!s->iV.empty() && (r2 = upload_vec(p, &p->d_iV, s->iV))) return r2;
            if (eq == FRGPU_BGK1D) {
                if ((r2 = upload_vec(p, &p->d_velo, p->velo))) return r2;
                if ((r2 = upload_vec(p, &p->d_w, p->weights))) return r2;
                if (p->d.precision == FRGPU_FP32K && (r2 = fr_bgk_tc_setup(p))) return r2;
            }
            return FRGPU_OK;
        }()))
        return fail(rc);
    *out = p;
    return FRGPU_OK;
    FR_CATCH
}

FRGPU_API void frgpu_problem_destroy(frgpu_problem *p) { free_problem(p); }

FRGPU_API long frgpu_problem_ndof(const frgpu_problem *p) { return p ? p->ndof : -1; }

// Host (Julia layout, FP64) <-> device layout/precision.
// Host <-> device state conversions run on the GPU (transfer.cu).
static int put_state(frgpu_problem *p, const double *u, void *hi, void *lo) {
    const int rc = fr_put_state(p, u, hi, lo);
    p->launches += 1;
    return rc;
}

static int get_state(frgpu_problem *p, const void *hi, const void *lo, double *u) {
    const int rc = fr_get_state(p, hi, lo, u);
    p->launches += 1;
    return rc;
}

FRGPU_API int frgpu_state_upload(frgpu_problem *p, const double *u) {
    FR_REQ(p && u, "state_upload: null argument");
    FR_TRY
    FR_CUDA(cudaStreamSynchronize(p->stream));
    p->parity = 0;
    return put_state(p, u, p->s0, p->s3);
    FR_CATCH
}

FRGPU_API int frgpu_state_download(frgpu_problem *p, double *u) {
    FR_REQ(p && u, "state_download: null argument");
    FR_TRY
    return get_state(p, fr_state_hi(p), p->s3, u);
    FR_CATCH
}

FRGPU_API int frgpu_rhs(frgpu_problem *p, double *du, const double *u, double t) {
    (void)t; // the residuals are autonomous
    FR_REQ(p && du && u, "rhs: null argument");
    FR_TRY
    const size_t bytes = (size_t)p->ndof * p->esize;
    if (!p->rhs_in) {
        FR_CUDA(cudaMalloc(&p->rhs_in, bytes));
        FR_CUDA(cudaMalloc(&p->rhs_out, bytes));
    }
    int rc = put_state(p, u, p->rhs_in, nullptr);
    if (rc) return rc;
    if ((rc = launch_stage(p, 0, p->rhs_in, nullptr, p->rhs_out))) return rc;
    if ((rc = check_status(p))) return rc;
    return get_state(p, p->rhs_out, nullptr, du);
    FR_CATCH
}

// Replay nsteps fused steps of the problem's method (p->meth) from the step
// graphs; `wait` = 0 enqueues them and leaves the status check to the next
// synchronising call.
static int run_fused_steps(frgpu_problem *p, double dt, int nsteps, bool wait = true) {
    if (dt != p->host_dt) {
        FR_CUDA(cudaMemcpyAsync(p->d_dt, &dt, sizeof(double), cudaMemcpyHostToDevice, p->stream));
        FR_CUDA(cudaStreamSynchronize(p->stream));
        p->host_dt = dt;
    }
    if (!p->gexec[0] || p->graph_ind != p->indicator) {
        int rc = build_graphs(p);
        if (rc) return rc;
    }
    for (int s = 0; s < nsteps; ++s) {
        const int g = p->d.precision == FRGPU_FP32K ? p->parity : 0;
        FR_CUDA(cudaGraphLaunch(p->gexec[g], p->stream));
        if (p->d.precision == FRGPU_FP32K) p->parity ^= 1;
        p->launches += p->graph_launches;
    }
    return wait ? check_status(p) : FRGPU_OK;
}

static void use_method(frgpu_problem *p, const fr_method &m) {
    if (!(m == p->meth)) {
        p->meth = m;
        p->graph_ind = -2; // re-capture the step graphs
    }
}

FRGPU_API int frgpu_step_ssprk3(frgpu_problem *p, double dt, int nsteps) {
    FR_REQ(p, "step_ssprk3: null problem");
    FR_REQ(nsteps >= 0, "step_ssprk3: negative step count");
    if (!(dt > 0.0) || !std::isfinite(dt)) {
        fr_set_error("step_ssprk3: dt must be positive and finite");
        return FRGPU_ERR_DT;
    }
    if (nsteps == 0) return FRGPU_OK;
    FR_TRY
    use_method(p, fr_method());
    return run_fused_steps(p, dt, nsteps);
    FR_CATCH
}

FRGPU_API int frgpu_step_ssprk3_async(frgpu_problem *p, double dt, int nsteps) {
    FR_REQ(p, "step_ssprk3_async: null problem");
    FR_REQ(nsteps >= 0, "step_ssprk3_async: negative step count");
    if (!(dt > 0.0) || !std::isfinite(dt)) {
        fr_set_error("step_ssprk3_async: dt must be positive and finite");
        return FRGPU_ERR_DT;
    }
    if (nsteps == 0) return FRGPU_OK;
    FR_TRY
    use_method(p, fr_method());
    return run_fused_steps(p, dt, nsteps, false);
    FR_CATCH
}

FRGPU_API int frgpu_step_erk(frgpu_problem *p, int s, const double *A, const double *b, double dt, int nsteps) {
    FR_REQ(p && A && b, "step_erk: null argument");
    FR_REQ(s >= 1 && s <= FR_ERK_MAXS, "step_erk: need 1 <= stages <= 16");
    FR_REQ(nsteps >= 0, "step_erk: negative step count");
    for (int i = 0; i < s; ++i)
        for (int j = i; j < s; ++j)
            FR_REQ(A[i * s + j] == 0.0, "step_erk: the tableau must be explicit (A strictly lower triangular)");
    if (!(dt > 0.0) || !std::isfinite(dt)) {
        fr_set_error("step_erk: dt must be positive and finite");
        return FRGPU_ERR_DT;
    }
    if (nsteps == 0) return FRGPU_OK;
    FR_TRY
    // two-stage methods on the 2D Euler problem run fused into the stage kernel
    // (stages 1 and 3 with the method's coefficients, see fr_method)
    if (p->d.equation == FRGPU_EULER2D && s == 2 && A[2] != 0.0 && b[1] != 0.0 && p->fuse_erk &&
        p->d.flux != FRGPU_FLUX_CENTRAL) {
        const double a21 = A[2], b1 = b[0], b2 = b[1];
        fr_method m;
        m.stages = 2;
        m.c1 = a21;
        m.fa = b1 / (a21 * b2);
        m.fs = b2;
        m.g3 = b2;
        m.al3 = b1 / a21;
        m.be3 = 1.0 - b1 / a21;
        m.s3 = 1.0;
        use_method(p, m);
        return run_fused_steps(p, dt, nsteps);
    }
    if (dt != p->host_dt) {
        FR_CUDA(cudaMemcpyAsync(p->d_dt, &dt, sizeof(double), cudaMemcpyHostToDevice, p->stream));
        FR_CUDA(cudaStreamSynchronize(p->stream));
        p->host_dt = dt;
    }
    std::vector<double> Av(A, A + (size_t)s * s), bv(b, b + s);
    if (s != p->erk_s || Av != p->erk_A || bv != p->erk_b) {
        p->erk_s = s;
        p->erk_A = Av;
        p->erk_b = bv;
        p->erk_dirty = true;
    }
    if ((size_t)s > p->erk_cap) {
        FR_CUDA(cudaStreamSynchronize(p->stream));
        if (p->d_erk) cudaFree(p->d_erk);
        p->d_erk = nullptr;
        p->erk_cap = 0;
        FR_CUDA(cudaMalloc(&p->d_erk, (size_t)(s + 1) * p->ndof * p->esize));
        p->erk_cap = s;
        p->erk_dirty = true;
    }
    // the graph updates the high part in place: FP32K SSPRK3 steps in between
    // may have moved it to the other buffer
    if (fr_state_hi(p) != p->erk_hi) p->erk_dirty = true;
    if (p->erk_dirty || !p->erk_gexec) {
        int rc = build_erk_graph(p);
        if (rc) return rc;
    }
    for (int it = 0; it < nsteps; ++it) {
        FR_CUDA(cudaGraphLaunch(p->erk_gexec, p->stream));
        p->launches += p->erk_launches;
    }
    return check_status(p);
    FR_CATCH
}

// ---------------------------------------------------------------- stabilised steps
static int residual_ctx(void *ctx, const void *in, void *out) { return residual_into((frgpu_problem *)ctx, in, out); }

// One stabilised step (limiter before it, filter after it, as for ERK).
static int enqueue_rock(frgpu_problem *p, fr_rock_raw r) {
    int rc;
    if (p->limiter && (rc = fr_launch_limiter(p, p->lim_w, p->lim_t0))) return rc;
    r.prepare_only = p->prepare_only;
    p->lag_src = step_start_state(p);
    rc = fr_rock_enqueue_raw(r, residual_ctx, p);
    p->lag_src = nullptr;
    if (rc) return rc;
    if (p->indicator != FRGPU_IND_NONE) {
        rc = p->sp.dim == 2 ? fr_launch_filter2d(p, p->indicator, p->lam, p->S0, p->kappa)
                            : fr_launch_filter1d(p, p->indicator, p->lam, p->S0, p->kappa);
        if (rc) return rc;
    }
    return FRGPU_OK;
}

static int step_rock_impl(frgpu_problem *p, int m, const double *alpha, const double *beta, const double *mu,
                          const double *delta, int sf, const double *A, const double *b, double dt, int nsteps,
                          bool wait);

FRGPU_API int frgpu_step_rock(frgpu_problem *p, int m, const double *alpha, const double *beta, const double *mu,
                              const double *delta, int sf, const double *A, const double *b, double dt, int nsteps) {
    return step_rock_impl(p, m, alpha, beta, mu, delta, sf, A, b, dt, nsteps, true);
}

// wait = false: the steps are queued and their status is left in the device
// status word for the next synchronising call
static int step_rock_impl(frgpu_problem *p, int m, const double *alpha, const double *beta, const double *mu,
                          const double *delta, int sf, const double *A, const double *b, double dt, int nsteps,
                          bool wait) {
    FR_REQ(p && alpha && beta && mu && delta, "step_rock: null coefficient array");
    FR_REQ(m >= 1 && m <= FR_ROCK_MAXM, "step_rock: need 1 <= recurrence stages <= 4096");
    FR_REQ(sf >= 0 && sf <= FR_ERK_MAXS, "step_rock: need 0 <= finishing stages <= 16");
    FR_REQ(sf == 0 || (A && b), "step_rock: null finishing tableau");
    FR_REQ(nsteps >= 0, "step_rock: negative step count");
    for (int j = 0; j < m; ++j)
        FR_REQ(std::isfinite(alpha[j]) && std::isfinite(beta[j]) && std::isfinite(mu[j]) && std::isfinite(delta[j]),
               "step_rock: recurrence coefficients must be finite");
    for (int i = 0; i < sf; ++i) {
        FR_REQ(std::isfinite(b[i]), "step_rock: finishing weights must be finite");
        for (int j = 0; j < sf; ++j) {
            FR_REQ(std::isfinite(A[i * sf + j]), "step_rock: finishing tableau must be finite");
            FR_REQ(j < i || A[i * sf + j] == 0.0, "step_rock: the finishing tableau must be explicit");
        }
    }
    if (!(dt > 0.0) || !std::isfinite(dt)) {
        fr_set_error("step_rock: dt must be positive and finite");
        return FRGPU_ERR_DT;
    }
    if (nsteps == 0) return FRGPU_OK;
    FR_TRY
    if (dt != p->host_dt) {
        FR_CUDA(cudaMemcpyAsync(p->d_dt, &dt, sizeof(double), cudaMemcpyHostToDevice, p->stream));
        FR_CUDA(cudaStreamSynchronize(p->stream));
        p->host_dt = dt;
    }
    const size_t need = (size_t)(7 + sf) * p->ndof;
    if (need > p->rock_cap) {
        FR_CUDA(cudaStreamSynchronize(p->stream));
        drop_rock_graphs(p);
        if (p->d_rock) cudaFree(p->d_rock);
        p->d_rock = nullptr;
        p->rock_cap = 0;
        FR_CUDA(cudaMalloc(&p->d_rock, need * p->esize));
        p->rock_cap = need;
    }
    std::vector<double> key;
    key.reserve(2 + 4 * (size_t)m + (size_t)sf * (sf + 1));
    key.push_back(m);
    key.push_back(sf);
    for (const double *c : {alpha, beta, mu, delta}) key.insert(key.end(), c, c + m);
    if (sf) {
        key.insert(key.end(), A, A + (size_t)sf * sf);
        key.insert(key.end(), b, b + sf);
    }
    const bool f32 = p->d.precision == FRGPU_FP32K;
    void *hi = fr_state_hi(p);
    int gi = -1;
    for (size_t k = 0; k < p->rock_graphs.size(); ++k)
        if (p->rock_graphs[k].hi == hi && p->rock_graphs[k].key == key) gi = (int)k;
    if (gi >= 0) { // most recently used last
        std::rotate(p->rock_graphs.begin() + gi, p->rock_graphs.begin() + gi + 1, p->rock_graphs.end());
    } else {
        fr_rock_raw r;
        r.stream = p->stream;
        r.m = m;
        r.alpha = alpha;
        r.beta = beta;
        r.mu = mu;
        r.delta = delta;
        r.sf = sf;
        r.A = A;
        r.b = b;
        r.n = (size_t)p->ndof;
        r.f32 = f32;
        r.u = hi;
        r.lo = f32 ? p->s3 : nullptr;
        r.buf = (char *)p->d_rock;
        r.d_dt = p->d_dt;
        r.d_status = p->d_status;
        r.prepare_only = false;
        r.launches = &p->launches;
        p->prepare_only = true;
        int rc = enqueue_rock(p, r);
        p->prepare_only = false;
        if (rc) return rc;
        const long before = p->launches;
        cudaGraph_t g = nullptr;
        FR_CUDA(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
        rc = enqueue_rock(p, r);
        cudaError_t ce = cudaStreamEndCapture(p->stream, &g);
        const long nl = p->launches - before;
        p->launches = before;
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (ce != cudaSuccess) return fr_cuda_fail(ce, "cudaStreamEndCapture");
        cudaGraphExec_t ge = nullptr;
        ce = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return fr_cuda_fail(ce, "cudaGraphInstantiate");
        if ((int)p->rock_graphs.size() >= FR_ROCK_GRAPHS) {
            FR_CUDA(cudaStreamSynchronize(p->stream));
            cudaGraphExecDestroy(p->rock_graphs.front().gexec);
            p->rock_graphs.erase(p->rock_graphs.begin());
        }
        p->rock_graphs.push_back({std::move(key), hi, ge, nl});
    }
    const frgpu_problem::rock_graph &g = p->rock_graphs.back();
    for (int it = 0; it < nsteps; ++it) {
        FR_CUDA(cudaGraphLaunch(g.gexec, p->stream));
        p->launches += g.launches;
    }
    return wait ? check_status(p) : FRGPU_OK;
    FR_CATCH
}

// Nonlinear power method for the spectral radius of the Jacobian of the
// residual at the current state (the estimate of the RKC code, B. P. Sommeijer,
// L. F. Shampine, J. G. Verwer, J. Comput. Appl. Math. 88 (1997) 315-326, that
// the ROCK methods use): v = u + dynrm d / |d|, sigma = |f(v) - f(u)| / dynrm,
// v <- u + (f(v) - f(u)) dynrm / |f(v) - f(u)| until sigma changes by at most
// 1 %, rho = 1.2 sigma.  d starts from the previous call's direction, else f(u).
// The warm-started power method (a direction from the previous call) as one
// graph: the prologue (f(u), the norms of u and of the direction, the start
// vector), a while-loop node whose body is one iteration (f(v), ||f(v) - f(u)||,
// the estimate and its test on the device, which ends the loop, and the update
// of v), and the epilogue (the next direction, rho and the iteration count into
// page-locked host words).  One host synchronisation per call instead of one per
// iteration; the same operations as the host loop, so the same bits.
static int build_pm_graph(frgpu_problem *p, int maxiter, const void *u, frgpu_problem::pm_graph &out) {
    const bool f32 = p->d.precision == FRGPU_FP32K;
    const size_t n = (size_t)p->ndof, es = p->esize;
    char *base = (char *)p->d_eig;
    void *dir = base, *v = base + n * es, *fu = base + 2 * n * es, *fv = base + 3 * n * es;
    cudaStream_t st = p->stream;
    unsigned *cnt = reinterpret_cast<unsigned *>(p->d_eig_red + FR_RED_BLOCKS);
    fr_power_ctl *c = p->d_pm;
    const double uround = f32 ? 0x1p-24 : 0x1p-53, sq = std::sqrt(uround);
    auto norm_to = [&](const void *x, const void *y, double *dev_out) {
        return fr_vec_norm2_to(st, f32, n, x, y, p->d_eig_red, cnt, dev_out, p->d_status, &p->h_words->status);
    };
    cudaGraph_t gp = nullptr, ge = nullptr, g = nullptr;
    auto cleanup = [&]() {
        for (cudaGraph_t x : {gp, ge, g})
            if (x) cudaGraphDestroy(x);
    };
    const long l0 = p->launches;
    int rc = FRGPU_OK;
    cudaError_t ce;
    // prologue
    FR_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    rc = residual_into(p, u, fu);
    if (!rc) rc = norm_to(u, nullptr, &c->ynrm);
    if (!rc) rc = norm_to(dir, nullptr, &c->vnrm);
    if (!rc) rc = fr_pm_start(st, c, n, uround, sq, maxiter);
    if (!rc) rc = fr_pm_vinit(st, f32, n, v, u, dir, c);
    ce = cudaStreamEndCapture(st, &gp);
    const long pro = p->launches - l0 + 4;
    if (rc || ce != cudaSuccess) {
        p->launches = l0;
        cleanup();
        return rc ? rc : fr_cuda_fail(ce, "power method graph: prologue capture");
    }
    // the while-loop over the iterations
    cudaGraphNode_t npro = nullptr, ncond = nullptr, nepi = nullptr;
    cudaGraphConditionalHandle h;
    cudaGraphNodeParams cp = {};
    if ((ce = cudaGraphCreate(&g, 0)) != cudaSuccess ||
        (ce = cudaGraphAddChildGraphNode(&npro, g, nullptr, 0, gp)) != cudaSuccess ||
        (ce = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess) {
        p->launches = l0;
        cleanup();
        return fr_cuda_fail(ce, "power method graph: loop node");
    }
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    if ((ce = cudaGraphAddNode(&ncond, g, &npro, nullptr, 1, &cp)) != cudaSuccess) {
        p->launches = l0;
        cleanup();
        return fr_cuda_fail(ce, "power method graph: loop node");
    }
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    const long l1 = p->launches;
    if ((ce = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
        cudaSuccess) {
        p->launches = l0;
        cleanup();
        return fr_cuda_fail(ce, "power method graph: body capture");
    }
    rc = residual_into(p, v, fv);
    if (!rc) rc = norm_to(fv, fu, &c->dfnrm);
    if (!rc) rc = fr_pm_step(st, c, n, h);
    if (!rc) rc = fr_pm_update(st, f32, n, v, u, fv, fu, c);
    ce = cudaStreamEndCapture(st, &body);
    const long bodyk = p->launches - l1 + 3;
    if (rc || ce != cudaSuccess) {
        p->launches = l0;
        cleanup();
        return rc ? rc : fr_cuda_fail(ce, "power method graph: body capture");
    }
    // epilogue
    FR_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    rc = fr_vec_axpy_diff(st, f32, n, dir, nullptr, v, u, 1.0);
    if (!rc) rc = fr_pm_finish(st, c, &p->h_words->pm_rho, &p->h_words->pm_iters);
    ce = cudaStreamEndCapture(st, &ge);
    p->launches = l0;
    if (rc || ce != cudaSuccess) {
        cleanup();
        return rc ? rc : fr_cuda_fail(ce, "power method graph: epilogue capture");
    }
    if ((ce = cudaGraphAddChildGraphNode(&nepi, g, &ncond, 1, ge)) != cudaSuccess ||
        (ce = cudaGraphInstantiate(&out.gexec, g, 0)) != cudaSuccess) {
        cleanup();
        return fr_cuda_fail(ce, "power method graph: instantiate");
    }
    cleanup();
    out.u = u;
    out.maxiter = maxiter;
    out.pro = pro;
    out.body = bodyk;
    out.epi = 2;
    return FRGPU_OK;
}

static int spectral_radius_graph(frgpu_problem *p, int maxiter, double *rho, int *iters) {
    const void *u = fr_state_hi(p);
    if (!p->d_pm) FR_CUDA(cudaMalloc((void **)&p->d_pm, sizeof(fr_power_ctl)));
    frgpu_problem::pm_graph *g = nullptr;
    for (auto &x : p->pm_graphs)
        if (x.u == u && x.maxiter == maxiter) g = &x;
    if (!g) {
        if (p->pm_graphs.size() >= 4) {
            FR_CUDA(cudaStreamSynchronize(p->stream));
            cudaGraphExecDestroy(p->pm_graphs.front().gexec);
            p->pm_graphs.erase(p->pm_graphs.begin());
        }
        frgpu_problem::pm_graph ng{};
        int rc = build_pm_graph(p, maxiter, u, ng);
        if (rc) return rc;
        p->pm_graphs.push_back(ng);
        g = &p->pm_graphs.back();
    }
    FR_CUDA(cudaGraphLaunch(g->gexec, p->stream));
    FR_CUDA(cudaStreamSynchronize(p->stream));
    const int it = p->h_words->pm_iters;
    p->launches += g->pro + (long)(it < 0 ? -it : it) * g->body + g->epi;
    *rho = p->h_words->pm_rho;
    if (iters) *iters = it;
    return status_error(p, p->h_words->status);
}

FRGPU_API int frgpu_spectral_radius(frgpu_problem *p, int maxiter, double *rho, int *iters) {
    FR_REQ(p && rho, "spectral_radius: null argument");
    FR_REQ(maxiter >= 1 && maxiter <= 10000, "spectral_radius: need 1 <= maxiter <= 10000");
    FR_TRY
    const bool f32 = p->d.precision == FRGPU_FP32K;
    const size_t n = (size_t)p->ndof, es = p->esize;
    if (!p->d_eig) {
        FR_CUDA(cudaMalloc(&p->d_eig, 4 * n * es));
        FR_CUDA(cudaMalloc((void **)&p->d_eig_red, sizeof(double) * (FR_RED_BLOCKS + 1)));
        FR_CUDA(cudaMemset(p->d_eig_red + FR_RED_BLOCKS, 0, sizeof(double))); // the norms' last-block counter
        p->have_eig = false;
    }
    if (p->have_eig) return spectral_radius_graph(p, maxiter, rho, iters);
    char *base = (char *)p->d_eig;
    void *dir = base, *v = base + n * es, *fu = base + 2 * n * es, *fv = base + 3 * n * es;
    const void *u = fr_state_hi(p);
    cudaStream_t st = p->stream;
    int rc;
    unsigned *cnt = reinterpret_cast<unsigned *>(p->d_eig_red + FR_RED_BLOCKS);
    // the norm lands in page-locked host word `slot`; `wait` synchronises
    auto norm = [&](const void *x, const void *y, int slot, bool wait) -> int {
        int r = fr_vec_norm2(st, f32, n, x, y, p->d_eig_red, cnt, &p->h_words->norm[slot], p->d_status,
                             &p->h_words->status);
        if (r) return r;
        p->launches += 1;
        if (wait) FR_CUDA(cudaStreamSynchronize(st));
        return FRGPU_OK;
    };
    const double uround = f32 ? 0x1p-24 : 0x1p-53, sq = std::sqrt(uround);
    if ((rc = residual_into(p, u, fu))) return rc;
    const void *d0 = p->have_eig ? dir : fu;
    double dynrm;
    if ((rc = norm(u, nullptr, 0, false)) || (rc = norm(d0, nullptr, 1, true))) return rc;
    const double ynrm = p->h_words->norm[0], vnrm = p->h_words->norm[1];
    if (ynrm != 0.0 && vnrm != 0.0) {
        dynrm = ynrm * sq;
        rc = fr_vec_axpy(st, f32, n, v, u, d0, dynrm / vnrm);
    } else if (ynrm != 0.0) {
        dynrm = ynrm * sq;
        rc = fr_vec_axpy(st, f32, n, v, u, nullptr, sq);
    } else if (vnrm != 0.0) {
        dynrm = uround;
        rc = fr_vec_axpy(st, f32, n, v, u, d0, dynrm / vnrm);
    } else {
        dynrm = uround;
        rc = fr_vec_fill(st, f32, n, v, dynrm / std::sqrt((double)n));
    }
    if (rc) return rc;
    p->launches += 1;
    double sigma = 0.0;
    int it = 1, converged = 0;
    for (; it <= maxiter; ++it) {
        if ((rc = residual_into(p, v, fv))) return rc;
        if ((rc = norm(fv, fu, 0, true))) return rc;
        const double dfnrm = p->h_words->norm[0];
        const double sigmal = sigma;
        sigma = dfnrm / dynrm;
        if (it >= 2 && std::fabs(sigma - sigmal) <= std::max(sigma, 1e-300) * 0.01) {
            converged = 1;
            break;
        }
        if (it == maxiter) break;
        if (dfnrm != 0.0) {
            if ((rc = fr_vec_axpy_diff(st, f32, n, v, u, fv, fu, dynrm / dfnrm))) return rc;
            p->launches += 1;
        } else {
            if ((rc = fr_vec_flip(st, f32, v, u, (size_t)it % n))) return rc;
            p->launches += 1;
        }
    }
    // the direction for the next call; the status word came back with the last norm
    if ((rc = fr_vec_axpy_diff(st, f32, n, dir, nullptr, v, u, 1.0))) return rc;
    p->launches += 1;
    p->have_eig = true;
    *rho = 1.2 * sigma;
    if (iters) *iters = converged ? it : -it;
    return status_error(p, p->h_words->status);
    FR_CATCH
}

// RKC2 coefficients (the closed forms of Sommeijer, Shampine and Verwer, J.
// Comput. Appl. Math. 88 (1997) 315-326): Chebyshev T_j and its first two
// derivatives at w0 = 1 + eps/s^2, w1 = T_s'/T_s'', b_j = T_j''/T_j'^2 (b_0 = b_1
// = b_2), a_j = 1 - b_j T_j; in the increment form D_j = alpha_j D_{j-1} +
// beta_j D_{j-2} + dt (mu_j f(u + D_{j-1}) + delta_j f(u)): mu_1 = b_1 w1 and for
// j >= 2 alpha_j = 2 b_j w0 / b_{j-1}, beta_j = -b_j / b_{j-2}, mu_j = 2 b_j w1 /
// b_{j-1}, delta_j = -a_{j-1} mu_j.  The operations and their order are those of
// the Python restatement frgpu.rkc2_coefficients, so both give the same bits.
static void rkc2_coeffs(int s, double eps, double *alpha, double *beta, double *mu, double *delta, double *bound) {
    const double w0 = 1.0 + eps / (double)(s * s);
    std::vector<double> T(s + 1, 0.0), dT(s + 1, 0.0), d2T(s + 1, 0.0), b(s + 1, 0.0), a(s + 1, 0.0);
    T[0] = 1.0;
    T[1] = w0;
    dT[1] = 1.0;
    for (int j = 2; j <= s; ++j) {
        T[j] = 2 * w0 * T[j - 1] - T[j - 2];
        dT[j] = 2 * T[j - 1] + 2 * w0 * dT[j - 1] - dT[j - 2];
        d2T[j] = 4 * dT[j - 1] + 2 * w0 * d2T[j - 1] - d2T[j - 2];
    }
    const double w1 = dT[s] / d2T[s];
    for (int j = 2; j <= s; ++j) b[j] = d2T[j] / (dT[j] * dT[j]);
    b[0] = b[1] = b[2];
    for (int j = 0; j <= s; ++j) a[j] = 1.0 - b[j] * T[j];
    for (int j = 0; j < s; ++j) alpha[j] = beta[j] = mu[j] = delta[j] = 0.0;
    mu[0] = b[1] * w1;
    for (int j = 2; j <= s; ++j) {
        alpha[j - 1] = 2 * b[j] * w0 / b[j - 1];
        beta[j - 1] = -b[j] / b[j - 2];
        mu[j - 1] = 2 * b[j] * w1 / b[j - 1];
        delta[j - 1] = -a[j - 1] * mu[j - 1];
    }
    *bound = (w0 + 1) * d2T[s] / dT[s];
}

FRGPU_API int frgpu_rkc2_coefficients(int s, double eps, double *alpha, double *beta, double *mu, double *delta,
                                      double *bound) {
    FR_REQ(s >= 2 && s <= FR_ROCK_MAXM, "rkc2_coefficients: need 2 <= s <= 4096");
    FR_REQ(std::isfinite(eps) && eps >= 0.0, "rkc2_coefficients: eps must be finite and >= 0");
    FR_REQ(alpha && beta && mu && delta && bound, "rkc2_coefficients: null output");
    FR_TRY
    rkc2_coeffs(s, eps, alpha, beta, mu, delta, bound);
    return FRGPU_OK;
    FR_CATCH
}

FRGPU_API int frgpu_step_rkc2(frgpu_problem *p, double dt, int nsteps, double eps, int smax, int maxiter,
                              int *stages) {
    FR_REQ(p, "step_rkc2: null problem");
    FR_REQ(nsteps >= 0, "step_rkc2: negative step count");
    FR_REQ(smax >= 2 && smax <= FR_ROCK_MAXM, "step_rkc2: need 2 <= smax <= 4096");
    FR_REQ(maxiter >= 1 && maxiter <= 10000, "step_rkc2: need 1 <= maxiter <= 10000");
    FR_REQ(std::isfinite(eps) && eps >= 0.0, "step_rkc2: eps must be finite and >= 0");
    if (!(dt > 0.0) || !std::isfinite(dt)) {
        fr_set_error("step_rkc2: dt must be positive and finite");
        return FRGPU_ERR_DT;
    }
    FR_TRY
    if (p->rkc2_eps != eps) { // the cache of coefficient sets belongs to one damping
        p->rkc2_cache.clear();
        p->rkc2_eps = eps;
    }
    auto coeffs = [&](int s) -> const std::vector<double> & {
        auto it = p->rkc2_cache.find(s);
        if (it != p->rkc2_cache.end()) return it->second;
        std::vector<double> c(4 * (size_t)s + 1);
        rkc2_coeffs(s, eps, c.data(), c.data() + s, c.data() + 2 * s, c.data() + 3 * s, c.data() + 4 * s);
        return p->rkc2_cache.emplace(s, std::move(c)).first->second;
    };
    for (int n = 0; n < nsteps; ++n) {
        double rho = 0.0;
        int it = 0;
        int rc = frgpu_spectral_radius(p, maxiter, &rho, &it);
        if (rc) return rc;
        const double z = dt * rho;
        int s = 2;
        for (;;) {
            if (coeffs(s)[4 * (size_t)s] >= z || s >= smax) break;
            s = std::min(smax, std::max(s + 1, (int)(s * 1.1)));
        }
        const std::vector<double> &c = coeffs(s);
        if (c[4 * (size_t)s] < z) {
            fr_set_error("step_rkc2: dt * rho needs more than smax stages");
            return FRGPU_ERR_DT;
        }
        // queued without a wait: the next spectral radius (or the check below)
        // synchronises and reports the step's status
        rc = step_rock_impl(p, s, c.data(), c.data() + s, c.data() + 2 * s, c.data() + 3 * s, 0, nullptr, nullptr,
                            dt, 1, false);
        if (rc) return rc;
        if (stages) stages[n] = s;
    }
    return check_status(p);
    FR_CATCH
}

FRGPU_API int frgpu_reduce(frgpu_problem *p, double *sums, double *maxspeed) {
    FR_REQ(p, "reduce: null problem");
    if (p->d.equation != FRGPU_EULER2D) {
        fr_set_error("reduce: implemented for the 2D Euler problem");
        return FRGPU_ERR_UNSUPPORTED;
    }
    FR_TRY
    double sp[2];
    int st = 0;
    int rc = fr_launch_euler2d_reduce(p, fr_state_hi(p), p->d.precision == FRGPU_FP32K ? p->s3 : nullptr, sums, sp,
                                      1.0 / p->sp.dx, 1.0 / p->sp.dy, &st);
    if (rc) return rc;
    if (maxspeed) *maxspeed = sp[0];
    // the status of steps queued before (frgpu_step_ssprk3_async) comes back with the sums
    return status_error(p, st);
    FR_CATCH
}

FRGPU_API int frgpu_step_ssprk3_reduce(frgpu_problem *p, double dt, int nsteps, double *sums, double *maxspeed) {
    FR_REQ(p, "step_ssprk3_reduce: null problem");
    FR_REQ(nsteps >= 0, "step_ssprk3_reduce: negative step count");
    if (p->d.equation != FRGPU_EULER2D) {
        fr_set_error("step_ssprk3_reduce: implemented for the 2D Euler problem");
        return FRGPU_ERR_UNSUPPORTED;
    }
    if (!(dt > 0.0) || !std::isfinite(dt)) {
        fr_set_error("step_ssprk3_reduce: dt must be positive and finite");
        return FRGPU_ERR_DT;
    }
    FR_TRY
    if (nsteps > 0) {
        use_method(p, fr_method());
        int rc = run_fused_steps(p, dt, nsteps, false);
        if (rc) return rc;
    }
    return frgpu_reduce(p, sums, maxspeed);
    FR_CATCH
}

FRGPU_API int frgpu_cfl_dt(frgpu_problem *p, double cfl, double *dt) {
    FR_REQ(p && dt && cfl > 0, "cfl_dt: bad arguments");
    FR_TRY
    if (p->d.equation == FRGPU_EULER2D) {
        double sp[2];
        int rc = fr_launch_euler2d_reduce(p, fr_state_hi(p), p->d.precision == FRGPU_FP32K ? p->s3 : nullptr,
                                          nullptr, sp, 1.0 / p->sp.dx, 1.0 / p->sp.dy);
        if (rc) return rc;
        if (!(sp[1] > 0) || !std::isfinite(sp[1])) {
            fr_set_error("cfl_dt: non-positive or non-finite wave speed");
            return FRGPU_ERR_DT;
        }
        *dt = cfl / sp[1];
        return FRGPU_OK;
    }
    if (p->d.equation == FRGPU_ADVECTION) {
        double dxmin = 1e300;
        for (int i = 0; i < p->sp.nx; ++i) dxmin = std::min(dxmin, p->sp.J.empty() ? p->sp.dx : 2 * p->sp.J[i]);
        *dt = cfl * dxmin / std::max(std::fabs(p->d.a), 1e-300);
        return FRGPU_OK;
    }
    if (p->d.equation == FRGPU_BGK1D) {
        double dxmin = 1e300, vmax = 0;
        for (int i = 0; i < p->sp.nx; ++i) dxmin = std::min(dxmin, p->sp.J.empty() ? p->sp.dx : 2 * p->sp.J[i]);
        for (double v : p->velo) vmax = std::max(vmax, std::fabs(v));
        *dt = cfl * dxmin / vmax;
        return FRGPU_OK;
    }
    fr_set_error("cfl_dt: not available for this equation");
    return FRGPU_ERR_UNSUPPORTED;
    FR_CATCH
}

FRGPU_API int frgpu_set_filter(frgpu_problem *p, int indicator, double lam, double S0, double kappa) {
    FR_REQ(p, "set_filter: null problem");
    FR_REQ(indicator >= FRGPU_IND_NONE && indicator <= FRGPU_IND_MLP, "set_filter: unknown indicator");
    FR_REQ(p->d.equation == FRGPU_EULER2D || p->d.equation == FRGPU_EULER1D || indicator == FRGPU_IND_NONE,
           "set_filter: the modal filter is available for the Euler problems");
    p->indicator = indicator;
    p->lam = lam;
    p->S0 = S0;
    p->kappa = kappa;
    p->graph_ind = -2; // force a re-capture
    p->erk_dirty = true;
    drop_rock_graphs(p);
    return FRGPU_OK;
}

FRGPU_API int frgpu_problem_set_option(frgpu_problem *p, int option, int value) {
    FR_REQ(p, "set_option: null problem");
    FR_REQ(option == FRGPU_OPT_BGK_TENSOR || option == FRGPU_OPT_FUSED_INDICATOR ||
               option == FRGPU_OPT_FUSED_TWO_STAGE || option == FRGPU_OPT_BGK_CLOSURE ||
               option == FRGPU_OPT_GHOSTS_PER_STEP,
           "set_option: unknown option");
    FR_REQ(option != FRGPU_OPT_BGK_CLOSURE || value == 0 || value == 1, "set_option: BGK closure is 0 or 1");
    FR_REQ(option != FRGPU_OPT_BGK_TENSOR || (value >= 0 && value <= 2), "set_option: BGK tensor form is 0, 1 or 2");
    if (option == FRGPU_OPT_BGK_TENSOR) p->bgk_tensor = value;
    if (option == FRGPU_OPT_BGK_CLOSURE) p->bgk_closure = value;
    if (option == FRGPU_OPT_GHOSTS_PER_STEP) p->ghosts_per_step = value != 0;
    if (option == FRGPU_OPT_FUSED_INDICATOR) p->fuse_indicator = value != 0;
    if (option == FRGPU_OPT_FUSED_TWO_STAGE) p->fuse_erk = value != 0;
    p->graph_ind = -2; // force a re-capture
    p->erk_dirty = true;
    drop_rock_graphs(p);
    return FRGPU_OK;
}

FRGPU_API int frgpu_problem_set_flux_dissipation(frgpu_problem *p, double c) {
    FR_REQ(p, "set_flux_dissipation: null problem");
    FR_REQ(std::isfinite(c) && c >= 0.0, "set_flux_dissipation: need a finite c >= 0");
    p->flux_c = c;
    p->erk_dirty = true; // the coefficient is baked into the captured kernels
    drop_rock_graphs(p);
    return FRGPU_OK;
}

FRGPU_API int frgpu_modal_filter(frgpu_problem *p, int indicator, double lam, double S0, double kappa,
                                 int *ntroubled) {
    FR_REQ(p, "modal_filter: null problem");
    FR_REQ(p->d.equation == FRGPU_EULER2D || p->d.equation == FRGPU_EULER1D,
           "modal_filter: available for the Euler problems");
    FR_REQ(indicator == FRGPU_IND_PLAIN || indicator == FRGPU_IND_MLP, "modal_filter: unknown indicator");
    FR_TRY
    int rc = p->sp.dim == 2 ? fr_launch_filter2d(p, indicator, lam, S0, kappa)
                            : fr_launch_filter1d(p, indicator, lam, S0, kappa);
    if (rc) return rc;
    if (ntroubled) {
        FR_CUDA(cudaMemcpyAsync(ntroubled, p->d_count, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
    }
    FR_CUDA(cudaStreamSynchronize(p->stream));
    return check_status(p);
    FR_CATCH
}

FRGPU_API int frgpu_positive_limiter(frgpu_problem *p, const double *weights, double t0, int *nlimited) {
    FR_REQ(p, "positive_limiter: null problem");
    FR_REQ(t0 > 0.0 && t0 <= 1.0, "positive_limiter: need 0 < t0 <= 1");
    FR_TRY
    std::vector<double> w;
    int rc = fr_limiter_weights(p, weights, w);
    if (rc) return rc;
    if ((rc = fr_launch_limiter(p, w, t0))) return rc;
    int n = 0;
    FR_CUDA(cudaMemcpyAsync(&n, p->d_count + FR_COUNT_LIMITER, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
    FR_CUDA(cudaStreamSynchronize(p->stream));
    if (nlimited) *nlimited = n;
    return check_status(p);
    FR_CATCH
}

// host array (column-major, the 2 components last) -> device pairs (c fastest)
static int upload_pairs(frgpu_problem *p, void **dst, const double *h, size_t nfaces) {
    std::vector<double> dev(2 * nfaces);
    for (size_t f = 0; f < nfaces; ++f)
        for (int c = 0; c < 2; ++c) {
            const double v = h[f + nfaces * c];
            if (!std::isfinite(v)) {
                fr_set_error("problem_set_metric: non-finite face normal");
                return FRGPU_ERR_ARG;
            }
            dev[2 * f + c] = v;
        }
    if (!*dst) FR_CUDA(cudaMalloc(dst, 2 * nfaces * p->esize));
    if (p->esize == 8) {
        FR_CUDA(cudaMemcpy(*dst, dev.data(), sizeof(double) * dev.size(), cudaMemcpyHostToDevice));
    } else {
        std::vector<float> f(dev.begin(), dev.end());
        FR_CUDA(cudaMemcpy(*dst, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice));
    }
    return FRGPU_OK;
}

FRGPU_API int frgpu_problem_set_metric(frgpu_problem *p, const double *iJ, const double *n1, const double *n2) {
    FR_REQ(p, "problem_set_metric: null problem");
    FR_REQ(p->d.equation == FRGPU_EULER2D, "problem_set_metric: 2D Euler problems only");
    FR_REQ((n1 == nullptr) == (n2 == nullptr), "problem_set_metric: pass both face-normal arrays or neither");
    FR_REQ(iJ || !n1, "problem_set_metric: face normals need the metric");
    FR_TRY
    FR_CUDA(cudaStreamSynchronize(p->stream));
    fr_drop_reduce_graphs(p); // they hold the metric buffer's address
    for (void **b : {&p->d_nfx, &p->d_nfy, &p->d_fsc})
        if (*b) {
            cudaFree(*b);
            *b = nullptr;
        }
    if (!iJ) {
        if (p->d_met) cudaFree(p->d_met);
        p->d_met = nullptr;
    } else {
        // host iJ[nx, ny, np, np, 2, 2] (column-major: blocks a11, a21, a12, a22)
        // -> device (a11, a12, a21, a22) per point in the state's point-vector layout
        const size_t ne = (size_t)p->sp.nx * p->sp.ny, nq = (size_t)p->sp.np * p->sp.np, blk = ne * nq;
        const int from[4] = {0, 2, 1, 3};
        std::vector<double> dev(4 * blk);
        for (size_t q = 0; q < nq; ++q)
            for (size_t e = 0; e < ne; ++e)
                for (int m = 0; m < 4; ++m) {
                    const double v = iJ[e + ne * q + blk * from[m]];
                    if (!std::isfinite(v)) {
                        fr_set_error("problem_set_metric: non-finite metric value");
                        return FRGPU_ERR_ARG;
                    }
                    dev[(q * ne + e) * 4 + m] = v;
                }
        if (!p->d_met) FR_CUDA(cudaMalloc(&p->d_met, 4 * blk * p->esize));
        if (p->esize == 8) {
            FR_CUDA(cudaMemcpy(p->d_met, dev.data(), sizeof(double) * dev.size(), cudaMemcpyHostToDevice));
        } else {
            std::vector<float> f(dev.begin(), dev.end());
            FR_CUDA(cudaMemcpy(p->d_met, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice));
        }
        if (n1) {
            const size_t nx = p->sp.nx, ny = p->sp.ny;
            int rc = upload_pairs(p, &p->d_nfx, n1, (nx + 1) * ny);
            if (!rc) rc = upload_pairs(p, &p->d_nfy, n2, nx * (ny + 1));
            if (rc) return rc;
        }
    }
    p->graph_ind = -2; // force a re-capture
    p->erk_dirty = true;
    drop_rock_graphs(p);
    return FRGPU_OK;
    FR_CATCH
}

// (inv(J) n)_comp of a 2 x 2 matrix J (column-major j00, j10, j01, j11) and a
// vector n, in the order of the oracle's restatement
static double inv_dot(double j00, double j10, double j01, double j11, double n0, double n1, int comp) {
    const double det = j00 * j11 - j01 * j10;
    return comp == 0 ? (j11 * n0 - j01 * n1) / det : (j00 * n1 - j10 * n0) / det;
}

FRGPU_API int frgpu_problem_set_face_jacobians(frgpu_problem *p, const double *Ji, const double *n1, const double *n2) {
    FR_REQ(p, "problem_set_face_jacobians: null problem");
    FR_REQ(p->d.equation == FRGPU_EULER2D, "problem_set_face_jacobians: 2D Euler problems only");
    FR_REQ(p->d_met && p->d_nfx && p->d_nfy,
           "problem_set_face_jacobians: set the metric and the face normals first (frgpu_problem_set_metric)");
    FR_REQ(n1 && n2, "problem_set_face_jacobians: pass the face normals the metric was set with");
    FR_TRY
    FR_CUDA(cudaStreamSynchronize(p->stream));
    if (p->d_fsc) {
        cudaFree(p->d_fsc);
        p->d_fsc = nullptr;
    }
    if (Ji) {
        // host Ji[nx, ny, 4, np, 2, 2] (column-major) -> per (point line q, element e)
        // the scales (sL, sR, sB, sT) of the element's left, right, bottom and top
        // interface fluxes at point q of the face
        const long nx = p->sp.nx, ny = p->sp.ny, np = p->sp.np, ne = nx * ny;
        auto J = [&](long i, long j, int f, long k, int a, int b) {
            return Ji[i + nx * (j + ny * (f + 4 * (k + np * (a + 2 * b))))];
        };
        const long nfx = (nx + 1) * ny, nfy = nx * (ny + 1);
        std::vector<double> dev(4 * np * ne);
        for (long j = 0; j < ny; ++j)
            for (long i = 0; i < nx; ++i)
                for (long q = 0; q < np; ++q) {
                    const long e = i + nx * j;
                    const long fl = i + (nx + 1) * j, fb = i + nx * j;
                    // faces 1..4 of the reference (bottom, right, top, left) -> f = 0..3
                    double *d = &dev[(q * ne + e) * 4];
                    d[0] = inv_dot(J(i, j, 3, q, 0, 0), J(i, j, 3, q, 1, 0), J(i, j, 3, q, 0, 1), J(i, j, 3, q, 1, 1),
                                   n1[fl], n1[fl + nfx], 0);
                    d[1] = inv_dot(J(i, j, 1, q, 0, 0), J(i, j, 1, q, 1, 0), J(i, j, 1, q, 0, 1), J(i, j, 1, q, 1, 1),
                                   n1[fl + 1], n1[fl + 1 + nfx], 0);
                    d[2] = inv_dot(J(i, j, 0, q, 0, 0), J(i, j, 0, q, 1, 0), J(i, j, 0, q, 0, 1), J(i, j, 0, q, 1, 1),
                                   n2[fb], n2[fb + nfy], 1);
                    d[3] = inv_dot(J(i, j, 2, q, 0, 0), J(i, j, 2, q, 1, 0), J(i, j, 2, q, 0, 1), J(i, j, 2, q, 1, 1),
                                   n2[fb + nx], n2[fb + nx + nfy], 1);
                    for (int c = 0; c < 4; ++c)
                        if (!std::isfinite(d[c])) {
                            fr_set_error("problem_set_face_jacobians: singular face Jacobian or non-finite value");
                            return FRGPU_ERR_ARG;
                        }
                }
        FR_CUDA(cudaMalloc(&p->d_fsc, dev.size() * p->esize));
        if (p->esize == 8) {
            FR_CUDA(cudaMemcpy(p->d_fsc, dev.data(), sizeof(double) * dev.size(), cudaMemcpyHostToDevice));
        } else {
            std::vector<float> f(dev.begin(), dev.end());
            FR_CUDA(cudaMemcpy(p->d_fsc, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice));
        }
    }
    p->graph_ind = -2; // force a re-capture
    p->erk_dirty = true;
    drop_rock_graphs(p);
    return FRGPU_OK;
    FR_CATCH
}

FRGPU_API int frgpu_set_limiter(frgpu_problem *p, int on, const double *weights, double t0) {
    FR_REQ(p, "set_limiter: null problem");
    FR_REQ(p->d.equation != FRGPU_BGK1D, "set_limiter: not defined for the kinetic equation");
    FR_REQ(!on || (t0 > 0.0 && t0 <= 1.0), "set_limiter: need 0 < t0 <= 1");
    if (on) {
        std::vector<double> w;
        const int rc = fr_limiter_weights(p, weights, w);
        if (rc) return rc;
        p->lim_w = w;
        p->lim_t0 = t0;
    }
    p->limiter = on != 0;
    p->graph_ind = -2; // force a re-capture
    p->erk_dirty = true;
    drop_rock_graphs(p);
    return FRGPU_OK;
}

FRGPU_API int frgpu_problem_set_mlp(frgpu_problem *p, const frgpu_mlp *m, double threshold, double band) {
    FR_REQ(p, "problem_set_mlp: null problem");
    FR_REQ(p->d.equation == FRGPU_EULER2D && p->sp.np == 4, "problem_set_mlp: 2D Euler with deg = 3");
    FR_REQ(threshold > 0 && threshold < 1 && band >= 0 && band < 0.5, "problem_set_mlp: need 0 < threshold < 1, 0 <= band < 0.5");
    p->mlp = m;
    p->mlp_thr = (float)threshold;
    p->mlp_band = (float)band;
    p->graph_ind = -2; // the captured step refers to the network: re-capture
    p->erk_dirty = true;
    drop_rock_graphs(p);
    return FRGPU_OK;
}

FRGPU_API int frgpu_modal_features(frgpu_problem *p, float *feat, long n) {
    FR_REQ(p && feat, "modal_features: null argument");
    const long ne = (long)p->sp.nx * p->sp.ny;
    FR_REQ(n >= ne * 32, "modal_features: output needs nx*ny*32 floats");
    FR_TRY
    float *d = nullptr;
    FR_CUDA(cudaMalloc(&d, sizeof(float) * ne * 32));
    int rc = fr_launch_features(p, d);
    cudaError_t e = cudaSuccess;
    if (!rc) {
        e = cudaMemcpyAsync(feat, d, sizeof(float) * ne * 32, cudaMemcpyDeviceToHost, p->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    }
    cudaFree(d);
    if (rc) return rc;
    if (e != cudaSuccess) return fr_cuda_fail(e, "modal_features copy");
    return FRGPU_OK;
    FR_CATCH
}

FRGPU_API int frgpu_indicator_stats(frgpu_problem *p, int *stats) {
    FR_REQ(p && stats, "indicator_stats: null argument");
    FR_CUDA(cudaStreamSynchronize(p->stream));
    FR_CUDA(cudaMemcpy(stats, p->d_count, sizeof(int) * 3, cudaMemcpyDeviceToHost));
    return FRGPU_OK;
}

FRGPU_API int frgpu_troubled_flags(frgpu_problem *p, int *flags, long n) {
    FR_REQ(p && flags, "troubled_flags: null argument");
    const long ne = (long)p->sp.nx * p->sp.ny;
    FR_REQ(n >= ne, "troubled_flags: output too small");
    FR_CUDA(cudaStreamSynchronize(p->stream));
    FR_CUDA(cudaMemcpy(flags, p->d_flags, sizeof(int) * ne, cudaMemcpyDeviceToHost));
    return FRGPU_OK;
}

FRGPU_API int frgpu_problem_device_state(frgpu_problem *p, void **dptr, int *elem_bytes) {
    FR_REQ(p && dptr, "problem_device_state: null argument");
    *dptr = fr_state_hi(p);
    if (elem_bytes) *elem_bytes = (int)p->esize;
    return FRGPU_OK;
}

FRGPU_API int frgpu_problem_stream(frgpu_problem *p, void **stream) {
    FR_REQ(p && stream, "problem_stream: null argument");
    *stream = (void *)p->stream;
    return FRGPU_OK;
}

FRGPU_API long frgpu_problem_launches(const frgpu_problem *p) { return p ? p->launches : -1; }

FRGPU_API int frgpu_synchronize(frgpu_problem *p) {
    FR_REQ(p, "synchronize: null problem");
    FR_TRY
    return check_status(p);
    FR_CATCH
}

// ------------------------------------------------------------------ stateless operators
static int stateless_op(const double *f, long n, int np, const double *a, int na, const double *b, int nb,
                        double *out, int nout, bool derivative) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        fr_set_error("no CUDA device");
        return FRGPU_ERR_CUDA;
    }
    double *d_f = nullptr, *d_a = nullptr, *d_b = nullptr, *d_o = nullptr;
    cudaStream_t st = nullptr;
    int rc = [&]() -> int {
        FR_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        FR_CUDA(cudaMalloc(&d_f, sizeof(double) * n * np));
        FR_CUDA(cudaMalloc(&d_a, sizeof(double) * na));
        if (nb) FR_CUDA(cudaMalloc(&d_b, sizeof(double) * nb));
        FR_CUDA(cudaMalloc(&d_o, sizeof(double) * n * nout));
        FR_CUDA(cudaMemcpyAsync(d_f, f, sizeof(double) * n * np, cudaMemcpyHostToDevice, st));
        FR_CUDA(cudaMemcpyAsync(d_a, a, sizeof(double) * na, cudaMemcpyHostToDevice, st));
        if (nb) FR_CUDA(cudaMemcpyAsync(d_b, b, sizeof(double) * nb, cudaMemcpyHostToDevice, st));
        int r = derivative ? fr_launch_poly_derivative(d_f, n, np, d_a, d_o, st)
                           : fr_launch_interp_face(d_f, n, np, d_a, d_b, d_o, st);
        if (r) return r;
        FR_CUDA(cudaMemcpyAsync(out, d_o, sizeof(double) * n * nout, cudaMemcpyDeviceToHost, st));
        FR_CUDA(cudaStreamSynchronize(st));
        return FRGPU_OK;
    }();
    if (d_f) cudaFree(d_f);
    if (d_a) cudaFree(d_a);
    if (d_b) cudaFree(d_b);
    if (d_o) cudaFree(d_o);
    if (st) cudaStreamDestroy(st);
    return rc;
}

FRGPU_API int frgpu_interp_face(const double *f, long n, int np, const double *ll, const double *lr, double *fdelta) {
    FR_REQ(f && ll && lr && fdelta && n >= 0 && np >= 1, "interp_face: bad arguments");
    if (n == 0) return FRGPU_OK;
    return stateless_op(f, n, np, ll, np, lr, np, fdelta, 2, false);
}

FRGPU_API int frgpu_poly_derivative(const double *f, long n, int np, const double *pdm, double *df) {
    FR_REQ(f && pdm && df && n >= 0 && np >= 1, "poly_derivative: bad arguments");
    if (n == 0) return FRGPU_OK;
    return stateless_op(f, n, np, pdm, np * np, nullptr, 0, df, np, true);
}

} // extern "C"
