// erk.cu -- fixed-step explicit Runge-Kutta methods given by a Butcher
// tableau (OrdinaryDiffEq's Midpoint, Heun, RK4, Tsit5, ... with
// adaptive=false), built on the residual kernels (stage 0 of each equation)
// and one elementwise combination kernel per stage.
//
// Per step and stage i: acc = sum over j < i with a_ij != 0, in ascending j,
// as the chain acc = a_ij0 k_j0; acc = fma(a_ij, k_j, acc); the stage input is
// fma(dt, acc, u^n) (u^n itself when no a_ij is nonzero); k_i = L(stage).
// Then u^n+1 = fma(dt, acc_b, u^n) with the b weights.  FP64 is bit-identical
// to the oracle's fro_erk.  FP32K forms the stage inputs from the high part
// and adds the step's increment dt acc_b to the high + low pair with the
// compensated sum of the SSPRK3 form; the update is elementwise, so it runs in
// place (no ping-pong of the high part).
#include <string>

#include "fr_common.cuh"
#include "frgpu_internal.h"

namespace {

template <class Real> struct Comb {
    int nt;                  // number of terms
    int j[FR_ERK_MAXS];      // k buffer of term t
    Real a[FR_ERK_MAXS];     // coefficient of term t
};

template <class Real>
__device__ __forceinline__ Real comb_acc(const Real *__restrict__ k, size_t kstride, size_t q, const Comb<Real> &c) {
    Real acc = c.a[0] * __ldg(k + c.j[0] * kstride + q);
    for (int t = 1; t < c.nt; ++t) acc = frk::fmaR<Real>(c.a[t], __ldg(k + c.j[t] * kstride + q), acc);
    return acc;
}

// stage input: out = fma(dt, acc, u)
template <class Real>
__global__ void __launch_bounds__(256) k_erk_stage(const Real *__restrict__ u, const Real *__restrict__ k,
                                                   size_t kstride, size_t n, const Comb<Real> c,
                                                   const double *dtp, Real *__restrict__ out) {
    FR_PDL_ENTRY();
    const Real dt = (Real)*dtp;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        out[q] = frk::fmaR<Real>(dt, comb_acc<Real>(k, kstride, q, c), __ldg(u + q));
}

// step update: FP64 u = fma(dt, acc, u); FP32K compensated add of dt acc to hi + lo
template <class Real>
__global__ void __launch_bounds__(256) k_erk_update(Real *__restrict__ u, Real *__restrict__ lo,
                                                    const Real *__restrict__ k, size_t kstride, size_t n, const Comb<Real> c,
                                                    const double *dtp, int *status) {
    FR_PDL_ENTRY();
    const Real dt = (Real)*dtp;
    bool bad = false;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const Real acc = comb_acc<Real>(k, kstride, q, c);
        Real t;
        if (lo == nullptr) {
            t = frk::fmaR<Real>(dt, acc, u[q]);
        } else {
            const Real hi = u[q], y = dt * acc + lo[q];
            t = hi + y;
            lo[q] = y - (t - hi);
        }
        u[q] = t;
        bad |= !isfinite(t);
    }
    if (bad) atomicOr(status, frk::ST_NONFINITE);
}

int grid_for(size_t n) {
    const size_t g = (n + 255) / 256;
    return (int)(g < 152 * 8 ? (g > 0 ? g : 1) : 152 * 8);
}

template <class Real> Comb<Real> comb_of(const double *coef, int nterms) {
    Comb<Real> c{};
    for (int j = 0; j < nterms; ++j)
        if (coef[j] != 0.0) {
            c.j[c.nt] = j;
            c.a[c.nt] = (Real)coef[j];
            ++c.nt;
        }
    return c;
}

} // namespace

// Enqueue one ERK step on a stream (capturable) over raw buffers: r.kbuf holds
// the s stage derivatives and one stage input, n values each; residual(ctx,
// in, out) evaluates k = L(in).
int fr_erk_enqueue_raw(const fr_erk_raw &r, int (*residual)(void *, const void *, void *), void *ctx) {
    const int s = r.s;
    const size_t n = r.n, kstride = n;
    char *kb = r.kbuf;
    char *stage = kb + (size_t)s * n * r.esize;
    int rc;
    for (int i = 0; i < s; ++i) {
        const double *Ai = &r.A[(size_t)i * s];
        const int nt = comb_of<double>(Ai, i).nt;
        void *ki = kb + (size_t)i * n * r.esize;
        const void *in = r.u;
        if (nt > 0) {
            if (!r.prepare_only) {
                if (r.f32)
                    FR_CUDA(fr_launch(k_erk_stage<float>, grid_for(n), 256, 0, r.stream,
                        (const float *)r.u, (const float *)kb, kstride, n, comb_of<float>(Ai, i), r.d_dt, (float *)stage));
                else
                    FR_CUDA(fr_launch(k_erk_stage<double>, grid_for(n), 256, 0, r.stream, (const double *)r.u, (const double *)kb,
                                                                           kstride, n, comb_of<double>(Ai, i),
                                                                           r.d_dt, (double *)stage));
                FR_CUDA(cudaGetLastError());
                *r.launches += 1;
            }
            in = stage;
        }
        if ((rc = residual(ctx, in, ki))) return rc;
    }
    if (comb_of<double>(r.b, s).nt == 0 || r.prepare_only) return FRGPU_OK;
    if (r.f32)
        FR_CUDA(fr_launch(k_erk_update<float>, grid_for(n), 256, 0, r.stream, (float *)r.u, (float *)r.lo, (const float *)kb, kstride,
                                                               n, comb_of<float>(r.b, s), r.d_dt, r.d_status));
    else
        FR_CUDA(fr_launch(k_erk_update<double>, grid_for(n), 256, 0, r.stream, (double *)r.u, nullptr, (const double *)kb, kstride,
                                                                n, comb_of<double>(r.b, s), r.d_dt, r.d_status));
    FR_CUDA(cudaGetLastError());
    *r.launches += 1;
    return FRGPU_OK;
}

namespace {
struct ProblemResidual {
    frgpu_problem *p;
    int (*launch)(frgpu_problem *, const void *, void *);
};
int problem_residual(void *ctx, const void *in, void *out) {
    const ProblemResidual *c = (const ProblemResidual *)ctx;
    return c->launch(c->p, in, out);
}
} // namespace

// Enqueue one ERK step on the problem's stream (capturable).  launch_residual
// evaluates k = L(in) with the equation's stage-0 kernel.
int fr_enqueue_erk_step(frgpu_problem *p, int (*launch_residual)(frgpu_problem *, const void *, void *)) {
    const bool f32 = p->d.precision == FRGPU_FP32K;
    fr_erk_raw r;
    r.stream = p->stream;
    r.s = p->erk_s;
    r.A = p->erk_A.data();
    r.b = p->erk_b.data();
    r.n = (size_t)p->ndof;
    r.f32 = f32;
    r.u = f32 ? fr_state_hi(p) : p->s0;
    r.lo = f32 ? p->s3 : nullptr;
    r.kbuf = (char *)p->d_erk;
    r.esize = p->esize;
    r.d_dt = p->d_dt;
    r.d_status = p->d_status;
    r.prepare_only = p->prepare_only;
    r.launches = &p->launches;
    ProblemResidual ctx{p, launch_residual};
    return fr_erk_enqueue_raw(r, problem_residual, &ctx);
}

// ---------------------------------------------------------------- stabilised steps
// Three-term recurrence of m stages (ROCK2/ROCK4, RKC) in increment form: with
// D_0 = 0 and Y_j = u + D_j,
//   D_j = alpha_j D_{j-1} + beta_j D_{j-2} + dt (mu_j f(Y_{j-1}) + delta_j f(u)),
// which is Y_j = alpha_j Y_{j-1} + beta_j Y_{j-2} + (1 - alpha_j - beta_j) u +
// dt (mu_j f(Y_{j-1}) + delta_j f(u)) written for the increments (D_{-1} = 0).
// Evaluation order: t = mu F; t = fma(delta, F0, t) when delta != 0; t = dt t;
// t = fma(beta, D_{j-2}, t) when j >= 3 and beta != 0; t = fma(alpha, D_{j-1}, t)
// when j >= 2 and alpha != 0.  Then an explicit finishing tableau (A, b) of sf
// stages from g = Y_m: stage input u + fma(dt, acc, D_m) (Y_m when the row of A
// is zero), and the step u <- u + fma(dt, acc_b, D_m); FP32K adds that
// increment to the high + low pair with the compensated sum.  FP64 is
// bit-identical to the oracle's fro_rock.
namespace {

template <class Real>
__global__ void __launch_bounds__(256) k_rock_rec(const Real *__restrict__ u, const Real *__restrict__ F,
                                                  const Real *__restrict__ F0, const Real *__restrict__ d1,
                                                  const Real *__restrict__ d2, size_t n, Real alpha, Real beta,
                                                  Real mu, Real delta, const double *dtp, Real *__restrict__ dout,
                                                  Real *__restrict__ yout) {
    FR_PDL_ENTRY();
    const Real dt = (Real)*dtp;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        Real t = mu * __ldg(F + q);
        if (F0) t = frk::fmaR<Real>(delta, __ldg(F0 + q), t);
        t = dt * t;
        if (d2) t = frk::fmaR<Real>(beta, __ldg(d2 + q), t);
        if (d1) t = frk::fmaR<Real>(alpha, __ldg(d1 + q), t);
        dout[q] = t;
        yout[q] = __ldg(u + q) + t;
    }
}

template <class Real>
__global__ void __launch_bounds__(256) k_rock_fin(const Real *__restrict__ u, const Real *__restrict__ dm,
                                                  const Real *__restrict__ k, size_t kstride, size_t n,
                                                  const Comb<Real> c, const double *dtp, Real *__restrict__ out) {
    FR_PDL_ENTRY();
    const Real dt = (Real)*dtp;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        out[q] = __ldg(u + q) + frk::fmaR<Real>(dt, comb_acc<Real>(k, kstride, q, c), __ldg(dm + q));
}

template <class Real>
__global__ void __launch_bounds__(256) k_rock_update(Real *__restrict__ u, Real *__restrict__ lo,
                                                     const Real *__restrict__ dm, const Real *__restrict__ k,
                                                     size_t kstride, size_t n, const Comb<Real> c,
                                                     const double *dtp, int *status) {
    FR_PDL_ENTRY();
    const Real dt = (Real)*dtp;
    bool bad = false;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const Real t = c.nt ? frk::fmaR<Real>(dt, comb_acc<Real>(k, kstride, q, c), dm[q]) : dm[q];
        Real v;
        if (lo == nullptr) {
            v = u[q] + t;
        } else {
            const Real hi = u[q], y = t + lo[q];
            v = hi + y;
            lo[q] = y - (v - hi);
        }
        u[q] = v;
        bad |= !isfinite(v);
    }
    if (bad) atomicOr(status, frk::ST_NONFINITE);
}

template <class Real>
int rock_enqueue_t(const fr_rock_raw &r, int (*residual)(void *, const void *, void *), void *ctx) {
    const size_t n = r.n;
    Real *buf = (Real *)r.buf;
    Real *D[3] = {buf, buf + n, buf + 2 * n};
    Real *F0 = buf + 3 * n, *F = buf + 4 * n, *Y = buf + 5 * n, *S = buf + 6 * n, *K = buf + 7 * n;
    Real *u = (Real *)r.u;
    const int g = grid_for(n);
    int rc;
    if ((rc = residual(ctx, u, F0))) return rc;
    auto Dj = [&](int j) { return D[j % 3]; };
    for (int j = 1; j <= r.m; ++j) {
        if (j >= 2 && (rc = residual(ctx, Y, F))) return rc;
        if (!r.prepare_only) {
            const double al = r.alpha[j - 1], be = r.beta[j - 1], mu = r.mu[j - 1], de = r.delta[j - 1];
            FR_CUDA(fr_launch(k_rock_rec<Real>, g, 256, 0, r.stream, u, j == 1 ? F0 : F, de != 0.0 ? F0 : nullptr,
                                                      (j >= 2 && al != 0.0) ? Dj(j - 1) : nullptr,
                                                      (j >= 3 && be != 0.0) ? Dj(j - 2) : nullptr, n, (Real)al,
                                                      (Real)be, (Real)mu, (Real)de, r.d_dt, Dj(j), Y));
            FR_CUDA(cudaGetLastError());
            *r.launches += 1;
        }
    }
    const Real *Dm = Dj(r.m);
    for (int i = 0; i < r.sf; ++i) {
        const double *Ai = &r.A[(size_t)i * r.sf];
        const Comb<Real> c = comb_of<Real>(Ai, i);
        const Real *in = Y;
        if (c.nt > 0) {
            if (!r.prepare_only) {
                FR_CUDA(fr_launch(k_rock_fin<Real>, g, 256, 0, r.stream, u, Dm, K, n, n, c, r.d_dt, S));
                FR_CUDA(cudaGetLastError());
                *r.launches += 1;
            }
            in = S;
        }
        if ((rc = residual(ctx, in, K + (size_t)i * n))) return rc;
    }
    if (r.prepare_only) return FRGPU_OK;
    const Comb<Real> cb = r.sf > 0 ? comb_of<Real>(r.b, r.sf) : Comb<Real>{};
    FR_CUDA(fr_launch(k_rock_update<Real>, g, 256, 0, r.stream, u, (Real *)r.lo, Dm, K, n, n, cb, r.d_dt, r.d_status));
    FR_CUDA(cudaGetLastError());
    *r.launches += 1;
    return FRGPU_OK;
}

// ---- nonlinear power method helpers ----
// out = x + c y (y = null: out = x + c x)
template <class Real>
__global__ void __launch_bounds__(256) k_axpy(Real *__restrict__ out, const Real *__restrict__ x,
                                              const Real *__restrict__ y, double c, size_t n) {
    FR_PDL_ENTRY();
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const Real yq = y ? y[q] : x[q];
        out[q] = x[q] + (Real)c * yq;
    }
}

// out = x - y
template <class Real>
__global__ void __launch_bounds__(256) k_sub(Real *__restrict__ out, const Real *__restrict__ x,
                                             const Real *__restrict__ y, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        out[q] = x[q] - y[q];
}

// out = x + c (a - b) (x = null: c (a - b))
template <class Real>
__global__ void __launch_bounds__(256) k_axpy_diff(Real *__restrict__ out, const Real *__restrict__ x,
                                                   const Real *__restrict__ a, const Real *__restrict__ b, double c,
                                                   size_t n) {
    FR_PDL_ENTRY();
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        out[q] = (x ? x[q] : Real(0)) + (Real)c * (a[q] - b[q]);
}

// ||x - y||_2 (y = null: ||x||_2) in FP64: per-block partial sums in a fixed
// order, and the last block to finish sums the partials in block order and
// writes the root to host_out (a page-locked word through its device mapping)
template <class Real>
__global__ void __launch_bounds__(256) k_norm2(const Real *__restrict__ x, const Real *__restrict__ y, size_t n,
                                               double *__restrict__ part, unsigned *cnt, double *host_out,
                                               const int *dstatus, int *host_status) {
    FR_PDL_ENTRY();
    __shared__ double s[8];
    __shared__ bool last;
    double acc = 0.0;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const double d = y ? (double)x[q] - (double)y[q] : (double)x[q];
        acc = fma(d, d, acc);
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += s[w];
        part[blockIdx.x] = t;
        __threadfence();
        last = atomicAdd(cnt, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x >= 32) return;
    __threadfence();
    // warp 0 of the last block: lane l sums blocks l, l + 32, ... (loads issued
    // together, 19 per lane at most), then a fixed butterfly
    const int lane = threadIdx.x;
    double t = 0.0;
    constexpr int B = 20;
    for (unsigned b0 = 0; b0 < gridDim.x; b0 += 32 * B) {
        double y[B];
#pragma unroll
        for (int k = 0; k < B; ++k) {
            const unsigned b = b0 + lane + 32 * k;
            y[k] = b < gridDim.x ? __ldcg(part + b) : 0.0;
        }
#pragma unroll
        for (int k = 0; k < B; ++k) t += y[k];
    }
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    if (lane == 0) {
        *host_out = sqrt(t);
        *host_status = __ldcg(dstatus); // the device status word as of this norm
        *cnt = 0u;                      // ready for the next launch
    }
}

template <class Real> __global__ void __launch_bounds__(256) k_fill(Real *__restrict__ v, double c, size_t n) {
    FR_PDL_ENTRY();
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        v[q] = (Real)c;
}

// flip one component of v about u: v[i] = u[i] - (v[i] - u[i])
template <class Real> __global__ void k_flip(Real *v, const Real *u, size_t i) {
    FR_PDL_ENTRY();
    v[i] = u[i] - (v[i] - u[i]);
}

// ---- the power method's scalar logic on the device (its graph form) ----
// The same double arithmetic and tests as frgpu_spectral_radius's host loop
// (this file is built without multiply-add contraction), so both forms take the
// same iterations to the same bits.
__global__ void k_pm_start(fr_power_ctl *c, size_t n, double uround, double sq, int maxiter) {
    FR_PDL_ENTRY();
    const double ynrm = c->ynrm, vnrm = c->vnrm;
    double dynrm;
    if (ynrm != 0.0 && vnrm != 0.0) {
        dynrm = ynrm * sq;
        c->mode = 0; // v = u + (dynrm / vnrm) d0
        c->coef = dynrm / vnrm;
    } else if (ynrm != 0.0) {
        dynrm = ynrm * sq;
        c->mode = 1; // v = u + sq u
        c->coef = sq;
    } else if (vnrm != 0.0) {
        dynrm = uround;
        c->mode = 0;
        c->coef = dynrm / vnrm;
    } else {
        dynrm = uround;
        c->mode = 2; // v = dynrm / sqrt(n)
        c->coef = dynrm / sqrt((double)n);
    }
    c->dynrm = dynrm;
    c->sigma = 0.0;
    c->it = 0;
    c->done = 0;
    c->converged = 0;
    c->maxiter = maxiter;
}

template <class Real>
__global__ void __launch_bounds__(256) k_pm_vinit(Real *__restrict__ v, const Real *__restrict__ u,
                                                  const Real *__restrict__ d0, const fr_power_ctl *c, size_t n) {
    FR_PDL_ENTRY();
    const int mode = c->mode;
    const double coef = c->coef;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        if (mode == 2)
            v[q] = (Real)coef;
        else
            v[q] = u[q] + (Real)coef * (mode == 1 ? u[q] : d0[q]);
    }
}

// One iteration's estimate and test; ends the loop (condition 0) when it
// settled or reached maxiter, else prepares the update of v.
__global__ void k_pm_step(fr_power_ctl *c, size_t n, cudaGraphConditionalHandle h) {
    FR_PDL_ENTRY();
    const int it = ++c->it;
    const double dfnrm = c->dfnrm;
    const double sigmal = c->sigma;
    const double sigma = dfnrm / c->dynrm;
    c->sigma = sigma;
    if (it >= 2 && fabs(sigma - sigmal) <= fmax(sigma, 1e-300) * 0.01) {
        c->converged = 1;
        c->done = 1;
    } else if (it >= c->maxiter) {
        c->done = 1;
    } else if (dfnrm != 0.0) {
        c->mode = 0; // v = u + (dynrm / dfnrm) (f(v) - f(u))
        c->coef = c->dynrm / dfnrm;
    } else {
        c->mode = 1; // flip component it % n of v about u
        c->flip = (long)((size_t)it % n);
    }
    cudaGraphSetConditional(h, c->done ? 0u : 1u);
}

template <class Real>
__global__ void __launch_bounds__(256) k_pm_update(Real *__restrict__ v, const Real *__restrict__ u,
                                                   const Real *__restrict__ fv, const Real *__restrict__ fu,
                                                   const fr_power_ctl *c, size_t n) {
    FR_PDL_ENTRY();
    if (c->done) return;
    if (c->mode == 1) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            const size_t i = (size_t)c->flip;
            v[i] = u[i] - (v[i] - u[i]);
        }
        return;
    }
    const double coef = c->coef;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        v[q] = u[q] + (Real)coef * (fv[q] - fu[q]);
}

__global__ void k_pm_finish(const fr_power_ctl *c, double *host_rho, int *host_iters) {
    FR_PDL_ENTRY();
    *host_rho = 1.2 * c->sigma;
    *host_iters = c->converged ? c->it : -c->it;
}

} // namespace

int fr_pm_start(cudaStream_t st, fr_power_ctl *ctl, size_t n, double uround, double sq, int maxiter) {
    FR_CUDA(fr_launch(k_pm_start, 1, 1, 0, st, ctl, n, uround, sq, maxiter));
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}

int fr_pm_vinit(cudaStream_t st, bool f32, size_t n, void *v, const void *u, const void *d0, const fr_power_ctl *ctl) {
    if (f32)
        FR_CUDA(fr_launch(k_pm_vinit<float>, grid_for(n), 256, 0, st, (float *)v, (const float *)u, (const float *)d0, ctl, n));
    else
        FR_CUDA(fr_launch(k_pm_vinit<double>, grid_for(n), 256, 0, st, (double *)v, (const double *)u, (const double *)d0, ctl, n));
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}

int fr_pm_step(cudaStream_t st, fr_power_ctl *ctl, size_t n, cudaGraphConditionalHandle h) {
    FR_CUDA(fr_launch(k_pm_step, 1, 1, 0, st, ctl, n, h));
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}

int fr_pm_update(cudaStream_t st, bool f32, size_t n, void *v, const void *u, const void *fv, const void *fu,
                 const fr_power_ctl *ctl) {
    if (f32)
        FR_CUDA(fr_launch(k_pm_update<float>, grid_for(n), 256, 0, st, (float *)v, (const float *)u, (const float *)fv,
                                                        (const float *)fu, ctl, n));
    else
        FR_CUDA(fr_launch(k_pm_update<double>, grid_for(n), 256, 0, st, (double *)v, (const double *)u, (const double *)fv,
                                                         (const double *)fu, ctl, n));
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}

int fr_pm_finish(cudaStream_t st, const fr_power_ctl *ctl, double *host_rho, int *host_iters) {
    double *dr = nullptr;
    int *di = nullptr;
    FR_CUDA(cudaHostGetDevicePointer((void **)&dr, host_rho, 0));
    FR_CUDA(cudaHostGetDevicePointer((void **)&di, host_iters, 0));
    FR_CUDA(fr_launch(k_pm_finish, 1, 1, 0, st, ctl, dr, di));
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}

int fr_rock_enqueue_raw(const fr_rock_raw &r, int (*residual)(void *, const void *, void *), void *ctx) {
    return r.f32 ? rock_enqueue_t<float>(r, residual, ctx) : rock_enqueue_t<double>(r, residual, ctx);
}

int fr_vec_axpy(cudaStream_t st, bool f32, size_t n, void *out, const void *x, const void *y, double c) {
    if (f32)
        FR_CUDA(fr_launch(k_axpy<float>, grid_for(n), 256, 0, st, (float *)out, (const float *)x, (const float *)y, c, n));
    else
        FR_CUDA(fr_launch(k_axpy<double>, grid_for(n), 256, 0, st, (double *)out, (const double *)x, (const double *)y, c, n));
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}

int fr_vec_axpy_diff(cudaStream_t st, bool f32, size_t n, void *out, const void *x, const void *a, const void *b,
                     double c) {
    if (f32)
        FR_CUDA(fr_launch(k_axpy_diff<float>, grid_for(n), 256, 0, st, (float *)out, (const float *)x, (const float *)a,
                                                        (const float *)b, c, n));
    else
        FR_CUDA(fr_launch(k_axpy_diff<double>, grid_for(n), 256, 0, st, (double *)out, (const double *)x, (const double *)a,
                                                         (const double *)b, c, n));
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}

int fr_vec_fill(cudaStream_t st, bool f32, size_t n, void *v, double c) {
    if (f32)
        FR_CUDA(fr_launch(k_fill<float>, grid_for(n), 256, 0, st, (float *)v, c, n));
    else
        FR_CUDA(fr_launch(k_fill<double>, grid_for(n), 256, 0, st, (double *)v, c, n));
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}

int fr_vec_flip(cudaStream_t st, bool f32, void *v, const void *u, size_t i) {
    if (f32)
        FR_CUDA(fr_launch(k_flip<float>, 1, 1, 0, st, (float *)v, (const float *)u, i));
    else
        FR_CUDA(fr_launch(k_flip<double>, 1, 1, 0, st, (double *)v, (const double *)u, i));
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}

// ||x - y||_2 (y = null: ||x||_2) into the page-locked host word host_out and
// the device status word into host_status (their device mappings are taken
// here); d_part holds FR_RED_BLOCKS doubles, cnt a zeroed counter the kernel
// leaves at zero
int fr_vec_norm2(cudaStream_t st, bool f32, size_t n, const void *x, const void *y, double *d_part, unsigned *cnt,
                 double *host_out, const int *d_status, int *host_status) {
    double *dev_out = nullptr;
    FR_CUDA(cudaHostGetDevicePointer((void **)&dev_out, host_out, 0));
    return fr_vec_norm2_to(st, f32, n, x, y, d_part, cnt, dev_out, d_status, host_status);
}

// the same with the norm written to device memory (dev_out)
int fr_vec_norm2_to(cudaStream_t st, bool f32, size_t n, const void *x, const void *y, double *d_part, unsigned *cnt,
                    double *dev_out, const int *d_status, int *host_status) {
    int *dev_status = nullptr;
    FR_CUDA(cudaHostGetDevicePointer((void **)&dev_status, host_status, 0));
    const int nb = grid_for(n) < FR_RED_BLOCKS ? grid_for(n) : FR_RED_BLOCKS;
    if (f32)
        FR_CUDA(fr_launch(k_norm2<float>, nb, 256, 0, st, (const float *)x, (const float *)y, n, d_part, cnt, dev_out, d_status,
                                           dev_status));
    else
        FR_CUDA(fr_launch(k_norm2<double>, nb, 256, 0, st, (const double *)x, (const double *)y, n, d_part, cnt, dev_out,
                                            d_status, dev_status));
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}
