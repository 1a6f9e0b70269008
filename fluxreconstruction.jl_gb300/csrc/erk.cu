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
    const Real dt = (Real)*dtp;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        out[q] = frk::fmaR<Real>(dt, comb_acc<Real>(k, kstride, q, c), __ldg(u + q));
}

// step update: FP64 u = fma(dt, acc, u); FP32K compensated add of dt acc to hi + lo
template <class Real>
__global__ void __launch_bounds__(256) k_erk_update(Real *__restrict__ u, Real *__restrict__ lo,
                                                    const Real *__restrict__ k, size_t kstride, size_t n, const Comb<Real> c,
                                                    const double *dtp, int *status) {
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
                    k_erk_stage<float><<<grid_for(n), 256, 0, r.stream>>>(
                        (const float *)r.u, (const float *)kb, kstride, n, comb_of<float>(Ai, i), r.d_dt, (float *)stage);
                else
                    k_erk_stage<double><<<grid_for(n), 256, 0, r.stream>>>((const double *)r.u, (const double *)kb,
                                                                           kstride, n, comb_of<double>(Ai, i),
                                                                           r.d_dt, (double *)stage);
                FR_CUDA(cudaGetLastError());
                *r.launches += 1;
            }
            in = stage;
        }
        if ((rc = residual(ctx, in, ki))) return rc;
    }
    if (comb_of<double>(r.b, s).nt == 0 || r.prepare_only) return FRGPU_OK;
    if (r.f32)
        k_erk_update<float><<<grid_for(n), 256, 0, r.stream>>>((float *)r.u, (float *)r.lo, (const float *)kb, kstride,
                                                               n, comb_of<float>(r.b, s), r.d_dt, r.d_status);
    else
        k_erk_update<double><<<grid_for(n), 256, 0, r.stream>>>((double *)r.u, nullptr, (const double *)kb, kstride,
                                                                n, comb_of<double>(r.b, s), r.d_dt, r.d_status);
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
