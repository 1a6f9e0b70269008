// filter.cu -- troubled-cell indicator + :l2 modal filter, applied after a step.
//
// 2D: example/shock-vortex.jl:308-321 -- u_hat = iV rho, su = u_hat_N^2 / sum u_hat^2,
//     shock_detector(log10(su), deg, S0, kappa) (src/dissipation.jl:13-23); a troubled
//     element has every variable transformed, damped by the L2 filter
//     u_hat_q /= 1 + lam q^2 (q+1)^2 on the flattened mode index (KitBase
//     modal_filter!(u_hat, lam; filter = :l2) on the flat vector), and mapped back by V.
// 1D: example/euler_highlevel.jl:37-52 -- as above with su = u_N^2/(sum u^2 + 1e-6).
#include "fr_common.cuh"
#include "frgpu_internal.h"

using namespace frk;

namespace {

template <class Real>
__device__ __forceinline__ bool troubled_sigma(double Se, double S0, double kappa) {
    // sigma as in shock_detector; NaN falls through to sigma = 0 like the reference
    double sigma;
    if (Se < S0 - kappa)
        sigma = 1.0;
    else if (S0 - kappa <= Se && Se < S0 + kappa)
        sigma = 0.5 * (1.0 - sin(0.5 * 3.14159265358979323846 * (Se - S0) / kappa));
    else
        sigma = 0.0;
    return sigma < 0.99;
}

// Offset of variable m at point q of element e: the 1D Euler layout
// u[e, q, m] of the reference, or the 2D device layout.
template <int N, bool ONE_D> __device__ __forceinline__ size_t sidx(size_t e, int q, int m, size_t ne) {
    return ONE_D ? e + ne * ((size_t)q + (size_t)N * m) : e2d_index(e, q, m, ne);
}

template <class Real, int N, int NVAR, bool ONE_D>
__global__ void __launch_bounds__(128) k_filter(Real *u, Real *lo, size_t ne, const Real *__restrict__ V,
                                                const Real *__restrict__ iV, double lam, double S0, double kappa,
                                                int *flags, int *count) {
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    Real x[N], h[N];
#pragma unroll
    for (int q = 0; q < N; ++q) x[q] = u[sidx<N, ONE_D>(e, q, 0, ne)];
    Real tot = 0;
#pragma unroll
    for (int a = 0; a < N; ++a) {
        Real s = iV[a] * x[0];
#pragma unroll
        for (int b = 1; b < N; ++b) s = fmaR<Real>(iV[a + N * b], x[b], s);
        h[a] = s;
        tot = fmaR<Real>(s, s, tot);
    }
    const double su = ONE_D ? (double)(h[N - 1] * h[N - 1]) / ((double)tot + 1e-6)
                            : (double)(h[N - 1] * h[N - 1]) / (double)tot;
    const bool bad = troubled_sigma<Real>(log10(su), S0, kappa);
    flags[e] = bad ? 1 : 0;
    if (!bad) return;
    atomicAdd(count, 1);
#pragma unroll 1
    for (int m = 0; m < NVAR; ++m) {
#pragma unroll
        for (int q = 0; q < N; ++q) x[q] = u[sidx<N, ONE_D>(e, q, m, ne)];
#pragma unroll
        for (int a = 0; a < N; ++a) {
            Real s = iV[a] * x[0];
#pragma unroll
            for (int b = 1; b < N; ++b) s = fmaR<Real>(iV[a + N * b], x[b], s);
            h[a] = s / (Real(1) + Real(lam) * Real((double)(a + 1) * (a + 1) * (double)a * a));
        }
#pragma unroll
        for (int a = 0; a < N; ++a) {
            Real s = V[a] * h[0];
#pragma unroll
            for (int b = 1; b < N; ++b) s = fmaR<Real>(V[a + N * b], h[b], s);
            u[sidx<N, ONE_D>(e, a, m, ne)] = s;
            if (lo) lo[sidx<N, ONE_D>(e, a, m, ne)] = Real(0);
        }
    }
}

template <class Real, int N, int NVAR, bool ONE_D> int launch_filter(frgpu_problem *p, double lam, double S0, double kappa) {
    if (p->prepare_only) return FRGPU_OK;
    const size_t ne = (size_t)p->sp.nx * p->sp.ny;
    FR_CUDA(cudaMemsetAsync(p->d_count, 0, sizeof(int), p->stream));
    const int grid = (int)((ne + 127) / 128);
    k_filter<Real, N, NVAR, ONE_D><<<grid, 128, 0, p->stream>>>(
        (Real *)fr_state_hi(p), p->d.precision == FRGPU_FP32K ? (Real *)p->s3 : nullptr, ne, (const Real *)p->d_V,
        (const Real *)p->d_iV, lam, S0, kappa, p->d_flags, p->d_count);
    FR_CUDA(cudaGetLastError());
    p->launches += 1;
    return FRGPU_OK;
}

template <class Real> int filter2d_np(frgpu_problem *p, double lam, double S0, double kappa) {
    switch (p->sp.np) {
    case 2: return launch_filter<Real, 4, 4, false>(p, lam, S0, kappa);
    case 3: return launch_filter<Real, 9, 4, false>(p, lam, S0, kappa);
    case 4: return launch_filter<Real, 16, 4, false>(p, lam, S0, kappa);
    case 5: return launch_filter<Real, 25, 4, false>(p, lam, S0, kappa);
    case 6: return launch_filter<Real, 36, 4, false>(p, lam, S0, kappa);
    }
    fr_set_error("filter2d: polynomial degree must be 1..5");
    return FRGPU_ERR_UNSUPPORTED;
}

template <class Real> int filter1d_np(frgpu_problem *p, double lam, double S0, double kappa) {
    switch (p->sp.np) {
    case 2: return launch_filter<Real, 2, 3, true>(p, lam, S0, kappa);
    case 3: return launch_filter<Real, 3, 3, true>(p, lam, S0, kappa);
    case 4: return launch_filter<Real, 4, 3, true>(p, lam, S0, kappa);
    case 5: return launch_filter<Real, 5, 3, true>(p, lam, S0, kappa);
    case 6: return launch_filter<Real, 6, 3, true>(p, lam, S0, kappa);
    }
    fr_set_error("filter1d: polynomial degree must be 1..5");
    return FRGPU_ERR_UNSUPPORTED;
}

} // namespace

int fr_launch_filter2d(frgpu_problem *p, int indicator, double lam, double S0, double kappa) {
    if (!p->d_V || !p->d_iV) {
        fr_set_error("filter2d: the space has no Vandermonde matrices");
        return FRGPU_ERR_ARG;
    }
    if (indicator == FRGPU_IND_MLP) return fr_launch_mlp_indicator(p, lam, S0, kappa);
    return p->d.precision == FRGPU_FP64 ? filter2d_np<double>(p, lam, S0, kappa) : filter2d_np<float>(p, lam, S0, kappa);
}

int fr_launch_filter1d(frgpu_problem *p, int indicator, double lam, double S0, double kappa) {
    if (indicator == FRGPU_IND_MLP) {
        fr_set_error("filter1d: the learned indicator is available in 2D");
        return FRGPU_ERR_UNSUPPORTED;
    }
    if (!p->d_V || !p->d_iV) {
        fr_set_error("filter1d: the space has no Vandermonde matrices");
        return FRGPU_ERR_ARG;
    }
    return p->d.precision == FRGPU_FP64 ? filter1d_np<double>(p, lam, S0, kappa) : filter1d_np<float>(p, lam, S0, kappa);
}
