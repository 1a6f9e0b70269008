// scalar1d.cu -- 1D dispatch (scalar advection / Burgers, 1D Euler, BGK) and the
// stateless interp_face! (src/interpolate.jl:6-10) and poly_derivative!
// (src/derivative.jl:1-10) kernels.
#include <algorithm>

#include "fr_common.cuh"
#include "frgpu_internal.h"

int fr_dispatch1_fp64(int kind, frgpu_problem *p, int stage, const void *in, const void *din, void *out);
int fr_dispatch1_fp32k(int kind, frgpu_problem *p, int stage, const void *in, const void *din, void *out);

namespace {
enum { KIND_SCALAR, KIND_EULER, KIND_BGK };

int dispatch1(int kind, frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    if (p->d.precision == FRGPU_FP64) return fr_dispatch1_fp64(kind, p, stage, in, din, out);
    return fr_dispatch1_fp32k(kind, p, stage, in, din, out);
}

// ---------------------------------------------------------------- stateless
__global__ void k_interp_face(const double *__restrict__ f, long n, int np, const double *__restrict__ ll,
                              const double *__restrict__ lr, double *__restrict__ out) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double a = f[i] * ll[0], b = f[i] * lr[0];
        for (int k = 1; k < np; ++k) {
            a = fma(f[i + n * k], ll[k], a);
            b = fma(f[i + n * k], lr[k], b);
        }
        out[i] = a;
        out[i + n] = b;
    }
}

__global__ void k_poly_derivative(const double *__restrict__ f, long n, int np, const double *__restrict__ pdm,
                                  double *__restrict__ out) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        for (int m = 0; m < np; ++m) {
            double a = f[i] * pdm[m];
            for (int k = 1; k < np; ++k) a = fma(f[i + n * k], pdm[m + np * k], a);
            out[i + n * m] = a;
        }
    }
}

} // namespace

int fr_launch_scalar1d(frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    return dispatch1(KIND_SCALAR, p, stage, in, din, out);
}
int fr_launch_euler1d(frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    return dispatch1(KIND_EULER, p, stage, in, din, out);
}
// FP32: transport on the tensor cores (bgk_tc.cu) unless the problem's
// FRGPU_OPT_BGK_TENSOR option is 0; FP64: the CUDA-core kernel
int fr_launch_bgk1d(frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    if (p->d.precision != FRGPU_FP64 && p->bgk_tensor) return fr_launch_bgk1d_tc(p, stage, in, din, out);
    return dispatch1(KIND_BGK, p, stage, in, din, out);
}

int fr_launch_interp_face(const double *d_f, long n, int np, const double *ll, const double *lr, double *d_out,
                          cudaStream_t st) {
    const int grid = (int)std::min<long>((n + 255) / 256, 4096);
    k_interp_face<<<grid > 0 ? grid : 1, 256, 0, st>>>(d_f, n, np, ll, lr, d_out);
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}

int fr_launch_poly_derivative(const double *d_f, long n, int np, const double *pdm, double *d_out, cudaStream_t st) {
    const int grid = (int)std::min<long>((n + 255) / 256, 4096);
    k_poly_derivative<<<grid > 0 ? grid : 1, 256, 0, st>>>(d_f, n, np, pdm, d_out);
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}
