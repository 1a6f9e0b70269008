// scalar1d_f32.cu -- FP32 compensated (FP32K) instantiations of the fused 1D residual + SSPRK3 stage kernels.
#include "scalar1d_kernels.cuh"

int fr_dispatch1_fp32k(int kind, frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    return dispatch1_np<float, MODE_FP32K>(kind, p, stage, in, din, out);
}
