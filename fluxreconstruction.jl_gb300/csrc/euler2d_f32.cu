// euler2d_f32.cu -- FP32 compensated (FP32K) instantiations of the fused 2D Euler residual + SSPRK3 stage.
#include "euler2d_kernels.cuh"

int fr_euler2d_fp32k(frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    return dispatch_np<float, MODE_FP32K>(p, stage, in, din, out);
}
