// euler2d_met_f32.cu -- FP32K instantiations of the 2D Euler residual + SSPRK3
// stage with a per-point metric (general quadrilaterals).
#include "euler2d_kernels.cuh"

int fr_euler2d_met_fp32k(frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    return dispatch_np<float, MODE_FP32K, true>(p, stage, in, din, out);
}
