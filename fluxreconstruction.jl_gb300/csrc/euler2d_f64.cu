// euler2d_f64.cu -- FP64 instantiations of the fused 2D Euler residual + SSPRK3 stage.
#include "euler2d_kernels.cuh"

int fr_euler2d_fp64(frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    return dispatch_np<double, MODE_FP64>(p, stage, in, din, out);
}
