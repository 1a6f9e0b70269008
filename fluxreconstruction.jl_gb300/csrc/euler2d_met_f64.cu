// euler2d_met_f64.cu -- FP64 instantiations of the 2D Euler residual + SSPRK3
// stage with a per-point metric (general quadrilaterals).
#include "euler2d_kernels.cuh"

int fr_euler2d_met_fp64(frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    return dispatch_np<double, MODE_FP64, true>(p, stage, in, din, out);
}
