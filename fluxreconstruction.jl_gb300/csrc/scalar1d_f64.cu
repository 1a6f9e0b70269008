// scalar1d_f64.cu -- FP64 instantiations of the fused 1D residual + SSPRK3 stage kernels.
#include "scalar1d_kernels.cuh"

int fr_dispatch1_fp64(int kind, frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    return dispatch1_np<double, MODE_FP64>(kind, p, stage, in, din, out);
}
