// fr_stage.cuh -- SSPRK3 stage update shared by the fused residual kernels.
#pragma once
#include "fr_common.cuh"

namespace frk {

enum { MODE_FP64 = 0, MODE_FP32K = 1 };

template <class Real>
__device__ __forceinline__ Real ld_state(const Real *__restrict__ uin, const Real *__restrict__ din, size_t idx) {
    Real v = __ldg(uin + idx);
    if (din != nullptr) v += __ldg(din + idx);
    return v;
}

// Shu-Osher SSPRK3 stage applied to one DOF with residual du.
//  FP64 (buffers hold states):   1: u1 = u + dt L;  2: u2 = (3u + u1 + dt L)/4;
//                                3: u' = (u + 2 u2 + 2 dt L)/3
//  FP32K (buffers hold increments d relative to u^n = hi + lo):
//        1: d1 = dt L;  2: d2 = (d1 + dt L)/4;  3: d3 = 2 (d2 + dt L)/3 and
//        u^{n+1} = hi + (d3 + lo) by a compensated (Fast2Sum) addition whose
//        low part is kept for the next step.
// ui = the stage input value of this DOF (u^n in stage 1).
template <class Real, int MODE, int STAGE>
__device__ __forceinline__ Real stage_update(Real du, Real ui, Real dt, size_t idx, const Real *__restrict__ un,
                                             const Real *__restrict__ uin, const Real *__restrict__ din, Real *out,
                                             Real *ul) {
    Real res;
    if (STAGE == 0) {
        res = du;
        out[idx] = res;
    } else if (MODE == MODE_FP64) {
        if (STAGE == 1) {
            res = fmaR<Real>(dt, du, ui);
        } else if (STAGE == 2) {
            res = fmaR<Real>(dt, du, fmaR<Real>(Real(3), un[idx], ui)) * Real(0.25);
        } else {
            res = fmaR<Real>(Real(2) * dt, du, fmaR<Real>(Real(2), ui, un[idx])) * Real(1.0 / 3.0);
        }
        out[idx] = res;
    } else {
        if (STAGE == 1) {
            res = dt * du;
            out[idx] = res;
        } else if (STAGE == 2) {
            res = fmaR<Real>(dt, du, __ldg(din + idx)) * Real(0.25);
            out[idx] = res;
        } else {
            const Real d3 = fmaR<Real>(dt, du, __ldg(din + idx)) * Real(2.0 / 3.0);
            const Real hi = __ldg(uin + idx);
            const Real y = d3 + ul[idx];
            const Real t = hi + y;
            ul[idx] = y - (t - hi);
            out[idx] = t;
            res = t;
        }
    }
    return res;
}

} // namespace frk
