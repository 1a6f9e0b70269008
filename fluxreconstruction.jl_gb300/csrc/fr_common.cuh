// fr_common.cuh -- device helpers shared by the flux-reconstruction kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define FR_MAXNP 8

namespace frk {

// Status bits accumulated on the device and read back by the host.
enum : int { ST_NONFINITE = 1, ST_UNPHYSICAL = 2, ST_TIMEOUT = 4 };

template <class Real> __device__ __forceinline__ Real fmaR(Real a, Real b, Real c);
template <> __device__ __forceinline__ double fmaR<double>(double a, double b, double c) { return fma(a, b, c); }
template <> __device__ __forceinline__ float fmaR<float>(float a, float b, float c) { return fmaf(a, b, c); }

template <class Real> __device__ __forceinline__ Real sqrtR(Real a);
template <> __device__ __forceinline__ double sqrtR<double>(double a) { return sqrt(a); }
template <> __device__ __forceinline__ float sqrtR<float>(float a) { return sqrtf(a); }

// Reciprocal and square root of the physics kernels: IEEE in FP64 (the
// bit-exact path), hardware approximations in FP32 (MUFU.RCP / MUFU.RSQ,
// about 2 ulp), whose error is part of the FP32 form's stated tolerance.
template <class Real> __device__ __forceinline__ Real recipR(Real a);
template <> __device__ __forceinline__ double recipR<double>(double a) { return 1.0 / a; }
template <> __device__ __forceinline__ float recipR<float>(float a) { return __fdividef(1.0f, a); }
template <class Real> __device__ __forceinline__ Real divR(Real a, Real b);
template <> __device__ __forceinline__ double divR<double>(double a, double b) { return a / b; }
template <> __device__ __forceinline__ float divR<float>(float a, float b) { return __fdividef(a, b); }
template <class Real> __device__ __forceinline__ Real sqrtP(Real a); // a >= 0
template <> __device__ __forceinline__ double sqrtP<double>(double a) { return sqrt(a); }
template <> __device__ __forceinline__ float sqrtP<float>(float a) { return a > 0.0f ? a * rsqrtf(a) : 0.0f; }

// Global load that stays where it is written.  The stage updates read their
// extra inputs (u^n, increments, low parts) only after the residual; plain
// read-only loads there may be hoisted by the compiler across the block's
// barriers to the kernel start, where they would hold registers through the
// whole residual.
__device__ __forceinline__ float ld_here(const float *p) {
    float v;
    asm volatile("ld.global.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ double ld_here(const double *p) {
    double v;
    asm volatile("ld.global.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
}

template <class Real> __device__ __forceinline__ Real absR(Real a) { return a < Real(0) ? -a : a; }
template <class Real> __device__ __forceinline__ Real maxR(Real a, Real b) { return a > b ? a : b; }
template <class Real> __device__ __forceinline__ Real minR(Real a, Real b) { return a < b ? a : b; }

// Weighted sum of NP values in a fixed order, s = v0 w0; s = fma(vq, wq, s).
// Every face trace (own element or halo neighbour) goes through this one
// routine, so both sides of a face see bit-identical traces and the interface
// flux is computed from identical inputs on both sides (exact conservation).
template <class Real, int NP>
__device__ __forceinline__ Real dotw(const Real (&v)[NP], const Real *w) {
    Real s = v[0] * w[0];
#pragma unroll
    for (int q = 1; q < NP; ++q) s = fmaR<Real>(v[q], w[q], s);
    return s;
}

// Operators of one space, passed by value (kernel parameter / constant bank).
template <class Real, int NP> struct Ops {
    Real ll[NP], lr[NP], dgl[NP], dgr[NP];
    Real D[NP][NP]; // D[m][k] = l_k'(r_m)  (lpdm, row-major)
};

// 2D Euler physical flux of conserved state w in both directions, scaled by
// the diagonal inverse Jacobian (f = iJx F, g = iJy G).  Returns pressure
// and density reciprocal through out-parameters for the status checks.
template <class Real>
__device__ __forceinline__ void euler2d_flux(const Real (&w)[4], Real gm1, Real iJx, Real iJy, Real (&f)[4],
                                             Real (&g)[4], int &bad) {
    Real rinv = recipR<Real>(w[0]);
    Real U = w[1] * rinv, V = w[2] * rinv;
    Real p = gm1 * (w[3] - Real(0.5) * fmaR<Real>(w[1], U, w[2] * V));
    Real Ep = w[3] + p;
    f[0] = iJx * w[1];
    f[1] = iJx * fmaR<Real>(w[1], U, p);
    f[2] = iJx * (w[2] * U);
    f[3] = iJx * (Ep * U);
    g[0] = iJy * w[2];
    g[1] = iJy * (w[1] * V);
    g[2] = iJy * fmaR<Real>(w[2], V, p);
    g[3] = iJy * (Ep * V);
    if (!(w[0] > Real(0)) || !(p > Real(0))) bad |= ST_UNPHYSICAL;
}

// Directional Euler flux (DIR 0 = x, 1 = y) plus normal velocity and sound speed.
template <class Real, int DIR>
__device__ __forceinline__ void euler2d_dirflux(const Real (&w)[4], Real gamma, Real gm1, Real (&f)[4], Real &un,
                                                Real &c) {
    Real rinv = recipR<Real>(w[0]);
    Real U = w[1] * rinv, V = w[2] * rinv;
    Real p = gm1 * (w[3] - Real(0.5) * fmaR<Real>(w[1], U, w[2] * V));
    un = DIR == 0 ? U : V;
    f[0] = w[1 + DIR];
    f[1] = DIR == 0 ? fmaR<Real>(w[1], U, p) : w[1] * V;
    f[2] = DIR == 1 ? fmaR<Real>(w[2], V, p) : w[2] * U;
    f[3] = (w[3] + p) * un;
    c = sqrtP<Real>(gamma * p * rinv);
}

enum { FLUX_ROE = 0, FLUX_LF = 1, FLUX_HLL = 2, FLUX_UPWIND = 3 };

// Interface flux between left/lower state wL and right/upper state wR.
// LF: local Lax-Friedrichs (Rusanov).  HLL: Davis wave-speed estimates
// (Toro, Riemann Solvers and Numerical Methods for Fluid Dynamics, ch. 10).
template <class Real, int DIR, int FLUX>
__device__ __forceinline__ void riemann2d(const Real (&wL)[4], const Real (&wR)[4], Real gamma, Real gm1,
                                          Real (&F)[4]) {
    Real fL[4], fR[4], uL, uR, cL, cR;
    euler2d_dirflux<Real, DIR>(wL, gamma, gm1, fL, uL, cL);
    euler2d_dirflux<Real, DIR>(wR, gamma, gm1, fR, uR, cR);
    if (FLUX == FLUX_LF) {
        Real lam = maxR<Real>(absR<Real>(uL) + cL, absR<Real>(uR) + cR);
#pragma unroll
        for (int m = 0; m < 4; ++m) F[m] = Real(0.5) * (fL[m] + fR[m]) - Real(0.5) * lam * (wR[m] - wL[m]);
    } else {
        Real sl = minR<Real>(uL - cL, uR - cR);
        Real sr = maxR<Real>(uL + cL, uR + cR);
        if (sl >= Real(0)) {
#pragma unroll
            for (int m = 0; m < 4; ++m) F[m] = fL[m];
        } else if (sr <= Real(0)) {
#pragma unroll
            for (int m = 0; m < 4; ++m) F[m] = fR[m];
        } else {
            Real factor = recipR<Real>(sr - sl);
#pragma unroll
            for (int m = 0; m < 4; ++m) F[m] = factor * (sr * fL[m] - sl * fR[m] + sl * sr * (wR[m] - wL[m]));
        }
    }
}

template <class Real> __device__ __forceinline__ bool finiteR(Real x) { return isfinite(x); }

} // namespace frk
