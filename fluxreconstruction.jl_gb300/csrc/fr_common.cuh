// fr_common.cuh -- device helpers shared by the flux-reconstruction kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

#define FR_MAXNP 8

// Programmatic dependent launch.  A kernel launched with fr_launch starts with
// FR_PDL_ENTRY(): it waits until the previous kernel of its stream has
// completed with all its writes visible (griddepcontrol.wait; a no-op when the
// kernel was launched without the attribute), then lets the next kernel of the
// stream be scheduled, whose CTAs take SM slots as this grid's CTAs retire and
// wait at their own entry.  Launch and ramp latency of the next kernel then
// overlap this one's tail.
#define FR_PDL_ENTRY()                                                                                             \
    do {                                                                                                           \
        asm volatile("griddepcontrol.wait;" ::: "memory");                                                         \
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory");                                            \
    } while (0)

// pdl = false launches the same kernel with the ordinary stream dependency
// (measured faster for grids that fill the GPU in one wave, where early
// dependents only unbalance the next grid's placement).
template <class... KArgs, class... Args>
inline cudaError_t fr_launch_opt(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                 cudaStream_t st, Args &&...args) {
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}
template <class... KArgs, class... Args>
inline cudaError_t fr_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                             Args &&...args) {
    return fr_launch_opt(true, kernel, grid, block, smem, st, std::forward<Args>(args)...);
}

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

// Device layout of the 2D Euler state (both precisions): the 4 conserved
// variables of one solution point are adjacent, and each point's plane keeps
// the element index fastest:
//     u[(q ne + e) 4 + m],  element e = i + nx j,  point q = k + np l,  variable m.
// A thread reads or writes a whole point with one 16-byte access (FP32; two
// in FP64), and 32 consecutive elements make one contiguous 512-byte (1 KB)
// warp access.  The host arrays keep the reference's u[i, j, k, l, m];
// transfer.cu converts.
__host__ __device__ __forceinline__ size_t e2d_index(size_t e, int q, int m, size_t ne) {
    return ((size_t)q * ne + e) * 4 + (size_t)m;
}

// The 4 variables of one point: 16-byte vector loads (read-only path or
// plain) and stores.
__device__ __forceinline__ void ldg4(const float *p, float (&v)[4]) {
    const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void ldg4(const double *p, double (&v)[4]) {
    const double2 a = __ldg(reinterpret_cast<const double2 *>(p)), b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void ld4(const float *p, float (&v)[4]) {
    const float4 t = *reinterpret_cast<const float4 *>(p);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void ld4(const double *p, double (&v)[4]) {
    const double2 a = reinterpret_cast<const double2 *>(p)[0], b = reinterpret_cast<const double2 *>(p)[1];
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void st4(float *p, const float (&v)[4]) {
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st4(double *p, const double (&v)[4]) {
    reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
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

// Arithmetic on the 4 conserved variables of one point.  FP32 runs it as two
// packed pairs (variables 0-1 and 2-3) with the f32x2 instructions of sm_100+
// (__ffma2_rn, __fmul2_rn, __fadd2_rn): each lane rounds exactly as the scalar
// operation does, at half the instruction count.  FP64 runs the four scalar
// operations, in the same order as the oracle.
template <class Real> __device__ __forceinline__ void v4_mul(const Real (&a)[4], Real w, Real (&d)[4]) {
#pragma unroll
    for (int m = 0; m < 4; ++m) d[m] = a[m] * w;
}
template <class Real>
__device__ __forceinline__ void v4_fma(const Real (&a)[4], Real w, const Real (&c)[4], Real (&d)[4]) {
#pragma unroll
    for (int m = 0; m < 4; ++m) d[m] = fmaR<Real>(a[m], w, c[m]);
}
template <class Real> __device__ __forceinline__ void v4_add(const Real (&a)[4], const Real (&b)[4], Real (&d)[4]) {
#pragma unroll
    for (int m = 0; m < 4; ++m) d[m] = a[m] + b[m];
}
template <class Real> __device__ __forceinline__ void v4_sub(const Real (&a)[4], const Real (&b)[4], Real (&d)[4]) {
#pragma unroll
    for (int m = 0; m < 4; ++m) d[m] = a[m] - b[m];
}
__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
template <> __device__ __forceinline__ void v4_mul<float>(const float (&a)[4], float w, float (&d)[4]) {
    const float2 ww = f2(w, w), lo = __fmul2_rn(f2(a[0], a[1]), ww), hi = __fmul2_rn(f2(a[2], a[3]), ww);
    d[0] = lo.x; d[1] = lo.y; d[2] = hi.x; d[3] = hi.y;
}
template <>
__device__ __forceinline__ void v4_fma<float>(const float (&a)[4], float w, const float (&c)[4], float (&d)[4]) {
    const float2 ww = f2(w, w);
    const float2 lo = __ffma2_rn(f2(a[0], a[1]), ww, f2(c[0], c[1]));
    const float2 hi = __ffma2_rn(f2(a[2], a[3]), ww, f2(c[2], c[3]));
    d[0] = lo.x; d[1] = lo.y; d[2] = hi.x; d[3] = hi.y;
}
template <> __device__ __forceinline__ void v4_add<float>(const float (&a)[4], const float (&b)[4], float (&d)[4]) {
    const float2 lo = __fadd2_rn(f2(a[0], a[1]), f2(b[0], b[1])), hi = __fadd2_rn(f2(a[2], a[3]), f2(b[2], b[3]));
    d[0] = lo.x; d[1] = lo.y; d[2] = hi.x; d[3] = hi.y;
}
template <> __device__ __forceinline__ void v4_sub<float>(const float (&a)[4], const float (&b)[4], float (&d)[4]) {
    const float2 lo = __fadd2_rn(f2(a[0], a[1]), f2(-b[0], -b[1])), hi = __fadd2_rn(f2(a[2], a[3]), f2(-b[2], -b[3]));
    d[0] = lo.x; d[1] = lo.y; d[2] = hi.x; d[3] = hi.y;
}
// d = a w - c: FP64 rounds the product and the difference (the oracle's
// order); FP32 fuses them into one fma (what the FP32 build contracts it to)
template <class Real>
__device__ __forceinline__ void v4_fms(const Real (&a)[4], Real w, const Real (&c)[4], Real (&d)[4]) {
    if constexpr (sizeof(Real) == 4) {
        const Real nc[4] = {-c[0], -c[1], -c[2], -c[3]};
        v4_fma<Real>(a, w, nc, d);
    } else {
#pragma unroll
        for (int m = 0; m < 4; ++m) d[m] = a[m] * w - c[m];
    }
}
// d[m] = sum_q v[q][m] w[q] as the ascending chain of dotw, for 4 variables
template <class Real, int NP>
__device__ __forceinline__ void v4_dotw(const Real (&v)[NP][4], const Real *w, Real (&d)[4]) {
    Real s[4];
    v4_mul<Real>(v[0], w[0], s);
#pragma unroll
    for (int q = 1; q < NP; ++q) v4_fma<Real>(v[q], w[q], s, s);
#pragma unroll
    for (int m = 0; m < 4; ++m) d[m] = s[m];
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
        if constexpr (sizeof(Real) == 4) {
            // 0.5 (fL + fR) + (-0.5 lam)(wR - wL), one fma per variable
            Real s[4], d[4], h[4];
            v4_add<Real>(fL, fR, s);
            v4_sub<Real>(wR, wL, d);
            v4_mul<Real>(s, Real(0.5), h);
            v4_fma<Real>(d, Real(-0.5) * lam, h, F);
        } else {
#pragma unroll
            for (int m = 0; m < 4; ++m) F[m] = Real(0.5) * (fL[m] + fR[m]) - Real(0.5) * lam * (wR[m] - wL[m]);
        }
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
            if constexpr (sizeof(Real) == 4) {
                // factor (sr fL - sl fR + sl sr (wR - wL)), as fused pair operations
                Real d[4], t[4];
                v4_sub<Real>(wR, wL, d);
                v4_mul<Real>(fL, sr, t);
                v4_fma<Real>(fR, -sl, t, t);
                v4_fma<Real>(d, sl * sr, t, t);
                v4_mul<Real>(t, factor, F);
            } else {
#pragma unroll
                for (int m = 0; m < 4; ++m) F[m] = factor * (sr * fL[m] - sl * fR[m] + sl * sr * (wR[m] - wL[m]));
            }
        }
    }
}

// Interface flux across a face with unit normal (nx, ny): both states to the
// face frame (momentum along n and along t = (-ny, nx)), the x-direction flux,
// back to the global frame (dev/parallelogram.jl:60-73 with local_frame /
// global_frame).
template <class Real, int FLUX>
__device__ __forceinline__ void riemann_n(const Real (&wL)[4], const Real (&wR)[4], Real nx, Real ny, Real gamma,
                                          Real gm1, Real (&F)[4]) {
    const Real l[4] = {wL[0], fmaR<Real>(wL[2], ny, wL[1] * nx), fmaR<Real>(-wL[1], ny, wL[2] * nx), wL[3]};
    const Real r[4] = {wR[0], fmaR<Real>(wR[2], ny, wR[1] * nx), fmaR<Real>(-wR[1], ny, wR[2] * nx), wR[3]};
    Real f[4];
    riemann2d<Real, 0, FLUX>(l, r, gamma, gm1, f);
    F[0] = f[0];
    F[1] = fmaR<Real>(-f[2], ny, f[1] * nx);
    F[2] = fmaR<Real>(f[1], ny, f[2] * nx);
    F[3] = f[3];
}

template <class Real> __device__ __forceinline__ bool finiteR(Real x) { return isfinite(x); }

} // namespace frk
