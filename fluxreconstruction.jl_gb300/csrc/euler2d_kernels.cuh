// euler2d.cu -- fused 2D Euler flux-reconstruction residual + SSPRK3 stage.
//
// One launch evaluates the residual of example/shock-vortex.jl:26-118 (the
// dudt! closure: volume flux :48-55, face interpolation :57-71, interface
// Riemann flux :73-89, derivative :91-100, correction :102-115) on every
// element and applies one Shu-Osher SSPRK3 stage update to it.  The state is
// in the point-vector device layout (e2d_index: the 4 variables of a solution
// point together, element index fastest within a point's plane), so a thread
// moves a point with one 16-byte access and the TX consecutive elements of a
// tile row read a point plane with one contiguous TX x 16-byte access (256 or
// 512 bytes in FP32, 1 KB in FP64).
//
// CTA = TX x TY elements.  Thread (ex, ln, ey) is first an "x-line" thread
// (element ex, row s = ln: it owns the NP points along r) and later a
// "y-line" thread (element ex, column r = ln).  Shared memory carries the
// transposition between the two sweeps, the face traces and the interface
// fluxes.  Faces on the tile edge use traces of the neighbouring elements,
// recomputed from global memory (L2-resident) with the same arithmetic as the
// owner, so both sides of every face see bit-identical fluxes.
#pragma once
#include <type_traits>

#include "fr_common.cuh"
#include "frgpu_internal.h"
#include "mlp_device.cuh"

using namespace frk;

namespace {

enum { MODE_FP64 = 0, MODE_FP32K = 1 };
// troubled-cell indicator fused into the last stage: none, the learned network, the plain modal-decay test
enum { FUSE_NONE = 0, FUSE_LEARNED = 1, FUSE_PLAIN = 2 };

template <class Real, int NP> struct E2DArgs {
    int nx, ny;
    const Real *uin;  // stage input (FP64) or u^n high part (FP32K)
    const Real *din;  // FP32K: increment added to uin (stages 2, 3), else null
    const Real *un;   // FP64 stages 2, 3: u^n
    Real *out;        // residual (stage 0), next state (FP64) / increment or new high part (FP32K)
    Real *ul;         // FP32K stage 3: low part, updated in place
    const double *dtp;
    Real iJx, iJy, gamma, gm1;
    int bc[4];
    // ghosts refreshed once per step (the reference scripts copy their ghost
    // layers after each step): in the later stages of a step the periodic and
    // copy neighbours outside the domain are read from u^n, not the stage input
    // (stage 0, a residual evaluation inside an explicit or stabilised step:
    // from un, the step's start state)
    int lag;
    Real fixed[4][4];
    Ops<Real, NP> ops;
    int *status;
    // per-point inverse Jacobian (a11, a12, a21, a22) in the device layout of
    // the state (general quadrilaterals), or null for the uniform rectangles'
    // diagonal iJx, iJy
    const Real *met;
    // MET with face normals (straight-sided quadrilaterals, the formulation of
    // dev/parallelogram.jl): unit normal (nx, ny) of x face (i, j) at
    // nfx[2 (i + (nx + 1) j)], of y face (i, j) at nfy[2 (i + nx j)]; null: the
    // Cartesian axes with the dudt! scaling by a11 / a22
    const Real *nfx, *nfy;
    // with normals: the face-Jacobian form of the interface-flux scales (the
    // cylinder scripts, (inv(Ji) n) per face point): (sL, sR, sB, sT) of element e
    // at point line q at fsc[(q ne + e) 4 + c], or null for (iJ n) at the
    // solution points
    const Real *fsc;
    // stage coefficients of the method (SSPRK3: c1 = 1, fa = 1, fs = 2/3,
    // g = 2, al = 2, be = 1, s3 = 1/3; two-stage methods use stages 1 and 3):
    // stage 1: FP64 u1 = u + c1 dt L(u), FP32K d1 = c1 dt L(u); stage 3 (last):
    // FP64 (g dt L + al u_s + be u^n) s3, FP32K d = (fa d_prev + dt L) fs
    Real c1, fa, fs, g3, al3, be3, s3;
    // learned indicator fused into stage 3 (FP32K, np = 4): network, 1D inverse
    // Vandermonde factor, decision threshold / fallback band, plain-test S0 and
    // kappa, filter strength, V / iV of the filter, per-element flags and the
    // [troubled, misfires, fallbacks] counters
    frmlp::MLPDev mlp;
    frmlp::IV1 iv1;
    float ind_thr, ind_band, ind_S0, ind_kappa;
    double ind_lam;
    const Real *V, *iV;
    int *flags, *stats;
};

template <class Real, int NP, int FUSE = 0, int STAGE = 0> struct Tile;
// Tile shapes: TX elements along x, TY rows; TX x NP x TY threads.
// Shared memory per CTA (see Smem below) stays under 227 KB:
// FP64 NP=3/TY=4 158 KB, NP=4/TY=2 122 KB, NP=5/TY=1 98 KB, NP=6/TY=1 130 KB;
// FP32 NP=2/TY=8 86 KB, NP=4/TY=2 61 KB, NP=6/TY=1 65 KB.
template <int NP, int FUSE, int STAGE> struct Tile<double, NP, FUSE, STAGE> {
    static constexpr int TX = 32;
    static constexpr int TY = NP <= 3 ? 4 : (NP == 4 ? 2 : 1);
};
// FP32 np = 4: the residual and stages 1-2 take 16 x 4 tiles (40 halo traces per
// 64 elements instead of 68: 7 % and 3 % faster than 32 x 2 on the 512^2 density
// wave); stage 3, which also streams the low part, and the fused indicator keep
// 32 x 2 (8 x 8 tiles measured slower in every stage).
template <int NP, int FUSE, int STAGE> struct Tile<float, NP, FUSE, STAGE> {
    static constexpr bool V = NP == 4 && FUSE == 0 && STAGE != 3;
    static constexpr int TX = V ? 16 : 32;
    static constexpr int TY = V ? 4 : (NP <= 2 ? 8 : (NP <= 4 ? 2 : 1));
};

// NST: state-sized stash arrays holding the stage update's extra inputs,
// loaded together with the state so that their latency is not exposed after
// the residual: u^n in FP64 stages 2-3.  The FP32K stages instead read their
// extra inputs (increment; in stage 3 also the high and low parts) directly
// in the update (stage 3's low part after an L2 prefetch issued before the y
// sweep): that keeps shared memory at one residual's worth, so three CTAs fit
// on an SM.
template <int MODE, int STAGE> struct Stash {
    static constexpr int n = MODE == MODE_FP32K ? 0 : (STAGE >= 2 ? 1 : 0);
};

template <class Real, int NP, int TX, int TY, int NST = 0> struct Smem {
    static constexpr int U = TY * NP * NP * 4 * TX;
    static constexpr int TR = TY * NP * 4 * TX;
    static constexpr int HY = 2 * NP * 4 * TX;
    static constexpr int HX = 2 * TY * NP * 4;
    static constexpr int FX = TY * NP * 4 * (TX + 1);
    static constexpr int FY = (TY + 1) * NP * 4 * TX;
    static constexpr int total = 2 * U + 4 * TR + HY + HX + FX + FY + NST * U;
    static constexpr size_t bytes = sizeof(Real) * total;
};

// Element (io, jo) whose trace stands in for the neighbour at (i, j) outside
// the tile; false means the neighbour is a fixed ghost state.
__device__ __forceinline__ bool resolve(int i, int n, int bc_lo, int bc_hi, int &io) {
    if (i < 0) {
        if (bc_lo == FRGPU_BC_PERIODIC) { io = n - 1; return true; }
        if (bc_lo == FRGPU_BC_COPY) { io = 0; return true; }
        return false;
    }
    if (i >= n) {
        if (bc_hi == FRGPU_BC_PERIODIC) { io = 0; return true; }
        if (bc_hi == FRGPU_BC_COPY) { io = n - 1; return true; }
        return false;
    }
    io = i;
    return true;
}

// The 4 variables of one point of a stage input (at offset `at` of the device
// layout): uin, plus the increment din when there is one.
template <class Real>
__device__ __forceinline__ void ld_state4(const Real *__restrict__ uin, const Real *__restrict__ din, unsigned at,
                                          Real (&v)[4]) {
    ldg4(uin + at, v);
    if (din != nullptr) {
        Real d[4];
        ldg4(din + at, d);
        v4_add<Real>(v, d, v);
    }
}

// Shared-memory arrays keep the 4 conserved variables of a slot in 16-byte
// chunks (4 floats or 2 doubles): variable m of slot s at lane x of a row of W
// lanes sits at ((s * NC + m / VW) * W + x) * VW + m % VW.  A thread moves all
// 4 variables with NC 16-byte accesses, and a warp's lanes touch consecutive
// chunks (conflict-free).  cs is the distance between a slot's chunks.
template <class Real> struct Vec {
    static constexpr int VW = 16 / (int)sizeof(Real);
    static constexpr int NC = 4 / VW;
};
__device__ __forceinline__ void st16(float *p, const float *v) {
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st16(double *p, const double *v) {
    *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
}
__device__ __forceinline__ void ld16(const float *p, float *v) {
    const float4 t = *reinterpret_cast<const float4 *>(p);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void ld16(const double *p, double *v) {
    const double2 t = *reinterpret_cast<const double2 *>(p);
    v[0] = t.x; v[1] = t.y;
}
template <class Real> __device__ __forceinline__ void put4(Real *p, int cs, const Real (&v)[4]) {
#pragma unroll
    for (int c = 0; c < Vec<Real>::NC; ++c) st16(p + c * cs, v + c * Vec<Real>::VW);
}
template <class Real> __device__ __forceinline__ void get4(const Real *p, int cs, Real (&v)[4]) {
#pragma unroll
    for (int c = 0; c < Vec<Real>::NC; ++c) ld16(p + c * cs, v + c * Vec<Real>::VW);
}

// FP32 CTAs of up to 256 threads: registers capped so that three CTAs share an SM
// FUSE: stage 3 of the FP32K form with np = 4 also runs the troubled-cell
// indicator + :l2 filter on the elements it has just updated (the post-step
// filter of example/shock-vortex.jl:308-321): the learned network of mlp.cu
// (FUSE_LEARNED), or the plain modal-decay test of src/dissipation.jl:13-23
// (FUSE_PLAIN) on the same features, so that the two forms differ only in the
// decision.
// MET: per-point metric a.met (f = a11 F + a12 G, g = a21 F + a22 G; the
// corrections scale the interface fluxes by a11 and a22 at each point, as the
// dudt! closure of example/shock-vortex.jl:48-55, :102-115 does with iJ[i, j][k, l]).
template <class Real, int NP, int FLUX, int MODE, int STAGE, int FUSE = FUSE_NONE, bool MET = false>
__global__ void __launch_bounds__(Tile<Real, NP, FUSE, STAGE>::TX * NP * Tile<Real, NP, FUSE, STAGE>::TY,
                                  sizeof(Real) == 4 && Tile<Real, NP, FUSE, STAGE>::TX * NP * Tile<Real, NP, FUSE, STAGE>::TY <= 256 ? 3 : 1)
    k_euler2d(const E2DArgs<Real, NP> a) {
    FR_PDL_ENTRY(); // launched by fr_launch: the previous kernel's writes are visible from here on
    // stage 1 of a step whose third stage runs the fused indicator zeroes that
    // indicator's counters (a.stats), so that no memset separates the stages
    if (STAGE == 1 && a.stats != nullptr && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x < 4)
        a.stats[threadIdx.x] = 0;
    constexpr int TX = Tile<Real, NP, FUSE, STAGE>::TX, TY = Tile<Real, NP, FUSE, STAGE>::TY;
    constexpr int NT = TX * NP * TY;
    constexpr int NST = Stash<MODE, STAGE>::n;
    using S = Smem<Real, NP, TX, TY, NST>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real *s_u = reinterpret_cast<Real *>(smem_raw);
    Real *s_g = s_u + S::U;
    Real *s_uxl = s_g + S::U;
    Real *s_uxr = s_uxl + S::TR;
    Real *s_uyb = s_uxr + S::TR;
    Real *s_uyt = s_uyb + S::TR;
    Real *s_hy = s_uyt + S::TR;
    Real *s_hx = s_hy + S::HY;
    Real *s_Fx = s_hx + S::HX;
    Real *s_Fy = s_Fx + S::FX;
    Real *s_st = s_Fy + S::FY;
    constexpr int VW = Vec<Real>::VW, NC = Vec<Real>::NC;
#define VIX(sl, m, x, W) ((((sl) * NC + (m) / VW) * (W) + (x)) * VW + (m) % VW)
#define SST(q, ey, l, k, m, ex) s_st[(q) * S::U + VIX(((ey) * NP + (l)) * NP + (k), m, ex, TX)]
#define SU(ey, l, k, m, ex) s_u[VIX(((ey) * NP + (l)) * NP + (k), m, ex, TX)]
#define SG(ey, l, k, m, ex) s_g[VIX(((ey) * NP + (l)) * NP + (k), m, ex, TX)]
#define STR(arr, ey, q, m, ex) arr[VIX((ey) * NP + (q), m, ex, TX)]
#define SHY(side, k, m, ex) s_hy[VIX((side) * NP + (k), m, ex, TX)]
#define SHX(side, ey, l, m) s_hx[(((side) * TY + (ey)) * NP + (l)) * 4 + (m)]
#define SFX(ey, l, m, f) s_Fx[VIX((ey) * NP + (l), m, f, TX + 1)]
#define SFY(fy, k, m, ex) s_Fy[VIX((fy) * NP + (k), m, ex, TX)]
    // chunk strides: rows of TX lanes, the TX + 1 x-faces, and the contiguous SHX
    constexpr int CS = TX * VW, CSF = (TX + 1) * VW, CSX = VW;

    const int tid = threadIdx.x;
    const int ex = tid % TX, ln = (tid / TX) % NP, ey = tid / (TX * NP);
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
    const int nx = a.nx, ny = a.ny;
    const int vx = min(TX, nx - i0), vy = min(TY, ny - j0);
    const bool valid = ex < vx && ey < vy;
    // 32-bit offsets into the state arrays (problem_create keeps every array
    // below 2^32 values); 64-bit products of the plane stride cost the kernel
    // about 50 registers per thread
    const unsigned plane = (unsigned)nx * (unsigned)ny;
    const Real *__restrict__ uin = a.uin;
    const Real *__restrict__ din = a.din;
    const Ops<Real, NP> &op = a.ops;
    int bad = 0;

    // interface flux across x face (fi, fj) / y face (fi, fj): rotated into the
    // face frame when the problem has face normals, else along the axis
    const auto xflux = [&](const Real (&wL)[4], const Real (&wR)[4], int fi, int fj, Real (&F)[4]) {
        if constexpr (MET) {
            if (a.nfx != nullptr) {
                const Real *n = a.nfx + 2 * ((unsigned)fi + (unsigned)(nx + 1) * fj);
                riemann_n<Real, FLUX>(wL, wR, n[0], n[1], a.gamma, a.gm1, F);
                return;
            }
        }
        riemann2d<Real, 0, FLUX>(wL, wR, a.gamma, a.gm1, F);
    };
    const auto yflux = [&](const Real (&wL)[4], const Real (&wR)[4], int fi, int fj, Real (&F)[4]) {
        if constexpr (MET) {
            if (a.nfy != nullptr) {
                const Real *n = a.nfy + 2 * ((unsigned)fi + (unsigned)nx * fj);
                riemann_n<Real, FLUX>(wL, wR, n[0], n[1], a.gamma, a.gm1, F);
                return;
            }
        }
        riemann2d<Real, 1, FLUX>(wL, wR, a.gamma, a.gm1, F);
    };

    // ---- phase A loads, issued before the halo so that both are in flight ----
    const int i = i0 + ex, j = j0 + ey;
    const unsigned e = (unsigned)i + (unsigned)nx * j;
    Real u[NP][4];
    {
        const int l = ln;
        if (valid) {
#pragma unroll
            for (int k = 0; k < NP; ++k) {
                const unsigned at = ((unsigned)(k + NP * l) * plane + e) * 4;
                ldg4(uin + at, u[k]);
                if (MODE == MODE_FP32K && STAGE >= 2) {
                    Real d[4];
                    ldg4(din + at, d);
                    v4_add<Real>(u[k], d, u[k]); // u^n high part + increment
                }
                if (MODE == MODE_FP64 && STAGE >= 2) {
                    Real un[4];
                    ldg4(a.un + at, un);
                    put4(&SST(0, ey, l, k, 0, ex), CS, un);
                }
            }
        } else {
#pragma unroll
            for (int k = 0; k < NP; ++k) {
                u[k][0] = Real(1); u[k][1] = Real(0); u[k][2] = Real(0); u[k][3] = Real(1);
            }
        }
    }

    // ---- halo: traces of the neighbours across the tile edges --------------
    for (int t = tid; t < 2 * NP * (TX + TY); t += NT) {
        if (t < 2 * NP * TX) {
            const int hx = t % TX, hk = (t / TX) % NP, side = t / (TX * NP);
            if (hx >= vx) continue;
            // side 0: row below needs its top trace (lr along s);
            // side 1: row above needs its bottom trace (ll along s)
            const int jn = side == 0 ? j0 - 1 : j0 + vy;
            const Real *w = side == 0 ? op.lr : op.ll;
            int jo;
            if (resolve(jn, ny, a.bc[2], a.bc[3], jo)) {
                const unsigned en = (unsigned)(i0 + hx) + (unsigned)nx * jo;
                // a ghost outside the domain with ghosts refreshed once per step: u^n
                const bool lag = (STAGE >= 2 || STAGE == 0) && a.lag && (jn < 0 || jn >= ny);
                const Real *src = (MODE == MODE_FP64 || STAGE == 0) && lag ? a.un : uin;
                const Real *dsrc = lag ? nullptr : din;
                Real v[NP][4], h[4];
#pragma unroll
                for (int l = 0; l < NP; ++l) ld_state4(src, dsrc, ((unsigned)(hk + NP * l) * plane + en) * 4, v[l]);
                v4_dotw<Real, NP>(v, w, h);
                put4(&SHY(side, hk, 0, hx), CS, h);
            } else {
                const int s = side == 0 ? 2 : 3;
                Real h[4];
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    Real v[NP];
#pragma unroll
                    for (int l = 0; l < NP; ++l) v[l] = a.fixed[s][m];
                    h[m] = dotw<Real, NP>(v, w);
                }
                put4(&SHY(side, hk, 0, hx), CS, h);
            }
        } else {
            const int u = t - 2 * NP * TX;
            const int hy = u % TY, hl = (u / TY) % NP, side = u / (TY * NP);
            if (hy >= vy) continue;
            // side 0: left neighbour needs its right trace (lr along r);
            // side 1: right neighbour needs its left trace (ll along r)
            const int in_ = side == 0 ? i0 - 1 : i0 + vx;
            const Real *w = side == 0 ? op.lr : op.ll;
            int io;
            if (resolve(in_, nx, a.bc[0], a.bc[1], io)) {
                const unsigned en = (unsigned)io + (unsigned)nx * (j0 + hy);
                const bool lag = (STAGE >= 2 || STAGE == 0) && a.lag && (in_ < 0 || in_ >= nx);
                const Real *src = (MODE == MODE_FP64 || STAGE == 0) && lag ? a.un : uin;
                const Real *dsrc = lag ? nullptr : din;
                Real v[NP][4], h[4];
#pragma unroll
                for (int k = 0; k < NP; ++k) ld_state4(src, dsrc, ((unsigned)(k + NP * hl) * plane + en) * 4, v[k]);
                v4_dotw<Real, NP>(v, w, h);
                put4(&SHX(side, hy, hl, 0), CSX, h);
            } else {
                Real h[4];
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    Real v[NP];
#pragma unroll
                    for (int k = 0; k < NP; ++k) v[k] = a.fixed[side][m];
                    h[m] = dotw<Real, NP>(v, w);
                }
                put4(&SHX(side, hy, hl, 0), CSX, h);
            }
        }
    }

    // ---- phase A: x-line (element ex, row l = ln) --------------------------
    Real rx[NP][4], fxl[4], fxr[4];
    {
        const int l = ln;
        Real fx[NP][4], gy[NP][4];
        if constexpr (MET) {
#pragma unroll
            for (int k = 0; k < NP; ++k) {
                Real F[4], G[4], mt[4] = {Real(0), Real(0), Real(0), Real(0)};
                euler2d_flux<Real>(u[k], a.gm1, Real(1), Real(1), F, G, bad);
                if (valid) ldg4(a.met + ((unsigned)(k + NP * l) * plane + e) * 4, mt);
                v4_mul<Real>(F, mt[0], fx[k]);
                v4_fma<Real>(G, mt[1], fx[k], fx[k]);
                v4_mul<Real>(F, mt[2], gy[k]);
                v4_fma<Real>(G, mt[3], gy[k], gy[k]);
            }
        } else {
#pragma unroll
            for (int k = 0; k < NP; ++k) euler2d_flux<Real>(u[k], a.gm1, a.iJx, a.iJy, fx[k], gy[k], bad);
        }
        Real tl[4], tr[4];
#pragma unroll
        for (int k = 0; k < NP; ++k) v4_dotw<Real, NP>(fx, op.D[k], rx[k]);
        v4_dotw<Real, NP>(u, op.ll, tl);
        v4_dotw<Real, NP>(u, op.lr, tr);
        v4_dotw<Real, NP>(fx, op.ll, fxl);
        v4_dotw<Real, NP>(fx, op.lr, fxr);
        put4(&STR(s_uxl, ey, l, 0, ex), CS, tl);
        put4(&STR(s_uxr, ey, l, 0, ex), CS, tr);
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            put4(&SU(ey, l, k, 0, ex), CS, u[k]);
            put4(&SG(ey, l, k, 0, ex), CS, gy[k]);
        }
    }
    __syncthreads();

    // ---- phase B: y-line (element ex, column k = ln) + x interface flux ----
    Real ry[NP][4], gyb[4], gyt[4];
    {
        const int k = ln;
        {
            Real col[NP][4], tb[4], tt[4];
#pragma unroll
            for (int l = 0; l < NP; ++l) get4(&SU(ey, l, k, 0, ex), CS, col[l]);
            v4_dotw<Real, NP>(col, op.ll, tb);
            v4_dotw<Real, NP>(col, op.lr, tt);
            put4(&STR(s_uyb, ey, k, 0, ex), CS, tb);
            put4(&STR(s_uyt, ey, k, 0, ex), CS, tt);
        }
        {
            Real col[NP][4];
#pragma unroll
            for (int l = 0; l < NP; ++l) get4(&SG(ey, l, k, 0, ex), CS, col[l]);
#pragma unroll
            for (int l = 0; l < NP; ++l) v4_dotw<Real, NP>(col, op.D[l], ry[l]);
            v4_dotw<Real, NP>(col, op.ll, gyb);
            v4_dotw<Real, NP>(col, op.lr, gyt);
        }
        // x interface flux at the left face of element ex (row l = ln)
        if (valid) {
            const int l = ln;
            Real wL[4], wR[4], F[4];
            if (ex > 0) get4(&STR(s_uxr, ey, l, 0, ex - 1), CS, wL);
            else get4(&SHX(0, ey, l, 0), CSX, wL);
            get4(&STR(s_uxl, ey, l, 0, ex), CS, wR);
            xflux(wL, wR, i, j, F);
            put4(&SFX(ey, l, 0, ex), CSF, F);
        }
        // the TY * NP faces on the tile's right edge, by the first threads of
        // warp 0 only (an extra solve on every warp's last lane would make all
        // warps wait for it)
        if (tid < TY * NP) {
            const int ye = tid / NP, le = tid % NP;
            if (ye < vy) {
                Real wL[4], wR[4], F[4];
                get4(&STR(s_uxr, ye, le, 0, vx - 1), CS, wL);
                get4(&SHX(1, ye, le, 0), CSX, wR);
                xflux(wL, wR, i0 + vx, j0 + ye, F);
                put4(&SFX(ye, le, 0, vx), CSF, F);
            }
        }
    }
    __syncthreads();

    // ---- phase C: y interface flux; x correction into s_g -------------------
    // FP32K stage 3: bring the low part of this thread's column into L2 now;
    // phase D reads it after the Riemann solves and corrections.  (The high
    // part and the increments were just read by the CTA's row threads and are
    // L2-resident already; prefetching them as well measured slower.)
    if (MODE == MODE_FP32K && STAGE == 3 && valid) {
#pragma unroll
        for (int l = 0; l < NP; ++l) {
            const unsigned at = ((unsigned)(ln + NP * l) * plane + e) * 4;
            asm volatile("prefetch.global.L2 [%0];" ::"l"(a.ul + at));
        }
    }
    {
        const int k = ln;
        if (valid) {
            Real wL[4], wR[4], F[4];
            get4(ey > 0 ? &STR(s_uyt, ey - 1, k, 0, ex) : &SHY(0, k, 0, ex), CS, wL);
            get4(&STR(s_uyb, ey, k, 0, ex), CS, wR);
            yflux(wL, wR, i, j, F);
            put4(&SFY(ey, k, 0, ex), CS, F);
            if (ey == vy - 1) {
                get4(&STR(s_uyt, ey, k, 0, ex), CS, wL);
                get4(&SHY(1, k, 0, ex), CS, wR);
                yflux(wL, wR, i, j + 1, F);
                put4(&SFY(ey + 1, k, 0, ex), CS, F);
            }
            // x correction of row l = ln: rx + (F*_L iJx - f_L) dgl + (F*_R iJx - f_R) dgr
            const int l = ln;
            Real FL[4], FR[4], aL[4], aR[4];
            get4(&SFX(ey, l, 0, ex), CSF, FL);
            get4(&SFX(ey, l, 0, ex + 1), CSF, FR);
            if constexpr (!MET) {
                v4_fms<Real>(FL, a.iJx, fxl, aL);
                v4_fms<Real>(FR, a.iJx, fxr, aR);
            }
            [[maybe_unused]] Real fsL = Real(0), fsR = Real(0);
            if constexpr (MET) {
                if (a.fsc != nullptr) {
                    fsL = __ldg(a.fsc + ((unsigned)l * plane + e) * 4);
                    fsR = __ldg(a.fsc + ((unsigned)l * plane + e) * 4 + 1);
                }
            }
#pragma unroll
            for (int kk = 0; kk < NP; ++kk) {
                if constexpr (MET) {
                    // a11 at point (kk, l); with normals (iJ n)_1 of the left and right faces,
                    // or the face-Jacobian scales of the face points
                    const unsigned at = ((unsigned)(kk + NP * l) * plane + e) * 4;
                    Real sL = __ldg(a.met + at), sR = sL;
                    if (a.fsc != nullptr) {
                        sL = fsL;
                        sR = fsR;
                    } else if (a.nfx != nullptr) {
                        const Real a12 = __ldg(a.met + at + 1);
                        const Real *nL = a.nfx + 2 * ((unsigned)i + (unsigned)(nx + 1) * j);
                        sL = fmaR<Real>(a12, nL[1], sR * nL[0]);
                        sR = fmaR<Real>(a12, nL[3], sR * nL[2]);
                    }
                    v4_fms<Real>(FL, sL, fxl, aL);
                    v4_fms<Real>(FR, sR, fxr, aR);
                }
                Real g[4];
                v4_fma<Real>(aL, op.dgl[kk], rx[kk], g);
                v4_fma<Real>(aR, op.dgr[kk], g, g);
                put4(&SG(ey, l, kk, 0, ex), CS, g);
            }
        }
    }
    __syncthreads();

    // ---- phase D: y correction, residual, stage update (column k = ln) ------
    if (valid) {
        const int k = ln;
        const Real dt = (Real)(*a.dtp);
        Real chk[4] = {Real(0), Real(0), Real(0), Real(0)};
        Real FB[4], FT[4], bB[4], bT[4];
        get4(&SFY(ey, k, 0, ex), CS, FB);
        get4(&SFY(ey + 1, k, 0, ex), CS, FT);
        if constexpr (!MET) {
            v4_fms<Real>(FB, a.iJy, gyb, bB);
            v4_fms<Real>(FT, a.iJy, gyt, bT);
        }
        [[maybe_unused]] Real fsB = Real(0), fsT = Real(0);
        if constexpr (MET) {
            if (a.fsc != nullptr) {
                fsB = __ldg(a.fsc + ((unsigned)k * plane + e) * 4 + 2);
                fsT = __ldg(a.fsc + ((unsigned)k * plane + e) * 4 + 3);
            }
        }
#pragma unroll
        for (int l = 0; l < NP; ++l) {
            if constexpr (MET) {
                // a22 at point (k, l); with normals (iJ n)_2 of the bottom and top faces,
                // or the face-Jacobian scales of the face points
                const unsigned at = ((unsigned)(k + NP * l) * plane + e) * 4;
                Real sB = __ldg(a.met + at + 3), sT = sB;
                if (a.fsc != nullptr) {
                    sB = fsB;
                    sT = fsT;
                } else if (a.nfy != nullptr) {
                    const Real a21 = __ldg(a.met + at + 2);
                    const Real *nB = a.nfy + 2 * ((unsigned)i + (unsigned)nx * j), *nT = nB + 2 * nx;
                    sB = fmaR<Real>(sT, nB[1], a21 * nB[0]);
                    sT = fmaR<Real>(sT, nT[1], a21 * nT[0]);
                }
                v4_fms<Real>(FB, sB, gyb, bB);
                v4_fms<Real>(FT, sT, gyt, bT);
            }
            // r = -du/dt at the NP points of row l, column k, all 4 variables
            Real r[4], res[4];
            get4(&SG(ey, l, k, 0, ex), CS, r);
            v4_add<Real>(r, ry[l], r);
            v4_fma<Real>(bB, op.dgl[l], r, r);
            v4_fma<Real>(bT, op.dgr[l], r, r);
            const unsigned at = ((unsigned)(k + NP * l) * plane + e) * 4;
            if (STAGE == 0) {
#pragma unroll
                for (int m = 0; m < 4; ++m) res[m] = -r[m];
                st4(a.out + at, res);
            } else if (MODE == MODE_FP64) {
                Real ui4[4], un4[4];
                get4(&SU(ey, l, k, 0, ex), CS, ui4);
                if (STAGE >= 2) get4(&SST(0, ey, l, k, 0, ex), CS, un4);
                if (STAGE == 3 && a.be3 != Real(1)) { // two-stage methods other than Midpoint
#pragma unroll
                    for (int m = 0; m < 4; ++m) un4[m] *= a.be3;
                }
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    const Real du = -r[m], ui = ui4[m];
                    if (STAGE == 1) {
                        res[m] = fmaR<Real>(a.c1 * dt, du, ui);
                    } else if (STAGE == 2) {
                        res[m] = (fmaR<Real>(dt, du, fmaR<Real>(Real(3), un4[m], ui))) * Real(0.25);
                    } else {
                        res[m] = fmaR<Real>(a.g3 * dt, du, fmaR<Real>(a.al3, ui, un4[m])) * a.s3;
                    }
                }
                st4(a.out + at, res);
            } else {
                // FP32K: stage values are u^n + d; only increments are stored,
                // and the step's total increment is added to u^n with a
                // compensated (Kahan/Fast2Sum) sum whose low part persists.
                // dt du = (-dt) r exactly.
                if (STAGE == 1) {
                    v4_mul<Real>(r, -(a.c1 * dt), res);
                } else if (STAGE == 2) {
                    Real d1[4];
                    ldg4(din + at, d1);
                    v4_fma<Real>(r, -dt, d1, res);
                    v4_mul<Real>(res, Real(0.25), res);
                } else {
                    Real d2[4], hi[4], lo[4], y[4], c[4];
                    ldg4(din + at, d2);
                    ldg4(uin + at, hi);
                    ld4(a.ul + at, lo);
                    if (a.fa != Real(1)) v4_mul<Real>(d2, a.fa, d2);
                    v4_fma<Real>(r, -dt, d2, y);
                    v4_mul<Real>(y, a.fs, y); // d3
                    v4_add<Real>(y, lo, y);               // y = d3 + lo
                    v4_add<Real>(hi, y, res);             // t = hi + y
                    v4_sub<Real>(res, hi, c);
                    v4_sub<Real>(y, c, lo);               // lo_new = y - (t - hi)
                    st4(a.ul + at, lo);
                    // u is dead in FP32K phase D: with the fused indicator it now holds u^{n+1}
                    if (FUSE != FUSE_NONE) put4(&SU(ey, l, k, 0, ex), CS, res);
                }
                st4(a.out + at, res);
            }
            v4_add<Real>(chk, res, chk); // NaN and Inf propagate into the check sums
        }
        if (!isfinite(chk[0] + chk[1] + chk[2] + chk[3])) bad |= ST_NONFINITE;
    }
    if (bad) atomicOr(a.status, bad);

    // ---- fused learned indicator (FP32K stage 3, np = 4) --------------------
    // Warps 0-3 each take 16 elements of the tile (one half-row): features from
    // the new state in shared memory, the network (weights through L1; staging
    // them in shared memory per CTA measured slower), the
    // decision with the plain test as fallback and judge, and the :l2 filter
    // of the troubled elements in global memory.
    if constexpr (FUSE != FUSE_NONE) {
        static_assert(NP == 4 && TX == 32 && TY == 2, "the fused indicator works on 32 x 2 tiles of np = 4");
        __syncthreads();
        const int warp = tid >> 5, lane = tid & 31;
        if (warp < 4) {
            using namespace frmlp;
            __nv_bfloat16 *xs = reinterpret_cast<__nv_bfloat16 *>(s_g) + warp * 16 * NIN;
            float *prob = reinterpret_cast<float *>(s_g) + 2 * 16 * NIN + warp * 16;
            const int h = warp & 1, eyt = warp >> 1;
            const int exl = 16 * h + (lane & 15);
            const bool pr = lane >= 16;
            const bool ev = exl < vx && eyt < vy;
            float w[8][4];
#pragma unroll
            for (int kq = 0; kq < 8; ++kq) {
                const int q = (pr ? 8 : 0) + kq, kk = q & 3, ll = q >> 2;
                Real t4[4];
                get4(&SU(eyt, ll, kk, 0, exl), CS, t4);
#pragma unroll
                for (int m = 0; m < 4; ++m) w[kq][m] = ev ? (float)t4[m] : (m == 0 ? 1.f : 0.f);
            }
            float feat[16], su = 0.f;
            features_from_raw(w, ev, pr, a.iv1, (float)a.gm1, feat, su);
            // elements the network is consulted for (su is valid on the lower lanes)
            [[maybe_unused]] const bool cand = !pr && ev && !below_floor(su, a.ind_S0, a.ind_kappa);
            if constexpr (FUSE == FUSE_LEARNED) {
                // a warp whose 16 elements are all below the smooth floor skips the network
                if (__any_sync(0xffffffffu, cand)) {
                    store_features_bf16(xs + (lane & 15) * NIN + (pr ? 16 : 0), feat);
                    __syncwarp();
                    Fwd f;
                    // 12 KB of weights, L1-resident; warp-level mma.sync: the tcgen05 routine of the
                    // stand-alone kernel measured slower here (per-CTA TMEM allocation, weight
                    // copy and two MMA round trips for only 64 elements)
                    mlp_forward_tile(global_view(a.mlp), xs, f);
                    if ((lane & 3) == 0) {
                        prob[lane >> 2] = sigmoidf_(f.logit_g);
                        prob[(lane >> 2) + 8] = sigmoidf_(f.logit_g8);
                    }
                    __syncwarp();
                }
            }
            bool tr = false;
            int n_tr = 0, n_mis = 0, n_fb = 0;
            if (!pr && ev) {
                const bool plain = plain_troubled(su, a.ind_S0, a.ind_kappa);
                if constexpr (FUSE == FUSE_LEARNED) {
                    const float pm = cand ? prob[lane] : 0.f;
                    const bool fb = fabsf(pm - a.ind_thr) < a.ind_band, net = pm > a.ind_thr;
                    tr = fb ? plain : net;
                    n_mis = net != plain;
                    n_fb = fb;
                } else {
                    tr = plain;
                }
                n_tr = tr;
                a.flags[(i0 + exl) + nx * (j0 + eyt)] = tr ? 1 : 0;
            }
            const size_t ebase = (size_t)(i0 + 16 * h) + (size_t)nx * (j0 + eyt);
            warp_filter_elements<Real>(__ballot_sync(0xffffffffu, tr), ebase, a.out, a.ul, plane, a.V, a.iV,
                                       a.ind_lam);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                n_tr += __shfl_xor_sync(0xffffffffu, n_tr, off);
                n_mis += __shfl_xor_sync(0xffffffffu, n_mis, off);
                n_fb += __shfl_xor_sync(0xffffffffu, n_fb, off);
            }
            if (lane == 0) {
                if (n_tr) atomicAdd(&a.stats[0], n_tr);
                if (n_mis) atomicAdd(&a.stats[1], n_mis);
                if (n_fb) atomicAdd(&a.stats[2], n_fb);
            }
        }
    }
#undef SU
#undef SG
#undef STR
#undef SHY
#undef SHX
#undef SFX
#undef SFY
#undef SST
#undef VIX
}

template <class Real, int NP> Ops<Real, NP> make_ops(const frgpu_space &s) {
    Ops<Real, NP> o;
    for (int k = 0; k < NP; ++k) {
        o.ll[k] = (Real)s.ll[k];
        o.lr[k] = (Real)s.lr[k];
        o.dgl[k] = (Real)s.dhl[k];
        o.dgr[k] = (Real)s.dhr[k];
        for (int q = 0; q < NP; ++q) o.D[k][q] = (Real)s.dl[k + NP * q];
    }
    return o;
}

template <class Real, int NP, int FLUX, int MODE, int STAGE, int FUSE = FUSE_NONE, bool MET = false>
int launch_t(frgpu_problem *p, const void *in, const void *din, void *out) {
    using T = Tile<Real, NP, FUSE, STAGE>;
    using S = Smem<Real, NP, T::TX, T::TY, Stash<MODE, STAGE>::n>;
    E2DArgs<Real, NP> a;
    a.nx = p->sp.nx;
    a.ny = p->sp.ny;
    a.uin = (const Real *)in;
    a.din = (const Real *)din;
    a.un = (const Real *)p->s0;
    a.out = (Real *)out;
    a.ul = (Real *)p->s3;
    a.dtp = p->d_dt;
    a.iJx = (Real)(1.0 / (0.5 * p->sp.dx));
    a.iJy = (Real)(1.0 / (0.5 * p->sp.dy));
    a.gamma = (Real)p->d.gamma;
    a.gm1 = (Real)(p->d.gamma - 1.0);
    for (int s = 0; s < 4; ++s) {
        a.bc[s] = p->d.bc[s];
        for (int m = 0; m < 4; ++m) a.fixed[s][m] = (Real)p->d.fixed_state[s][m];
    }
    a.lag = p->ghosts_per_step;
    if (STAGE == 0) { // a residual inside a step: the step's start state, when the stepper gives one
        a.lag = p->ghosts_per_step && p->lag_src != nullptr;
        if (a.lag) a.un = (const Real *)p->lag_src;
    }
    a.ops = make_ops<Real, NP>(p->sp);
    a.status = p->d_status;
    a.mlp = frmlp::MLPDev{nullptr, nullptr, nullptr, nullptr, nullptr};
    a.V = a.iV = nullptr;
    a.flags = a.stats = nullptr;
    if (STAGE == 1 && fr_fused_indicator(p) != FRGPU_IND_NONE) a.stats = p->d_count;
    if (FUSE == FUSE_LEARNED) {
        const fr_mlp_ptrs m = fr_mlp_device(p->mlp);
        a.mlp = frmlp::MLPDev{m.P, (const __nv_bfloat16 *)m.W1, (const __nv_bfloat16 *)m.W2,
                              (const __nv_bfloat16 *)m.W2T, m.TC};
        a.ind_thr = p->mlp_thr;
        a.ind_band = p->mlp_band;
    }
    if (FUSE != FUSE_NONE) {
        fr_iv1_from_tensor(p->sp, &a.iv1.m[0][0]);
        a.ind_S0 = (float)p->S0;
        a.ind_kappa = (float)p->kappa;
        a.ind_lam = p->lam;
        a.V = (const Real *)p->d_V;
        a.iV = (const Real *)p->d_iV;
        a.flags = p->d_flags;
        a.stats = p->d_count;
    }
    static_assert(S::bytes <= 227 * 1024, "shared memory per CTA exceeds 227 KB");
    a.met = MET ? (const Real *)p->d_met : nullptr;
    a.nfx = MET ? (const Real *)p->d_nfx : nullptr;
    a.nfy = MET ? (const Real *)p->d_nfy : nullptr;
    a.fsc = MET ? (const Real *)p->d_fsc : nullptr;
    a.c1 = (Real)p->meth.c1;
    a.fa = (Real)p->meth.fa;
    a.fs = (Real)p->meth.fs;
    a.g3 = (Real)p->meth.g3;
    a.al3 = (Real)p->meth.al3;
    a.be3 = (Real)p->meth.be3;
    a.s3 = (Real)p->meth.s3;
    auto kern = k_euler2d<Real, NP, FLUX, MODE, STAGE, FUSE, MET>;
    // the dynamic shared-memory opt-in is raised once per instantiation and
    // device (and on every prepare pass, which precedes each graph capture)
    static fr_smem_optin optin;
    if (int rc = fr_raise_smem(kern, S::bytes, optin, p->prepare_only)) return rc;
    if (p->prepare_only) return FRGPU_OK;
    FR_CUDA(fr_launch(kern, dim3((a.nx + T::TX - 1) / T::TX, (a.ny + T::TY - 1) / T::TY), dim3(T::TX * NP * T::TY),
                      S::bytes, p->stream, a));
    p->launches += 1;
    return FRGPU_OK;
}

template <class Real, int NP, int MODE, bool MET>
int dispatch_stage(frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    const int flux = p->d.flux == FRGPU_FLUX_HLL ? FLUX_HLL : FLUX_LF;
#define FR_ST(S)                                                                                                   \
    return flux == FLUX_HLL ? launch_t<Real, NP, FLUX_HLL, MODE, S, FUSE_NONE, MET>(p, in, din, out)               \
                            : launch_t<Real, NP, FLUX_LF, MODE, S, FUSE_NONE, MET>(p, in, din, out)
    if constexpr (!MET && std::is_same<Real, float>::value && NP == 4 && MODE == MODE_FP32K) {
        const int fused = stage == 3 ? fr_fused_indicator(p) : FRGPU_IND_NONE;
        if (fused == FRGPU_IND_MLP)
            return flux == FLUX_HLL ? launch_t<Real, NP, FLUX_HLL, MODE, 3, FUSE_LEARNED>(p, in, din, out)
                                    : launch_t<Real, NP, FLUX_LF, MODE, 3, FUSE_LEARNED>(p, in, din, out);
        if (fused == FRGPU_IND_PLAIN)
            return flux == FLUX_HLL ? launch_t<Real, NP, FLUX_HLL, MODE, 3, FUSE_PLAIN>(p, in, din, out)
                                    : launch_t<Real, NP, FLUX_LF, MODE, 3, FUSE_PLAIN>(p, in, din, out);
    }
    switch (stage) {
    case 0: FR_ST(0);
    case 1: FR_ST(1);
    case 2: FR_ST(2);
    case 3: FR_ST(3);
    }
#undef FR_ST
    fr_set_error("euler2d: bad stage");
    return FRGPU_ERR_ARG;
}

template <class Real, int MODE, bool MET = false>
int dispatch_np(frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    switch (p->sp.np) {
    case 2: return dispatch_stage<Real, 2, MODE, MET>(p, stage, in, din, out);
    case 3: return dispatch_stage<Real, 3, MODE, MET>(p, stage, in, din, out);
    case 4: return dispatch_stage<Real, 4, MODE, MET>(p, stage, in, din, out);
    case 5: return dispatch_stage<Real, 5, MODE, MET>(p, stage, in, din, out);
    case 6: return dispatch_stage<Real, 6, MODE, MET>(p, stage, in, din, out);
    }
    fr_set_error("euler2d: polynomial degree must be 1..5");
    return FRGPU_ERR_UNSUPPORTED;
}

} // namespace
