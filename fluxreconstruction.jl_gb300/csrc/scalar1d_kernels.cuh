// scalar1d_kernels.cuh -- fused 1D flux-reconstruction residuals + SSPRK3 stage:
//   * scalar advection / Burgers: frode_advection! (src/Equation/eq_advection.jl:55-77)
//     with advection_dflux! (:103-111), advection_iflux! (:128-137),
//     scalar_rhs! (src/Equation/eq_scalar.jl:1-12), period_advection! (:158-175)
//     and dirichlet_advection! (:153-156);
//   * 1D Euler: frode_euler! (src/Equation/eq_euler.jl:29-73), period_euler!
//     (:80-98), dirichlet_euler! (:75-78);
//   * 1D1V BGK: mol! of example/bgk_wave.jl:69-129;
// plus the stateless interp_face! (src/interpolate.jl:6-10) and
// poly_derivative! (src/derivative.jl:1-10).
#pragma once
#include "fr_stage.cuh"
#include "frgpu_internal.h"

using namespace frk;

namespace {

constexpr int NT1 = 256;

template <class Real, int NP> struct S1DArgs {
    int ne;
    const Real *uin, *din, *un;
    Real *out, *ul;
    const double *dtp;
    const Real *J; // per-element Jacobian (device)
    Real a;
    Real gamma, gm1;
    Real eps_i, eps_p;
    int periodic;
    Ops<Real, NP> ops;
    int *status;
};

__device__ __forceinline__ int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// ---------------------------------------------------------------- scalar
template <class Real, int NP, bool BURGERS>
__device__ __forceinline__ void scalar_traces(const Real *__restrict__ uin, const Real *__restrict__ din, int ne, int i,
                                              Real a, Real J, const Ops<Real, NP> &op, Real (&u)[NP], Real (&f)[NP],
                                              Real &uL, Real &uR, Real &fL, Real &fR) {
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        u[k] = ld_state(uin, din, (size_t)i + (size_t)ne * k);
        const Real fl = BURGERS ? Real(0.5) * u[k] * u[k] : a * u[k];
        f[k] = divR<Real>(fl, J);
    }
    uL = dotw<Real, NP>(u, op.ll);
    uR = dotw<Real, NP>(u, op.lr);
    fL = dotw<Real, NP>(f, op.ll);
    fR = dotw<Real, NP>(f, op.lr);
}

// Scalar Roe-type interface flux of advection_iflux! (eq_advection.jl:130-133):
// au = (fR - fL)/(uR - uL + eps), F = (fR + fL)/2 - |au| (uR - uL)/2, where
// (uL, fL) is the right trace of the left element and (uR, fR) the left
// trace of the right element.
template <class Real>
__device__ __forceinline__ Real roe_scalar(Real uL, Real fL, Real uR, Real fR, Real eps) {
    const Real au = divR<Real>(fR - fL, uR - uL + eps);
    return Real(0.5) * (fR + fL) - Real(0.5) * absR<Real>(au) * (uR - uL);
}

template <class Real, int NP, int MODE, int STAGE, bool BURGERS>
__global__ void __launch_bounds__(NT1) k_scalar1d(const S1DArgs<Real, NP> a) {
    FR_PDL_ENTRY();
    __shared__ Real s_uR[NT1], s_fR[NT1], s_F[NT1 + 1], s_h[4];
    const int t = threadIdx.x;
    const int i0 = blockIdx.x * NT1;
    const int ne = a.ne;
    const int vn = min(NT1, ne - i0);
    const bool valid = t < vn;
    const int i = i0 + t;
    const Ops<Real, NP> &op = a.ops;
    Real u[NP], f[NP], uL = 0, uR = 0, fL = 0, fR = 0;
    if (valid) {
        scalar_traces<Real, NP, BURGERS>(a.uin, a.din, ne, i, a.a, a.J[i], op, u, f, uL, uR, fL, fR);
        s_uR[t] = uR;
        s_fR[t] = fR;
    }
    if (t == 0 || t == 1) {
        // halo: t = 0 -> left neighbour of the block (its right trace);
        //       t = 1 -> right neighbour of the block (its left trace)
        const int n = t == 0 ? wrap(i0 - 1, ne) : wrap(i0 + vn, ne);
        Real hu[NP], hf[NP], a0, a1, b0, b1;
        scalar_traces<Real, NP, BURGERS>(a.uin, a.din, ne, n, a.a, a.J[n], op, hu, hf, a0, a1, b0, b1);
        if (t == 0) { s_h[0] = a1; s_h[1] = b1; }
        else { s_h[2] = a0; s_h[3] = b0; }
    }
    __syncthreads();
    if (valid) {
        const Real ulN = t > 0 ? s_uR[t - 1] : s_h[0];
        const Real flN = t > 0 ? s_fR[t - 1] : s_h[1];
        const Real eps = (i == 0 && a.periodic) ? a.eps_p : a.eps_i;
        s_F[t] = roe_scalar<Real>(ulN, flN, uL, fL, eps);
        if (t == vn - 1) {
            const Real epsr = (i == ne - 1 && a.periodic) ? a.eps_p : a.eps_i;
            s_F[t + 1] = roe_scalar<Real>(uR, fR, s_h[2], s_h[3], epsr);
        }
    }
    __syncthreads();
    if (!valid) return;
    const bool frozen = !a.periodic && (i == 0 || i == ne - 1);
    const Real FL = s_F[t], FR = s_F[t + 1];
    const Real dt = (Real)(*a.dtp);
    int bad = 0;
#pragma unroll
    for (int m = 0; m < NP; ++m) {
        Real du;
        if (frozen) {
            du = Real(0);
        } else {
            const Real r = dotw<Real, NP>(f, op.D[m]);
            du = -fmaR<Real>(FR - fR, op.dgr[m], fmaR<Real>(FL - fL, op.dgl[m], r));
        }
        const size_t idx = (size_t)i + (size_t)ne * m;
        const Real res = stage_update<Real, MODE, STAGE>(du, u[m], dt, idx, a.un, a.uin, a.din, a.out, a.ul);
        if (!isfinite(res)) bad |= ST_NONFINITE;
    }
    if (bad) atomicOr(a.status, bad);
}

// ---------------------------------------------------------------- Euler 1D
template <class Real>
__device__ __forceinline__ void euler1d_flux(const Real (&w)[3], Real gm1, Real (&f)[3], Real &U, Real &p) {
    U = divR<Real>(w[1], w[0]);
    p = gm1 * (w[2] - Real(0.5) * w[1] * U);
    f[0] = w[1];
    f[1] = fmaR<Real>(w[1], U, p);
    f[2] = (w[2] + p) * U;
}

// HLL with Davis wave speeds (Toro ch. 10), for KitBase.flux_hll! at eq_euler.jl:53
template <class Real>
__device__ __forceinline__ void hll1d(const Real (&wL)[3], const Real (&wR)[3], Real gamma, Real gm1, Real (&F)[3]) {
    Real fL[3], fR[3], uL, uR, pL, pR;
    euler1d_flux<Real>(wL, gm1, fL, uL, pL);
    euler1d_flux<Real>(wR, gm1, fR, uR, pR);
    const Real cL = sqrtP<Real>(divR<Real>(gamma * pL, wL[0]));
    const Real cR = sqrtP<Real>(divR<Real>(gamma * pR, wR[0]));
    const Real sl = minR<Real>(uL - cL, uR - cR);
    const Real sr = maxR<Real>(uL + cL, uR + cR);
    if (sl >= Real(0)) {
#pragma unroll
        for (int m = 0; m < 3; ++m) F[m] = fL[m];
    } else if (sr <= Real(0)) {
#pragma unroll
        for (int m = 0; m < 3; ++m) F[m] = fR[m];
    } else {
        const Real factor = recipR<Real>(sr - sl);
#pragma unroll
        for (int m = 0; m < 3; ++m) F[m] = factor * (sr * fL[m] - sl * fR[m] + sl * sr * (wR[m] - wL[m]));
    }
}

template <class Real, int NP>
__device__ __forceinline__ void euler1d_load(const Real *__restrict__ uin, const Real *__restrict__ din, int ne, int i,
                                             Real (&u)[NP][3]) {
#pragma unroll
    for (int m = 0; m < 3; ++m)
#pragma unroll
        for (int k = 0; k < NP; ++k) u[k][m] = ld_state(uin, din, (size_t)i + (size_t)ne * (k + NP * m));
}

template <class Real, int NP>
__device__ __forceinline__ void trace3(const Real (&u)[NP][3], const Real *w, Real (&t)[3]) {
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        Real v[NP];
#pragma unroll
        for (int k = 0; k < NP; ++k) v[k] = u[k][m];
        t[m] = dotw<Real, NP>(v, w);
    }
}

template <class Real, int NP, int MODE, int STAGE>
__global__ void __launch_bounds__(NT1) k_euler1d(const S1DArgs<Real, NP> a) {
    FR_PDL_ENTRY();
    __shared__ Real s_uR[3][NT1], s_F[3][NT1 + 1], s_h[2][3];
    const int t = threadIdx.x;
    const int i0 = blockIdx.x * NT1;
    const int ne = a.ne;
    const int vn = min(NT1, ne - i0);
    const bool valid = t < vn;
    const int i = i0 + t;
    const Ops<Real, NP> &op = a.ops;
    Real u[NP][3], f[NP][3], uLt[3], uRt[3], fLt[3], fRt[3];
    int bad = 0;
    if (valid) {
        euler1d_load<Real, NP>(a.uin, a.din, ne, i, u);
        const Real J = a.J[i];
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            Real fl[3], U, p;
            euler1d_flux<Real>(u[k], a.gm1, fl, U, p);
            if (!(u[k][0] > Real(0)) || !(p > Real(0))) bad |= ST_UNPHYSICAL;
#pragma unroll
            for (int m = 0; m < 3; ++m) f[k][m] = divR<Real>(fl[m], J);
        }
        trace3<Real, NP>(u, op.ll, uLt);
        trace3<Real, NP>(u, op.lr, uRt);
        trace3<Real, NP>(f, op.ll, fLt);
        trace3<Real, NP>(f, op.lr, fRt);
#pragma unroll
        for (int m = 0; m < 3; ++m) s_uR[m][t] = uRt[m];
    }
    if (t == 0 || t == 1) {
        const int n = t == 0 ? wrap(i0 - 1, ne) : wrap(i0 + vn, ne);
        Real hu[NP][3], tr[3];
        euler1d_load<Real, NP>(a.uin, a.din, ne, n, hu);
        trace3<Real, NP>(hu, t == 0 ? op.lr : op.ll, tr);
#pragma unroll
        for (int m = 0; m < 3; ++m) s_h[t][m] = tr[m];
    }
    __syncthreads();
    if (valid) {
        Real wL[3], F[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) wL[m] = t > 0 ? s_uR[m][t - 1] : s_h[0][m];
        hll1d<Real>(wL, uLt, a.gamma, a.gm1, F);
#pragma unroll
        for (int m = 0; m < 3; ++m) s_F[m][t] = F[m];
        if (t == vn - 1) {
            Real wR[3];
#pragma unroll
            for (int m = 0; m < 3; ++m) wR[m] = s_h[1][m];
            hll1d<Real>(uRt, wR, a.gamma, a.gm1, F);
#pragma unroll
            for (int m = 0; m < 3; ++m) s_F[m][t + 1] = F[m];
        }
    }
    __syncthreads();
    if (!valid) return;
    const bool frozen = !a.periodic && (i == 0 || i == ne - 1);
    const Real dt = (Real)(*a.dtp);
    const Real J = a.J[i];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const Real aL = divR<Real>(s_F[m][t], J) - fLt[m];
        const Real aR = divR<Real>(s_F[m][t + 1], J) - fRt[m];
        Real fc[NP];
#pragma unroll
        for (int k = 0; k < NP; ++k) fc[k] = f[k][m];
#pragma unroll
        for (int kk = 0; kk < NP; ++kk) {
            Real du = Real(0);
            if (!frozen) du = -fmaR<Real>(aR, op.dgr[kk], fmaR<Real>(aL, op.dgl[kk], dotw<Real, NP>(fc, op.D[kk])));
            const size_t idx = (size_t)i + (size_t)ne * (kk + NP * m);
            const Real res = stage_update<Real, MODE, STAGE>(du, u[kk][m], dt, idx, a.un, a.uin, a.din, a.out, a.ul);
            if (!isfinite(res)) bad |= ST_NONFINITE;
        }
    }
    if (bad) atomicOr(a.status, bad);
}

// ---------------------------------------------------------------- BGK 1D1V
// Internal layout: u[(i * NP + k) * nvel + v] (velocity fastest), so one CTA
// handles one element with its threads across velocities, reading every
// (element, point) row with coalesced transactions.
constexpr int NTB = 256;

template <class Real, int NP> struct BGKArgs {
    int ne, nvel;
    const Real *uin, *din, *un;
    Real *out, *ul;
    const double *dtp;
    const Real *J;
    const Real *velo, *w;
    Real tau;
    int closure;  // 0: conserve_prim(w, 3); 1: prim = [rho, a_adv, 1]
    double a_adv;
    Ops<Real, NP> ops;
    int *status;
};

// Transport, relaxation and stage update of velocity v of element i (neighbours
// il, ir), given the element's (rho, U, lambda) per solution point.
template <class Real, int NP, int MODE, int STAGE, class Prim>
__device__ __forceinline__ int bgk_velocity(const BGKArgs<Real, NP> &a, int i, int il, int ir, int v,
                                            const Prim &prim, int mfirst = 0, int mcount = NP) {
    const int nv = a.nvel;
    const Ops<Real, NP> &op = a.ops;
    const Real J = a.J[i], JL = a.J[il], JR = a.J[ir];
    const Real dt = (Real)(*a.dtp);
    const Real pi_inv = Real(0.31830988618379067154);
    int bad = 0;
    const Real vel = a.velo[v];
    const bool up = vel > Real(0); // heaviside(v)
    Real u[NP], f[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        u[k] = ld_state(a.uin, a.din, ((size_t)i * NP + k) * nv + v);
        f[k] = divR<Real>(vel * u[k], J);
    }
    const Real fL = dotw<Real, NP>(f, op.ll), fR = dotw<Real, NP>(f, op.lr);
    // upwind face fluxes: from the left neighbour's right trace when v > 0,
    // else from this element's left trace (and likewise on the right face)
    Real Fl, Fr;
    {
        Real g[NP];
        const int nb = up ? il : ir;
        const Real Jn = up ? JL : JR;
#pragma unroll
        for (int k = 0; k < NP; ++k) g[k] = vel * ld_state(a.uin, a.din, ((size_t)nb * NP + k) * nv + v) / Jn;
        if (up) {
            Fl = dotw<Real, NP>(g, op.lr);
            Fr = fR;
        } else {
            Fl = fL;
            Fr = dotw<Real, NP>(g, op.ll);
        }
    }
#pragma unroll
    for (int mm = 0; mm < NP; ++mm) {
        if (mm >= mcount) break;
        const int m = mfirst + mm;
        const Real rho = prim[mm][0], U = prim[mm][1], lam = prim[mm][2];
        const Real dv = vel - U;
        const Real M = rho * sqrtP<Real>(lam * pi_inv) * exp(-lam * dv * dv);
        const Real r = dotw<Real, NP>(f, op.D[m]);
        const Real du = -fmaR<Real>(Fr - fR, op.dgr[m], fmaR<Real>(Fl - fL, op.dgl[m], r)) + (M - u[m]) / a.tau;
        const size_t idx = ((size_t)i * NP + m) * nv + v;
        const Real res = stage_update<Real, MODE, STAGE>(du, u[m], dt, idx, a.un, a.uin, a.din, a.out, a.ul);
        if (!isfinite(res)) bad |= ST_NONFINITE;
    }
    return bad;
}

// (rho, U, lambda) of one solution point from its FP64 moments (rho, m, 2E):
// closure 0: conserve_prim(w, gamma = 3) (1D): lambda = 0.5 rho / (gamma - 1) / (E - m^2 / (2 rho));
// closure 1: prim = [rho, a, 1] (example/advection_kinetic.jl:80-86)
template <class Real, int NP>
__device__ __forceinline__ bool bgk_prim(const BGKArgs<Real, NP> &a, double w0, double w1, double w2, Real (&pr)[3]) {
    w2 *= 0.5;
    const double U = a.closure ? a.a_adv : w1 / w0;
    const double lam = a.closure ? 1.0 : 0.5 * w0 / 2.0 / (w2 - 0.5 * w1 * w1 / w0);
    pr[0] = (Real)w0;
    pr[1] = (Real)U;
    pr[2] = (Real)lam;
    return w0 > 0.0 && lam > 0.0;
}

// Small velocity sets (nvel <= 64): one warp per (element, solution point m),
// the NP warps of an element in one block.  A warp reduces the moments of its
// point m by a fixed butterfly and updates the values of point m only, so that
// each thread's dependent FP64 chain (the Maxwellian's exp, the divisions, the
// stage update) covers one point instead of NP: the form is bound by that chain
// (GB300's FP64 pipe runs at 1/64 of the FP32 rate), not by the FP64 work.  The
// block-per-element form would leave 7 of its 8 warps without velocities at 28
// of them, yet run their FP64 reductions.
template <class Real, int NP, int MODE, int STAGE>
__global__ void __launch_bounds__(32 * NP) k_bgk1d_warp(const BGKArgs<Real, NP> a) {
    FR_PDL_ENTRY();
    const int lane = threadIdx.x & 31, m = threadIdx.x >> 5;
    const int i = blockIdx.x;
    const int ne = a.ne, nv = a.nvel;
    const int il = i == 0 ? ne - 1 : i - 1, ir = i == ne - 1 ? 0 : i + 1;
    double mom[3] = {0.0, 0.0, 0.0};
    for (int v = lane; v < nv; v += 32) {
        const double vel = (double)a.velo[v], wv = (double)a.w[v];
        const double x = (double)ld_state(a.uin, a.din, ((size_t)i * NP + m) * nv + v);
        mom[0] += wv * x;
        mom[1] += wv * vel * x;
        mom[2] += wv * (vel * vel) * x;
    }
#pragma unroll
    for (int q = 0; q < 3; ++q)
        for (int off = 16; off > 0; off >>= 1) mom[q] += __shfl_xor_sync(0xffffffffu, mom[q], off);
    Real prim[1][3];
    if (!bgk_prim<Real, NP>(a, mom[0], mom[1], mom[2], prim[0]) && lane == 0) atomicOr(a.status, ST_UNPHYSICAL);
    int bad = 0;
    for (int v = lane; v < nv; v += 32) bad |= bgk_velocity<Real, NP, MODE, STAGE>(a, i, il, ir, v, prim, m, 1);
    if (bad) atomicOr(a.status, bad);
}

template <class Real, int NP, int MODE, int STAGE>
__global__ void __launch_bounds__(NTB) k_bgk1d(const BGKArgs<Real, NP> a) {
    FR_PDL_ENTRY();
    const int i = blockIdx.x;
    const int ne = a.ne, nv = a.nvel;
    const int il = i == 0 ? ne - 1 : i - 1, ir = i == ne - 1 ? 0 : i + 1;
    __shared__ double s_red[3 * NP][NTB / 32];
    __shared__ Real s_prim[NP][3];
    // moments: sum_v w_v [1, v, v^2/2] u(v) per solution point (FP64 accumulation)
    double mom[NP][3];
#pragma unroll
    for (int k = 0; k < NP; ++k) mom[k][0] = mom[k][1] = mom[k][2] = 0.0;
    for (int v = threadIdx.x; v < nv; v += NTB) {
        const double vel = (double)a.velo[v], wv = (double)a.w[v];
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            const double x = (double)ld_state(a.uin, a.din, ((size_t)i * NP + k) * nv + v);
            mom[k][0] += wv * x;
            mom[k][1] += wv * vel * x;
            mom[k][2] += wv * (vel * vel) * x;
        }
    }
#pragma unroll
    for (int k = 0; k < NP; ++k)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            double x = mom[k][q];
            for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
            if ((threadIdx.x & 31) == 0) s_red[k * 3 + q][threadIdx.x >> 5] = x;
        }
    __syncthreads();
    if (threadIdx.x < NP) {
        const int k = threadIdx.x;
        double w0 = 0, w1 = 0, w2 = 0;
        for (int wq = 0; wq < NTB / 32; ++wq) {
            w0 += s_red[k * 3 + 0][wq];
            w1 += s_red[k * 3 + 1][wq];
            w2 += s_red[k * 3 + 2][wq];
        }
        if (!bgk_prim<Real, NP>(a, w0, w1, w2, s_prim[k])) atomicOr(a.status, ST_UNPHYSICAL);
    }
    __syncthreads();
    int bad = 0;
    for (int v = threadIdx.x; v < nv; v += NTB) bad |= bgk_velocity<Real, NP, MODE, STAGE>(a, i, il, ir, v, s_prim);
    if (bad) atomicOr(a.status, bad);
}

// ---------------------------------------------------------------- launchers
template <class Real, int NP> Ops<Real, NP> make_ops1(const frgpu_space &s) {
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

template <class Real, int NP>
S1DArgs<Real, NP> make_args1(frgpu_problem *p, const void *in, const void *din, void *out) {
    S1DArgs<Real, NP> a;
    a.ne = p->sp.nx;
    a.uin = (const Real *)in;
    a.din = (const Real *)din;
    a.un = (const Real *)p->s0;
    a.out = (Real *)out;
    a.ul = (Real *)p->s3;
    a.dtp = p->d_dt;
    a.J = (const Real *)p->d_J;
    a.a = (Real)p->d.a;
    a.gamma = (Real)p->d.gamma;
    a.gm1 = (Real)(p->d.gamma - 1.0);
    a.eps_i = (Real)p->d.eps_interior;
    a.eps_p = (Real)p->d.eps_periodic;
    a.periodic = p->d.bc[0] == FRGPU_BC_PERIODIC;
    a.ops = make_ops1<Real, NP>(p->sp);
    a.status = p->d_status;
    return a;
}

template <class Real, int NP, int MODE, int STAGE>
int launch_scalar_t(frgpu_problem *p, const void *in, const void *din, void *out) {
    if (p->prepare_only) return FRGPU_OK;
    auto a = make_args1<Real, NP>(p, in, din, out);
    const int grid = (a.ne + NT1 - 1) / NT1;
    if (p->d.equation == FRGPU_BURGERS)
        FR_CUDA(fr_launch(k_scalar1d<Real, NP, MODE, STAGE, true>, grid, NT1, 0, p->stream, a));
    else
        FR_CUDA(fr_launch(k_scalar1d<Real, NP, MODE, STAGE, false>, grid, NT1, 0, p->stream, a));
    FR_CUDA(cudaGetLastError());
    p->launches += 1;
    return FRGPU_OK;
}

template <class Real, int NP, int MODE, int STAGE>
int launch_euler1d_t(frgpu_problem *p, const void *in, const void *din, void *out) {
    if (p->prepare_only) return FRGPU_OK;
    auto a = make_args1<Real, NP>(p, in, din, out);
    const int grid = (a.ne + NT1 - 1) / NT1;
    FR_CUDA(fr_launch(k_euler1d<Real, NP, MODE, STAGE>, grid, NT1, 0, p->stream, a));
    FR_CUDA(cudaGetLastError());
    p->launches += 1;
    return FRGPU_OK;
}

template <class Real, int NP, int MODE, int STAGE>
int launch_bgk_t(frgpu_problem *p, const void *in, const void *din, void *out) {
    if (p->prepare_only) return FRGPU_OK;
    BGKArgs<Real, NP> a;
    a.ne = p->sp.nx;
    a.nvel = p->d.nvel;
    a.uin = (const Real *)in;
    a.din = (const Real *)din;
    a.un = (const Real *)p->s0;
    a.out = (Real *)out;
    a.ul = (Real *)p->s3;
    a.dtp = p->d_dt;
    a.J = (const Real *)p->d_J;
    a.velo = (const Real *)p->d_velo;
    a.w = (const Real *)p->d_w;
    a.tau = (Real)p->d.tau;
    a.closure = p->bgk_closure;
    a.a_adv = p->d.a;
    a.ops = make_ops1<Real, NP>(p->sp);
    a.status = p->d_status;
    if (a.nvel <= 64)
        FR_CUDA(fr_launch(k_bgk1d_warp<Real, NP, MODE, STAGE>, a.ne, 32 * NP, 0, p->stream, a));
    else
        FR_CUDA(fr_launch_opt(false, k_bgk1d<Real, NP, MODE, STAGE>, a.ne, NTB, 0, p->stream, a));
    FR_CUDA(cudaGetLastError());
    p->launches += 1;
    return FRGPU_OK;
}

enum { KIND_SCALAR, KIND_EULER, KIND_BGK };

template <class Real, int NP, int MODE>
int dispatch1_stage(int kind, frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
#define FR_K(S)                                                                                                    \
    return kind == KIND_SCALAR  ? launch_scalar_t<Real, NP, MODE, S>(p, in, din, out)                              \
           : kind == KIND_EULER ? launch_euler1d_t<Real, NP, MODE, S>(p, in, din, out)                             \
                                : launch_bgk_t<Real, NP, MODE, S>(p, in, din, out)
    switch (stage) {
    case 0: FR_K(0);
    case 1: FR_K(1);
    case 2: FR_K(2);
    case 3: FR_K(3);
    }
#undef FR_K
    fr_set_error("1D residual: bad stage");
    return FRGPU_ERR_ARG;
}

template <class Real, int MODE>
int dispatch1_np(int kind, frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    switch (p->sp.np) {
    case 2: return dispatch1_stage<Real, 2, MODE>(kind, p, stage, in, din, out);
    case 3: return dispatch1_stage<Real, 3, MODE>(kind, p, stage, in, din, out);
    case 4: return dispatch1_stage<Real, 4, MODE>(kind, p, stage, in, din, out);
    case 5: return dispatch1_stage<Real, 5, MODE>(kind, p, stage, in, din, out);
    case 6: return dispatch1_stage<Real, 6, MODE>(kind, p, stage, in, din, out);
    }
    fr_set_error("1D residual: polynomial degree must be 1..5");
    return FRGPU_ERR_UNSUPPORTED;
}

} // namespace
