// central2d.cu -- the 2D Euler residual of dev/curve_euler.jl's active dudt!
// (FRGPU_FLUX_CENTRAL): per-point inverse Jacobian, interaction flux
// F* = 0.5 (f_L + f_R) - c (u_R - u_L) on the face traces of the transformed
// flux and of u, corrections with the traces unscaled, and the elements along
// a Dirichlet side left at du = 0.
//
// Three passes over the device layout u[((k + NP l) ne + e) 4 + m]:
//   k_c2_flux    one thread per (element, point): f = a11 F + a12 G,
//                g = a21 F + a22 G (fma(G, a12, F a11) as the oracle forms it);
//   k_c2_traces  one thread per (element, face point q): the traces of u and of
//                the face-normal component of the transformed flux on the four
//                faces (0 bottom, 1 right, 2 top, 3 left: the script's faces
//                1..4), each an ascending dotw chain with ll or lr;
//   k_c2_rhs     one thread per (element, point): the two line derivatives,
//                the four interaction fluxes from the element's own traces
//                and its neighbours' (periodic wrap), and the correction
//                combine of the 2D residual, written as du.
// Arithmetic follows the oracle's rhs_euler2d operation for operation (this
// file is built without multiply-add contraction), so FP64 is bit-identical.
#include "fr_common.cuh"
#include "frgpu_internal.h"

namespace {

using frk::dotw;
using frk::euler2d_flux;
using frk::fmaR;
using frk::ldg4;
using frk::v4_fma;
using frk::v4_mul;

template <class Real, int NP> struct C2Ops {
    Real ll[NP], lr[NP], dgl[NP], dgr[NP];
    Real D[NP][NP]; // D[m][k] = l_k'(r_m)
};

// transformed flux at every point: fv[((c * NP * NP + q) * ne + e) * 4 + m], c = 0 (x), 1 (y)
template <class Real, int NP>
__global__ void __launch_bounds__(256) k_c2_flux(const Real *__restrict__ u, const Real *__restrict__ met, int ne,
                                                 Real gm1, Real *__restrict__ fv, int *status) {
    FR_PDL_ENTRY();
    const long n = (long)ne * NP * NP;
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const long at = t * 4; // t = q * ne + e
    Real w[4], mt[4], F[4], G[4], f[4], g[4];
    ldg4(u + at, w);
    ldg4(met + at, mt);
    int bad = 0;
    euler2d_flux<Real>(w, gm1, Real(1), Real(1), F, G, bad);
    v4_mul<Real>(F, mt[0], f);
    v4_fma<Real>(G, mt[1], f, f);
    v4_mul<Real>(F, mt[2], g);
    v4_fma<Real>(G, mt[3], g, g);
    for (int m = 0; m < 4; ++m) {
        fv[at + m] = f[m];
        fv[n * 4 + at + m] = g[m];
    }
    if (bad) atomicOr(status, frk::ST_UNPHYSICAL);
}

// traces: tu[((face * NP + q) * ne + e) * 4 + m], tf likewise
template <class Real, int NP>
__global__ void __launch_bounds__(256) k_c2_traces(const Real *__restrict__ u, const Real *__restrict__ fv, int ne,
                                                   const C2Ops<Real, NP> op, Real *__restrict__ tu,
                                                   Real *__restrict__ tf) {
    FR_PDL_ENTRY();
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= (long)ne * NP) return;
    const int q = (int)(t / ne);
    const long e = t - (long)q * ne;
    const long pl = (long)ne * 4, gy = (long)NP * NP * ne * 4; // point stride, y-component offset
    for (int m = 0; m < 4; ++m) {
        Real us[NP], ur[NP], gs[NP], fr[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            const long a_s = (q + (long)NP * p) * pl + e * 4 + m; // point (k = q, l = p): along s
            const long a_r = (p + (long)NP * q) * pl + e * 4 + m; // point (k = p, l = q): along r
            us[p] = u[a_s];
            ur[p] = u[a_r];
            gs[p] = fv[gy + a_s];
            fr[p] = fv[a_r];
        }
        const long o = e * 4 + m, fs = (long)NP * ne * 4;
        tu[0 * fs + q * pl + o] = dotw<Real, NP>(us, op.ll);
        tu[1 * fs + q * pl + o] = dotw<Real, NP>(ur, op.lr);
        tu[2 * fs + q * pl + o] = dotw<Real, NP>(us, op.lr);
        tu[3 * fs + q * pl + o] = dotw<Real, NP>(ur, op.ll);
        tf[0 * fs + q * pl + o] = dotw<Real, NP>(gs, op.ll);
        tf[1 * fs + q * pl + o] = dotw<Real, NP>(fr, op.lr);
        tf[2 * fs + q * pl + o] = dotw<Real, NP>(gs, op.lr);
        tf[3 * fs + q * pl + o] = dotw<Real, NP>(fr, op.ll);
    }
}

template <class Real, int NP> struct C2Args {
    int nx, ny;
    int bc[4];
    Real c;
    const Real *fv, *tu, *tf;
    Real *out;
    C2Ops<Real, NP> op;
};

template <class Real, int NP>
__global__ void __launch_bounds__(256) k_c2_rhs(const C2Args<Real, NP> a) {
    FR_PDL_ENTRY();
    const int nx = a.nx, ny = a.ny;
    const long ne = (long)nx * ny;
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= ne * NP * NP) return;
    const int pq = (int)(t / ne);
    const long e = t - (long)pq * ne;
    const int k = pq % NP, l = pq / NP;
    const int i = (int)(e % nx), j = (int)(e / nx);
    const long pl = ne * 4, gy = (long)NP * NP * ne * 4, fs = (long)NP * ne * 4;
    Real *out = a.out + (long)pq * pl + e * 4;
    if ((i == 0 && a.bc[0] == FRGPU_BC_DIRICHLET) || (i == nx - 1 && a.bc[1] == FRGPU_BC_DIRICHLET) ||
        (j == 0 && a.bc[2] == FRGPU_BC_DIRICHLET) || (j == ny - 1 && a.bc[3] == FRGPU_BC_DIRICHLET)) {
        for (int m = 0; m < 4; ++m) out[m] = Real(0);
        return;
    }
    // neighbours (an element along a Dirichlet side never gets here, so the
    // wrap is only taken across periodic sides)
    const long eL = (i == 0 ? nx - 1 : i - 1) + (long)nx * j, eR = (i == nx - 1 ? 0 : i + 1) + (long)nx * j;
    const long eB = i + (long)nx * (j == 0 ? ny - 1 : j - 1), eT = i + (long)nx * (j == ny - 1 ? 0 : j + 1);
    const Real c = a.c;
    for (int m = 0; m < 4; ++m) {
        Real fx[NP], gy_[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            fx[p] = a.fv[(p + (long)NP * l) * pl + e * 4 + m];
            gy_[p] = a.fv[gy + (k + (long)NP * p) * pl + e * 4 + m];
        }
        const Real r1 = dotw<Real, NP>(fx, a.op.D[k]);
        const Real r2 = dotw<Real, NP>(gy_, a.op.D[l]);
        const auto TU = [&](int f, int q, long el) { return a.tu[f * fs + q * pl + el * 4 + m]; };
        const auto TF = [&](int f, int q, long el) { return a.tf[f * fs + q * pl + el * 4 + m]; };
        // x faces at s-point l: left = (eL face 1 | e face 3), right = (e face 1 | eR face 3)
        const Real fxl = Real(0.5) * (TF(1, l, eL) + TF(3, l, e)) - c * (TU(3, l, e) - TU(1, l, eL));
        const Real fxr = Real(0.5) * (TF(1, l, e) + TF(3, l, eR)) - c * (TU(3, l, eR) - TU(1, l, e));
        // y faces at r-point k: bottom = (eB face 2 | e face 0), top = (e face 2 | eT face 0)
        const Real fyb = Real(0.5) * (TF(2, k, eB) + TF(0, k, e)) - c * (TU(0, k, e) - TU(2, k, eB));
        const Real fyt = Real(0.5) * (TF(2, k, e) + TF(0, k, eT)) - c * (TU(0, k, eT) - TU(2, k, e));
        const Real aL = fxl - TF(3, l, e), aR = fxr - TF(1, l, e);
        const Real bB = fyb - TF(0, k, e), bT = fyt - TF(2, k, e);
        const Real cx = fmaR<Real>(aR, a.op.dgr[k], fmaR<Real>(aL, a.op.dgl[k], r1));
        out[m] = -fmaR<Real>(bT, a.op.dgr[l], fmaR<Real>(bB, a.op.dgl[l], cx + r2));
    }
}

template <class Real, int NP> int launch_c2(frgpu_problem *p, const void *in, void *out) {
    const int nx = p->sp.nx, ny = p->sp.ny;
    const long ne = (long)nx * ny, n = ne * NP * NP;
    const size_t need = (size_t)(2 * n * 4 + 2 * 4 * NP * ne * 4); // fv, tu, tf
    if (p->c2_cap < need) {
        FR_CUDA(cudaStreamSynchronize(p->stream));
        if (p->d_c2) cudaFree(p->d_c2);
        p->d_c2 = nullptr;
        p->c2_cap = 0;
        FR_CUDA(cudaMalloc(&p->d_c2, need * p->esize));
        p->c2_cap = need;
    }
    if (p->prepare_only) return FRGPU_OK;
    Real *fv = (Real *)p->d_c2, *tu = fv + 2 * n * 4, *tf = tu + 4 * NP * ne * 4;
    C2Ops<Real, NP> op;
    for (int q = 0; q < NP; ++q) {
        op.ll[q] = (Real)p->sp.ll[q];
        op.lr[q] = (Real)p->sp.lr[q];
        op.dgl[q] = (Real)p->sp.dhl[q];
        op.dgr[q] = (Real)p->sp.dhr[q];
        for (int r = 0; r < NP; ++r) op.D[q][r] = (Real)p->sp.dl[q + NP * r];
    }
    FR_CUDA(fr_launch(k_c2_flux<Real, NP>, (unsigned)((n + 255) / 256), 256, 0, p->stream,
        (const Real *)in, (const Real *)p->d_met, (int)ne, (Real)(p->d.gamma - 1.0), fv, p->d_status));
    FR_CUDA(cudaGetLastError());
    FR_CUDA(fr_launch(k_c2_traces<Real, NP>, (unsigned)((ne * NP + 255) / 256), 256, 0, p->stream, (const Real *)in, fv, (int)ne, op,
                                                                                     tu, tf));
    FR_CUDA(cudaGetLastError());
    C2Args<Real, NP> a;
    a.nx = nx;
    a.ny = ny;
    for (int s = 0; s < 4; ++s) a.bc[s] = p->d.bc[s];
    a.c = (Real)p->flux_c;
    a.fv = fv;
    a.tu = tu;
    a.tf = tf;
    a.out = (Real *)out;
    a.op = op;
    FR_CUDA(fr_launch(k_c2_rhs<Real, NP>, (unsigned)((n + 255) / 256), 256, 0, p->stream, a));
    FR_CUDA(cudaGetLastError());
    p->launches += 3;
    return FRGPU_OK;
}

template <class Real> int launch_c2_np(frgpu_problem *p, const void *in, void *out) {
    switch (p->sp.np) {
    case 2: return launch_c2<Real, 2>(p, in, out);
    case 3: return launch_c2<Real, 3>(p, in, out);
    case 4: return launch_c2<Real, 4>(p, in, out);
    case 5: return launch_c2<Real, 5>(p, in, out);
    case 6: return launch_c2<Real, 6>(p, in, out);
    }
    fr_set_error("central flux: polynomial degree must be 1..5");
    return FRGPU_ERR_ARG;
}

} // namespace

// Residual (stage 0) of a FRGPU_FLUX_CENTRAL problem.
int fr_launch_central2d(frgpu_problem *p, int stage, const void *in, void *out) {
    if (stage != 0) {
        fr_set_error("central flux (dev/curve_euler.jl): residual evaluations only; step with frgpu_step_erk "
                     "or frgpu_step_rock");
        return FRGPU_ERR_UNSUPPORTED;
    }
    if (!p->d_met || p->d_nfx) {
        fr_set_error("central flux: needs a per-point metric without face normals (frgpu_problem_set_metric)");
        return FRGPU_ERR_ARG;
    }
    return p->d.precision == FRGPU_FP64 ? launch_c2_np<double>(p, in, out) : launch_c2_np<float>(p, in, out);
}
