// ensemble_kernels.cuh -- persistent kernel advancing a batch of 1D Burgers
// instances of uneven size (ne_i elements) and degree (deg_i = 1..5) to t_end.
//
// Each instance runs the scalar residual of frode_advection!
// (src/Equation/eq_advection.jl:55-77, the Roe flux of :128-137 and the
// periodic face of :158-175) with the Burgers flux u^2/2, SSPRK3 steps of its
// own CFL time step (the last one shortened to land on t_end), and optionally
// the modal-decay indicator + :l2 filter of example/euler_highlevel.jl:37-52
// after every step.  One launch does everything: the CTAs of a persistent grid
// first take large instances from a queue (the whole CTA works on one
// instance), then each warp takes small instances from a second queue.  Which
// queue an instance joins is the tile-shape decision of the autotuner.
//
// The arithmetic is the same as k_scalar1d (fixed FMA order), so the FP64
// instantiation, compiled without implicit contraction, reproduces the oracle
// bit for bit.
//
// With a network bound (frgpu_ensemble_set_mlp) the post-step indicator is the
// learned one: per element, the modal energies feed the 32 -> 64 -> 64 -> 1
// perceptron (mma.sync BF16, one warp per 16 elements, weights in shared
// memory); the plain modal-decay test still runs on every element, decides
// where the network's probability is within `band` of the threshold, and
// counts the network's misfires.
#pragma once
#include "fr_stage.cuh"
#include "frgpu_internal.h"
#include "mlp_device.cuh"

namespace {

using namespace frk;

constexpr int ENS_THREADS = 256;
constexpr int ENS_WARPS = ENS_THREADS / 32;
constexpr int ENS_MAX_NE_CTA = 2048;  // largest instance a CTA handles
constexpr int ENS_MAX_NE_WARP = 512;  // largest instance a warp handles

// Per-degree operators (np = deg + 1 <= 6), filled by the host.
template <class Real> struct EnsOps {
    Real ll[5][6], lr[5][6], dgl[5][6], dgr[5][6], D[5][6][6], V[5][6][6], iV[5][6][6];
    double expfac[5]; // exp(0.875 deg) of the filter strength, evaluated on the host
};

struct EnsInstance {
    long off;    // offset of the instance's state in the flat arrays
    int ne, np;  // elements, points per element
    double dx;   // element size
};

template <class Real> struct EnsArgs {
    const EnsInstance *inst;
    const int *queue_cta, *queue_warp; // instance ids, largest first
    int n_cta, n_warp;
    int *counters;                     // [0] CTA queue head, [1] warp queue head
    Real *u, *s1, *s2;                 // state, stage buffers (FP64: states; FP32: states too)
    const EnsOps<Real> *ops;
    double t_end, cfl;                 // dt_i = cfl * dx_i / ((2 deg_i + 1) max|u_i|)
    int filter;
    double *dt_out;                    // per instance dt used (diagnostics)
    int *steps_out;                    // per instance number of steps
    int *failed;                       // per instance: 0, or the step (1-based) whose state was non-finite
    int *status;
    frmlp::MLPDev mlp;                 // P == nullptr: plain indicator
    float thr, band;                   // learned decision threshold, fallback band
    unsigned long long *istats;        // [troubled, misfires, fallbacks, judged] (learned)
};

// Shared memory of the learned indicator, after the trace scratch:
// W1, W2 (bf16), b1 b2 w3 b3 (fp32, padded), per warp a 16 x 32 bf16 feature
// tile and 16 probabilities.
constexpr int ENS_MLP_SB = ((3 * frmlp::NH + 1) * 4 + 15) / 16 * 16;
constexpr size_t ENS_MLP_SMEM = 2 * frmlp::NH * frmlp::NIN + 2 * frmlp::NH * frmlp::NH + ENS_MLP_SB +
                                ENS_WARPS * (2 * 16 * frmlp::NIN + 4 * 16);

struct EnsLearn {
    frmlp::MLPView view;
    __nv_bfloat16 *xs; // this warp's feature tile
    float *prob;       // this warp's probabilities
    float thr, band;
    bool on;
};

// Does any thread of the worker group (CTA or warp) hold p?  Also a barrier.
template <int G> __device__ __forceinline__ bool group_any(bool p) {
    if (G == 32) return __any_sync(0xffffffffu, p);
    return __syncthreads_or(p) != 0;
}

// Synchronisation of a worker group: the CTA (256 threads) or one warp.
template <int G> __device__ __forceinline__ void group_sync() {
    if (G == 32)
        __syncwarp();
    else
        __syncthreads();
}

template <class Real, int NP, int G>
__device__ __forceinline__ void ens_traces(const Real *__restrict__ u, int ne, int i, Real J,
                                           const EnsOps<Real> &op, Real &uL, Real &uR, Real &fL, Real &fR,
                                           Real (&uv)[NP], Real (&fv)[NP]) {
    const int d = NP - 2;
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        uv[k] = u[(size_t)i + (size_t)ne * k];
        // same expression as k_scalar1d: fl / J with fl = 0.5 u u
        fv[k] = divR<Real>(Real(0.5) * uv[k] * uv[k], J);
    }
    uL = dotw<Real, NP>(uv, op.ll[d]);
    uR = dotw<Real, NP>(uv, op.lr[d]);
    fL = dotw<Real, NP>(fv, op.ll[d]);
    fR = dotw<Real, NP>(fv, op.lr[d]);
}

template <class Real>
__device__ __forceinline__ Real ens_roe(Real uL, Real fL, Real uR, Real fR, Real eps) {
    const Real au = divR<Real>(fR - fL, uR - uL + eps);
    return Real(0.5) * (fR + fL) - Real(0.5) * absR<Real>(au) * (uR - uL);
}

// One residual + stage pass over an instance by a group of G threads (rank r).
// s_t: shared scratch of 4 * ne values (right traces of u and f, left traces of u and f).
template <class Real, int NP, int G, int STAGE>
__device__ void ens_stage(const Real *__restrict__ uin, const Real *__restrict__ un, Real *__restrict__ out, int ne,
                          Real J, Real dt, const EnsOps<Real> &op, Real *s_t, int r, int &bad) {
    const int d = NP - 2;
    Real *s_uR = s_t, *s_fR = s_t + ne, *s_uL = s_t + 2 * ne, *s_fL = s_t + 3 * ne;
    for (int i = r; i < ne; i += G) {
        Real uv[NP], fv[NP], uL, uR, fL, fR;
        ens_traces<Real, NP, G>(uin, ne, i, J, op, uL, uR, fL, fR, uv, fv);
        s_uR[i] = uR;
        s_fR[i] = fR;
        s_uL[i] = uL;
        s_fL[i] = fL;
    }
    group_sync<G>();
    const Real eps_i = Real(1e-8), eps_p = Real(1e-6);
    Real chk = Real(0);
    for (int i = r; i < ne; i += G) {
        const int il = i == 0 ? ne - 1 : i - 1, ir = i == ne - 1 ? 0 : i + 1;
        const Real uL = s_uL[i], fL = s_fL[i], uR = s_uR[i], fR = s_fR[i];
        const Real FL = ens_roe<Real>(s_uR[il], s_fR[il], uL, fL, i == 0 ? eps_p : eps_i);
        const Real FR = ens_roe<Real>(uR, fR, s_uL[ir], s_fL[ir], i == ne - 1 ? eps_p : eps_i);
        Real uv[NP], fv[NP];
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            uv[k] = uin[(size_t)i + (size_t)ne * k];
            fv[k] = divR<Real>(Real(0.5) * uv[k] * uv[k], J);
        }
#pragma unroll
        for (int m = 0; m < NP; ++m) {
            const Real rr = dotw<Real, NP>(fv, op.D[d][m]);
            const Real du = -fmaR<Real>(FR - fR, op.dgr[d][m], fmaR<Real>(FL - fL, op.dgl[d][m], rr));
            const size_t idx = (size_t)i + (size_t)ne * m;
            Real res;
            if (STAGE == 1)
                res = fmaR<Real>(dt, du, uv[m]);
            else if (STAGE == 2)
                res = fmaR<Real>(dt, du, fmaR<Real>(Real(3), un[idx], uv[m])) * Real(0.25);
            else
                res = fmaR<Real>(Real(2) * dt, du, fmaR<Real>(Real(2), uv[m], un[idx])) * Real(1.0 / 3.0);
            out[idx] = res;
            chk += res;
        }
    }
    if (!isfinite(chk)) bad |= ST_NONFINITE;
    group_sync<G>();
}

// Features of one element for the 1D learned indicator (row of 32):
//   [0, np): clamp(log10(u_hat_q^2 / sum u_hat^2 + 1e-16), -16, 0) / 8 + 1
//   8 + deg - 1: 1 (degree one-hot, slots 8..12)
//   16: clamp(log10(sum u_hat^2 + 1e-30) + 6, -8, 8) / 8 (energy against the
//       1e-6 floor of the plain test); all other slots 0.
template <class Real, int NP>
__device__ __forceinline__ void ens_feature_row(const Real (&h)[NP], Real tot, __nv_bfloat16 *row) {
    const float ft = (float)tot, it = ft > 0.f ? 1.0f / ft : 0.f;
#pragma unroll
    for (int q = 0; q < frmlp::NIN; ++q) {
        float x = 0.f;
        if (q < NP) {
            const float hq = (float)h[q];
            x = fminf(fmaxf(log10f(hq * hq * it + 1e-16f), -16.f), 0.f) * 0.125f + 1.0f;
        } else if (q == 8 + NP - 2) {
            x = 1.f;
        } else if (q == 16) {
            x = fminf(fmaxf(log10f(ft + 1e-30f) + 6.f, -8.f), 8.f) * 0.125f;
        }
        row[q] = __float2bfloat16_rn(x);
    }
}

// Modal coefficients, energy and plain modal-decay decision of element i
// (example/euler_highlevel.jl:37-52, the same arithmetic as ens_filter); below is
// set when Se lies below S0 - kappa, where the test's sigma is exactly 1 (smooth).
template <class Real, int NP>
__device__ __forceinline__ bool ens_modes(const Real *__restrict__ u, int ne, int i, const EnsOps<Real> &op,
                                          Real (&h)[NP], Real &tot, bool &below) {
    const int d = NP - 2;
    const int deg = NP - 1;
    const double S0 = -3.0 * log10((double)deg), kappa = 4.0;
    Real x[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) x[q] = u[(size_t)i + (size_t)ne * q];
    tot = Real(0);
#pragma unroll
    for (int a = 0; a < NP; ++a) {
        Real s = op.iV[d][a][0] * x[0];
#pragma unroll
        for (int b = 1; b < NP; ++b) s = fmaR<Real>(op.iV[d][a][b], x[b], s);
        h[a] = s;
        tot = fmaR<Real>(s, s, tot);
    }
    const double su = (double)(h[NP - 1] * h[NP - 1]) / ((double)tot + 1e-6);
    const double Se = log10(su);
    double sigma;
    below = Se < S0 - kappa;
    if (below)
        sigma = 1.0;
    else if (S0 - kappa <= Se && Se < S0 + kappa)
        sigma = 0.5 * (1.0 - sin(0.5 * 3.14159265358979323846 * (Se - S0) / kappa));
    else
        sigma = 0.0;
    return sigma < 0.99;
}

template <class Real, int NP>
__device__ __forceinline__ bool ens_modes(const Real *__restrict__ u, int ne, int i, const EnsOps<Real> &op,
                                          Real (&h)[NP], Real &tot) {
    bool below;
    return ens_modes<Real, NP>(u, ne, i, op, h, tot, below);
}

// :l2 filter of one element's modes h back into u (as ens_filter).
template <class Real, int NP>
__device__ __forceinline__ void ens_filter_elem(Real *__restrict__ u, int ne, int i, double lam,
                                                const EnsOps<Real> &op, Real (&h)[NP]) {
    const int d = NP - 2;
#pragma unroll
    for (int a = 0; a < NP; ++a) h[a] = h[a] / (Real(1) + Real(lam) * Real((double)((a + 1) * (a + 1) * a * a)));
#pragma unroll
    for (int a = 0; a < NP; ++a) {
        Real s = op.V[d][a][0] * h[0];
#pragma unroll
        for (int b = 1; b < NP; ++b) s = fmaR<Real>(op.V[d][a][b], h[b], s);
        u[(size_t)i + (size_t)ne * a] = s;
    }
}

// Modal-decay indicator + :l2 filter of example/euler_highlevel.jl:37-52 on one instance.
template <class Real, int NP, int G>
__device__ void ens_filter(Real *__restrict__ u, int ne, double lam, const EnsOps<Real> &op, int r) {
    for (int i = r; i < ne; i += G) {
        Real h[NP], tot;
        if (ens_modes<Real, NP>(u, ne, i, op, h, tot)) ens_filter_elem<Real, NP>(u, ne, i, lam, op, h);
    }
    group_sync<G>();
}

// Learned indicator + :l2 filter on one instance: each warp of the group takes
// 32 elements at a time (one per lane) and runs the network on each half of 16
// that holds an element outside the plain test's sigma = 1 region. Elements in
// that region are smooth without the network (they count as network decisions
// agreeing with the plain test). The network is row-independent, so every
// element gets the same probability whatever else shares its half.
template <class Real, int NP, int G>
__device__ void ens_filter_learned(Real *__restrict__ u, int ne, double lam, const EnsOps<Real> &op, int r,
                                   const EnsLearn &L, unsigned long long (&cnt)[4]) {
    const int lane = r & 31;
    constexpr int NW = G / 32;
    for (int tile = r >> 5; tile * 32 < ne; tile += NW) {
        const int i = tile * 32 + lane;
        const bool mine = i < ne;
        Real h[NP], tot = Real(0);
        bool plain = false, below = true;
        if (mine) plain = ens_modes<Real, NP>(u, ne, i, op, h, tot, below);
        const bool cand = mine && !below;
        const unsigned cm = __ballot_sync(0xffffffffu, cand);
        float pm = 0.f;
#pragma unroll 1
        for (int half = 0; half < 2; ++half) {
            if (!((cm >> (16 * half)) & 0xffffu)) continue; // warp-uniform
            const bool row = (lane >> 4) == half;
            if (row && mine) {
                ens_feature_row<Real, NP>(h, tot, L.xs + (lane & 15) * frmlp::NIN);
            } else if (row) {
#pragma unroll
                for (int q = 0; q < frmlp::NIN; ++q) L.xs[(lane & 15) * frmlp::NIN + q] = __float2bfloat16_rn(0.f);
            }
            __syncwarp();
            frmlp::Fwd f;
            frmlp::mlp_forward_tile(L.view, L.xs, f);
            if ((lane & 3) == 0) {
                L.prob[lane >> 2] = frmlp::sigmoidf_(f.logit_g);
                L.prob[(lane >> 2) + 8] = frmlp::sigmoidf_(f.logit_g8);
            }
            __syncwarp();
            if (row && cand) pm = L.prob[lane & 15];
            __syncwarp(); // the other half reuses the feature and probability tiles
        }
        if (mine) {
            const bool fb = fabsf(pm - L.thr) < L.band, net = pm > L.thr;
            const bool bad = fb ? plain : net;
            cnt[0] += bad;
            cnt[1] += net != plain;
            cnt[2] += fb;
            cnt[3] += 1;
            if (bad) ens_filter_elem<Real, NP>(u, ne, i, lam, op, h);
        }
        __syncwarp();
    }
    group_sync<G>();
}

// Run one instance to t_end with a group of G threads.
template <class Real, int NP, int G, bool LEARNED>
__device__ void ens_run(const EnsArgs<Real> &a, int id, Real *s_t, double *s_red, int r, int &bad,
                        const EnsLearn &L, unsigned long long (&cnt)[4]) {
    const EnsInstance in = a.inst[id];
    Real *u = a.u + in.off, *s1 = a.s1 + in.off, *s2 = a.s2 + in.off;
    const int ne = in.ne;
    const EnsOps<Real> &op = *a.ops;
    if (a.failed[id] != 0) { // stopped by an earlier run: its state is not finite
        if (r == 0) a.steps_out[id] = 0;
        return;
    }
    // max |u| over the instance (FP64), then the CFL time step
    double mx = 0.0;
    for (size_t q = r; q < (size_t)ne * NP; q += G) mx = fmax(mx, fabs((double)u[q]));
    for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    if (G > 32) {
        if ((r & 31) == 0) s_red[r >> 5] = mx;
        __syncthreads();
        mx = s_red[0];
        for (int w = 1; w < G / 32; ++w) mx = fmax(mx, s_red[w]);
        __syncthreads();
    }
    const double deg = NP - 1;
    double dt = a.cfl * in.dx / ((2.0 * deg + 1.0) * fmax(mx, 1e-300));
    // a state so large (or infinite) that its CFL step count has no int: stopped
    // before its first step, failed = -1 (the whole group sees the same mx)
    if (!(a.t_end / dt < 2.0e9)) {
        if (r == 0) {
            a.failed[id] = -1;
            a.steps_out[id] = 0;
            a.dt_out[id] = dt;
        }
        return;
    }
    const long nfull = (long)floor(a.t_end / dt);
    const double last = a.t_end - (double)nfull * dt;
    const long nsteps = nfull + (last > 0.0 ? 1 : 0);
    if (r == 0) {
        a.dt_out[id] = dt;
        a.steps_out[id] = (int)nsteps;
    }
    const Real J = (Real)(in.dx / 2);
    for (long s = 0; s < nsteps; ++s) {
        const double h = s < nfull ? dt : last;
        const Real hr = (Real)h;
        int sbad = 0;
        ens_stage<Real, NP, G, 1>(u, u, s1, ne, J, hr, op, s_t, r, sbad);
        ens_stage<Real, NP, G, 2>(s1, u, s2, ne, J, hr, op, s_t, r, sbad);
        ens_stage<Real, NP, G, 3>(s2, u, u, ne, J, hr, op, s_t, r, sbad);
        // an instance whose state turned non-finite stops here (the others go on);
        // the whole group takes the same decision
        if (group_any<G>(sbad != 0)) {
            if (r == 0) {
                a.failed[id] = (int)(s + 1);
                a.steps_out[id] = (int)(s + 1);
            }
            break;
        }
        if (a.filter) {
            const double lam = h * op.expfac[NP - 2] * 0.15;
            if (LEARNED)
                ens_filter_learned<Real, NP, G>(u, ne, lam, op, r, L, cnt);
            else
                ens_filter<Real, NP, G>(u, ne, lam, op, r);
        }
    }
}

template <class Real, int G, bool LEARNED>
__device__ __forceinline__ void ens_dispatch(const EnsArgs<Real> &a, int id, Real *s_t, double *s_red, int r, int &bad,
                                             const EnsLearn &L, unsigned long long (&cnt)[4]) {
    switch (a.inst[id].np) {
    case 2: ens_run<Real, 2, G, LEARNED>(a, id, s_t, s_red, r, bad, L, cnt); break;
    case 3: ens_run<Real, 3, G, LEARNED>(a, id, s_t, s_red, r, bad, L, cnt); break;
    case 4: ens_run<Real, 4, G, LEARNED>(a, id, s_t, s_red, r, bad, L, cnt); break;
    case 5: ens_run<Real, 5, G, LEARNED>(a, id, s_t, s_red, r, bad, L, cnt); break;
    case 6: ens_run<Real, 6, G, LEARNED>(a, id, s_t, s_red, r, bad, L, cnt); break;
    }
}

template <class Real> constexpr size_t ens_smem_bytes() {
    return sizeof(Real) * (4 * ENS_MAX_NE_CTA > 4 * ENS_MAX_NE_WARP * ENS_WARPS ? 4 * ENS_MAX_NE_CTA
                                                                                 : 4 * ENS_MAX_NE_WARP * ENS_WARPS);
}

// LEARNED: the post-step indicator is the network (a.mlp set); a separate
// instantiation, so that the plain kernel keeps its register budget.
template <class Real, bool LEARNED>
__global__ void __launch_bounds__(ENS_THREADS, sizeof(Real) == 4 ? 2 : 1) k_ensemble(const EnsArgs<Real> a) {
    extern __shared__ __align__(16) unsigned char ens_smem[];
    Real *s_all = reinterpret_cast<Real *>(ens_smem);
    __shared__ double s_red[ENS_WARPS];
    __shared__ int s_id;
    int bad = 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // learned indicator: weights and per-warp tiles after the trace scratch
    EnsLearn L;
    L.on = LEARNED;
    L.thr = a.thr;
    L.band = a.band;
    {
        unsigned char *m = ens_smem + ens_smem_bytes<Real>();
        __nv_bfloat16 *sW1 = reinterpret_cast<__nv_bfloat16 *>(m);
        __nv_bfloat16 *sW2 = sW1 + frmlp::NH * frmlp::NIN;
        float *sb = reinterpret_cast<float *>(sW2 + frmlp::NH * frmlp::NH);
        __nv_bfloat16 *xs = reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<unsigned char *>(sb) + ENS_MLP_SB);
        float *pr = reinterpret_cast<float *>(xs + ENS_WARPS * 16 * frmlp::NIN);
        L.view = frmlp::smem_view(sW1, sW2, sb);
        L.xs = xs + warp * 16 * frmlp::NIN;
        L.prob = pr + warp * 16;
        if (LEARNED) {
            frmlp::stage_weights(a.mlp, sW1, sW2, sb);
            __syncthreads();
        }
    }
    unsigned long long cnt[4] = {0, 0, 0, 0};
    // phase 1: the whole CTA on one large instance at a time
    for (;;) {
        if (threadIdx.x == 0) s_id = atomicAdd(&a.counters[0], 1);
        __syncthreads();
        const int q = s_id;
        __syncthreads();
        if (q >= a.n_cta) break;
        ens_dispatch<Real, ENS_THREADS, LEARNED>(a, a.queue_cta[q], s_all, s_red, threadIdx.x, bad, L, cnt);
    }
    // phase 2: every warp on small instances
    Real *s_w = s_all + (size_t)warp * 4 * ENS_MAX_NE_WARP;
    for (;;) {
        int q = 0;
        if (lane == 0) q = atomicAdd(&a.counters[1], 1);
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= a.n_warp) break;
        ens_dispatch<Real, 32, LEARNED>(a, a.queue_warp[q], s_w, s_red, lane, bad, L, cnt);
    }
    if (bad) atomicOr(a.status, bad);
    if (LEARNED) {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            unsigned long long v = cnt[c];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (lane == 0 && v) atomicAdd(&a.istats[c], v);
        }
    }
}

// Features (rows of 32) and plain labels of every element of every instance
// in the current state, for the training set of the 1D learned indicator.
template <class Real, int NP>
__device__ void ens_features_inst(const EnsArgs<Real> &a, int id, long eoff, float *feat, int *labels) {
    const EnsInstance in = a.inst[id];
    const Real *u = a.u + in.off;
    __nv_bfloat16 row[frmlp::NIN];
    for (int i = threadIdx.x; i < in.ne; i += blockDim.x) {
        Real h[NP], tot;
        const bool plain = ens_modes<Real, NP>(u, in.ne, i, *a.ops, h, tot);
        ens_feature_row<Real, NP>(h, tot, row);
        for (int q = 0; q < frmlp::NIN; ++q) feat[(eoff + i) * frmlp::NIN + q] = __bfloat162float(row[q]);
        labels[eoff + i] = plain ? 1 : 0;
    }
}

template <class Real>
__global__ void k_ens_features(const EnsArgs<Real> a, const long *__restrict__ eoff, float *feat, int *labels) {
    const int id = blockIdx.x;
    switch (a.inst[id].np) {
    case 2: ens_features_inst<Real, 2>(a, id, eoff[id], feat, labels); break;
    case 3: ens_features_inst<Real, 3>(a, id, eoff[id], feat, labels); break;
    case 4: ens_features_inst<Real, 4>(a, id, eoff[id], feat, labels); break;
    case 5: ens_features_inst<Real, 5>(a, id, eoff[id], feat, labels); break;
    case 6: ens_features_inst<Real, 6>(a, id, eoff[id], feat, labels); break;
    }
}

} // namespace
