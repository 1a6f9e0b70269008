// mlp.cu -- learned troubled-cell indicator: a 32 -> 64 -> 64 -> 1 perceptron
// (GELU, GELU, sigmoid) fed with per-element modal energies, trained and
// evaluated by hand-written BF16-in / FP32-accumulate tensor-core kernels
// (training: warp-level mma.sync m16n8k16 in the backward pass; inference and
// the indicator: tcgen05.mma with TMEM accumulators, mlp_device.cuh), and an
// indicator + :l2 modal filter kernel
// that uses it in place of the modal-decay test of example/shock-vortex.jl:308-321
// with the plain test (src/dissipation.jl:13-23) as fallback and judge.
//
// Parameter vector (FP32 master copy), row-major [out][in]:
//   W1[64][32] b1[64] W2[64][64] b2[64] W3[64] b3[1]        (6337 values)
// Features of an element with np x np points (np = 4): the normalised modal
// energies of density (16) and pressure (16),
//   x_q = clamp(log10(u_hat_q^2 / sum u_hat^2 + 1e-16), -16, 0) / 8 + 1.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "fr_common.cuh"
#include "frgpu_internal.h"

#include "mlp_device.cuh"

namespace {

using namespace frmlp;

// ---------------------------------------------------------------- forward (tests, evaluation)
// The network on n feature rows X[n][32] (FP32, rounded to BF16 as they load)
// -> y[n] = sigmoid(logit): persistent CTAs of four warps over groups of 64
// rows on the tcgen05 tensor cores, the same arithmetic as the indicator
// kernels.  A wait that times out sets *status.
__global__ void __launch_bounds__(32 * WARPS, 4) k_mlp_forward(MLPDev w, const float *__restrict__ X, long n,
                                                             float *__restrict__ y, int *__restrict__ status) {
    static_assert(WARPS == 4, "the tcgen05 network runs on four warps");
    __shared__ __align__(128) unsigned char sm[TCS_BYTES];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t tmem = tc_begin(sm, w.TC, tid);
    uint32_t phase = 0;
    const int half = lane >> 4, r = 16 * warp + (lane & 15);
    const float *prob = reinterpret_cast<const float *>(sm + TCS_PROB);
    const long ngroups = (n + 63) / 64;
    for (long grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        const long smp = grp * 64 + r;
        float feat[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) feat[q] = smp < n ? X[smp * NIN + 16 * half + q] : 0.0f;
        store_features_tc(sm, r, half, feat);
        if (!mlp_tc_forward64(sm, tmem, phase, tid)) break;
        if (half == 0 && smp < n) y[smp] = prob[r];
    }
    if (tc_end(sm, tmem, phase, tid) && tid == 0) atomicOr(status, frk::ST_TIMEOUT);
}

// ---------------------------------------------------------------- loss + gradient
// Mean binary cross-entropy over the n samples listed in idx (or 0..n-1), and
// its gradient accumulated into grad[NPARAM] (zeroed by the caller).  Each warp
// runs forward and backward for 16 samples; the weight gradients are tensor-core
// products over the sample dimension (K = 16).
__global__ void __launch_bounds__(32 * GWARPS) k_mlp_grad(MLPDev w, const float *__restrict__ X,
                                                       const float *__restrict__ T, const int *__restrict__ idx,
                                                       long n, float inv_total, float *__restrict__ grad,
                                                       float *__restrict__ loss) {
    __shared__ __align__(16) __nv_bfloat16 xs_all[GWARPS][16 * NIN];
    __shared__ __align__(16) __nv_bfloat16 h1s_all[GWARPS][16 * NH];
    __shared__ __align__(16) __nv_bfloat16 d2s_all[GWARPS][16 * NH];
    __shared__ __align__(16) __nv_bfloat16 d1s_all[GWARPS][16 * NH];
    __shared__ float gs[NPARAM];
    __shared__ float lsum;
    for (int q = threadIdx.x; q < NPARAM; q += blockDim.x) gs[q] = 0.f;
    if (threadIdx.x == 0) lsum = 0.f;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    __nv_bfloat16 *xs = xs_all[warp], *h1s = h1s_all[warp], *d2s = d2s_all[warp], *d1s = d1s_all[warp];
    const float *w3 = w.P + OFF_W3;
    const long ntiles = (n + 15) / 16;
    for (long tile = (long)blockIdx.x * GWARPS + warp; tile < ntiles; tile += (long)gridDim.x * GWARPS) {
        for (int q = lane; q < 16 * NIN; q += 32) {
            const long s = tile * 16 + q / NIN;
            float v = 0.f;
            if (s < n) v = X[(idx ? (long)idx[s] : s) * NIN + q % NIN];
            xs[q] = __float2bfloat16_rn(v);
        }
        __syncwarp();
        Fwd f;
        mlp_forward_tile(global_view(w), xs, f);
        // output layer: delta3 = (y - t) / N for the mean BCE with a sigmoid
        const long s0 = tile * 16 + g, s1 = tile * 16 + g + 8;
        float d3g = 0.f, d3g8 = 0.f, lpart = 0.f;
        if (s0 < n) {
            const float tt = T[idx ? idx[s0] : s0];
            const float yy = sigmoidf_(f.logit_g);
            d3g = (yy - tt) * inv_total;
            const float yc = fminf(fmaxf(yy, 1e-7f), 1.f - 1e-7f);
            lpart -= tt * logf(yc) + (1.f - tt) * logf(1.f - yc);
        }
        if (s1 < n) {
            const float tt = T[idx ? idx[s1] : s1];
            const float yy = sigmoidf_(f.logit_g8);
            d3g8 = (yy - tt) * inv_total;
            const float yc = fminf(fmaxf(yy, 1e-7f), 1.f - 1e-7f);
            lpart -= tt * logf(yc) + (1.f - tt) * logf(1.f - yc);
        }
        if (t == 0 && lpart != 0.f) atomicAdd(&lsum, lpart * inv_total);
        // dW3, db3 and delta2 = delta3 * w3 * gelu'(a2); db2
        float d2[8][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int c0 = 8 * j + 2 * t;
            float gw0 = d3g * gelu(f.a2[j][0]) + d3g8 * gelu(f.a2[j][2]);
            float gw1 = d3g * gelu(f.a2[j][1]) + d3g8 * gelu(f.a2[j][3]);
            const float w0 = __ldg(w3 + c0), w1 = __ldg(w3 + c0 + 1);
            d2[j][0] = d3g * w0 * dgelu(f.a2[j][0]);
            d2[j][1] = d3g * w1 * dgelu(f.a2[j][1]);
            d2[j][2] = d3g8 * w0 * dgelu(f.a2[j][2]);
            d2[j][3] = d3g8 * w1 * dgelu(f.a2[j][3]);
            float gb0 = d2[j][0] + d2[j][2], gb1 = d2[j][1] + d2[j][3];
#pragma unroll
            for (int off = 4; off < 32; off <<= 1) {
                gw0 += __shfl_xor_sync(0xffffffffu, gw0, off);
                gw1 += __shfl_xor_sync(0xffffffffu, gw1, off);
                gb0 += __shfl_xor_sync(0xffffffffu, gb0, off);
                gb1 += __shfl_xor_sync(0xffffffffu, gb1, off);
            }
            if (g == 0) {
                atomicAdd(&gs[OFF_W3 + c0], gw0);
                atomicAdd(&gs[OFF_W3 + c0 + 1], gw1);
                atomicAdd(&gs[OFF_B2 + c0], gb0);
                atomicAdd(&gs[OFF_B2 + c0 + 1], gb1);
            }
            // stash delta2 and h1 (bf16, [sample][unit]) for the weight products
            d2s[g * NH + c0] = __float2bfloat16_rn(d2[j][0]);
            d2s[g * NH + c0 + 1] = __float2bfloat16_rn(d2[j][1]);
            d2s[(g + 8) * NH + c0] = __float2bfloat16_rn(d2[j][2]);
            d2s[(g + 8) * NH + c0 + 1] = __float2bfloat16_rn(d2[j][3]);
            h1s[g * NH + c0] = __float2bfloat16_rn(gelu(f.a1[j][0]));
            h1s[g * NH + c0 + 1] = __float2bfloat16_rn(gelu(f.a1[j][1]));
            h1s[(g + 8) * NH + c0] = __float2bfloat16_rn(gelu(f.a1[j][2]));
            h1s[(g + 8) * NH + c0 + 1] = __float2bfloat16_rn(gelu(f.a1[j][3]));
        }
        {
            float gb = d3g + d3g8;
#pragma unroll
            for (int off = 4; off < 32; off <<= 1) gb += __shfl_xor_sync(0xffffffffu, gb, off);
            if (lane == 0) atomicAdd(&gs[OFF_B3], gb);
        }
        // delta1 = (delta2 W2) * gelu'(a1): A = delta2 [16 x 64], B(k=o, n=i) = W2[o][i] = W2T[i][o]
        uint32_t ad2[4][4];
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            ad2[kk][0] = pack_bf16(d2[2 * kk][0], d2[2 * kk][1]);
            ad2[kk][1] = pack_bf16(d2[2 * kk][2], d2[2 * kk][3]);
            ad2[kk][2] = pack_bf16(d2[2 * kk + 1][0], d2[2 * kk + 1][1]);
            ad2[kk][3] = pack_bf16(d2[2 * kk + 1][2], d2[2 * kk + 1][3]);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
            const __nv_bfloat16 *row = w.W2T + (8 * j + g) * NH;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
                mma16816(acc, ad2[kk], ld_pair(row + 16 * kk + 2 * t), ld_pair(row + 16 * kk + 8 + 2 * t));
            const int c0 = 8 * j + 2 * t;
            const float e0 = acc[0] * dgelu(f.a1[j][0]), e1 = acc[1] * dgelu(f.a1[j][1]);
            const float e2 = acc[2] * dgelu(f.a1[j][2]), e3 = acc[3] * dgelu(f.a1[j][3]);
            d1s[g * NH + c0] = __float2bfloat16_rn(e0);
            d1s[g * NH + c0 + 1] = __float2bfloat16_rn(e1);
            d1s[(g + 8) * NH + c0] = __float2bfloat16_rn(e2);
            d1s[(g + 8) * NH + c0 + 1] = __float2bfloat16_rn(e3);
            float gb0 = e0 + e2, gb1 = e1 + e3;
#pragma unroll
            for (int off = 4; off < 32; off <<= 1) {
                gb0 += __shfl_xor_sync(0xffffffffu, gb0, off);
                gb1 += __shfl_xor_sync(0xffffffffu, gb1, off);
            }
            if (g == 0) {
                atomicAdd(&gs[OFF_B1 + c0], gb0);
                atomicAdd(&gs[OFF_B1 + c0 + 1], gb1);
            }
        }
        __syncwarp();
        // dW2[o][i] = sum_s delta2[s][o] h1[s][i]: M = 64 (o), N = 64 (i), K = 16 (s)
#pragma unroll 1
        for (int mt = 0; mt < 4; ++mt) {
            uint32_t a[4];
            const int o0 = 16 * mt + g;
            a[0] = pack_bf16_raw(d2s[(2 * t) * NH + o0], d2s[(2 * t + 1) * NH + o0]);
            a[1] = pack_bf16_raw(d2s[(2 * t) * NH + o0 + 8], d2s[(2 * t + 1) * NH + o0 + 8]);
            a[2] = pack_bf16_raw(d2s[(2 * t + 8) * NH + o0], d2s[(2 * t + 9) * NH + o0]);
            a[3] = pack_bf16_raw(d2s[(2 * t + 8) * NH + o0 + 8], d2s[(2 * t + 9) * NH + o0 + 8]);
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const int i0 = 8 * nt + g;
                float acc[4] = {0.f, 0.f, 0.f, 0.f};
                mma16816(acc, a, pack_bf16_raw(h1s[(2 * t) * NH + i0], h1s[(2 * t + 1) * NH + i0]),
                         pack_bf16_raw(h1s[(2 * t + 8) * NH + i0], h1s[(2 * t + 9) * NH + i0]));
                const int c0 = 8 * nt + 2 * t;
                atomicAdd(&gs[OFF_W2 + o0 * NH + c0], acc[0]);
                atomicAdd(&gs[OFF_W2 + o0 * NH + c0 + 1], acc[1]);
                atomicAdd(&gs[OFF_W2 + (o0 + 8) * NH + c0], acc[2]);
                atomicAdd(&gs[OFF_W2 + (o0 + 8) * NH + c0 + 1], acc[3]);
            }
        }
        // dW1[i][f] = sum_s delta1[s][i] x[s][f]: M = 64 (i), N = 32 (f), K = 16 (s)
#pragma unroll 1
        for (int mt = 0; mt < 4; ++mt) {
            uint32_t a[4];
            const int o0 = 16 * mt + g;
            a[0] = pack_bf16_raw(d1s[(2 * t) * NH + o0], d1s[(2 * t + 1) * NH + o0]);
            a[1] = pack_bf16_raw(d1s[(2 * t) * NH + o0 + 8], d1s[(2 * t + 1) * NH + o0 + 8]);
            a[2] = pack_bf16_raw(d1s[(2 * t + 8) * NH + o0], d1s[(2 * t + 9) * NH + o0]);
            a[3] = pack_bf16_raw(d1s[(2 * t + 8) * NH + o0 + 8], d1s[(2 * t + 9) * NH + o0 + 8]);
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int f0 = 8 * nt + g;
                float acc[4] = {0.f, 0.f, 0.f, 0.f};
                mma16816(acc, a, pack_bf16_raw(xs[(2 * t) * NIN + f0], xs[(2 * t + 1) * NIN + f0]),
                         pack_bf16_raw(xs[(2 * t + 8) * NIN + f0], xs[(2 * t + 9) * NIN + f0]));
                const int c0 = 8 * nt + 2 * t;
                atomicAdd(&gs[OFF_W1 + o0 * NIN + c0], acc[0]);
                atomicAdd(&gs[OFF_W1 + o0 * NIN + c0 + 1], acc[1]);
                atomicAdd(&gs[OFF_W1 + (o0 + 8) * NIN + c0], acc[2]);
                atomicAdd(&gs[OFF_W1 + (o0 + 8) * NIN + c0 + 1], acc[3]);
            }
        }
        __syncwarp();
    }
    __syncthreads();
    for (int q = threadIdx.x; q < NPARAM; q += blockDim.x)
        if (gs[q] != 0.f) atomicAdd(&grad[q], gs[q]);
    if (threadIdx.x == 0 && lsum != 0.f) atomicAdd(loss, lsum);
}

// Parameter q of the FP32 vector into the packed network of the tcgen05 path.
__device__ __forceinline__ void tc_pack_param(unsigned char *tc, int q, float p) {
    if (q < OFF_B1) {
        const int o = (q - OFF_W1) / NIN, i = (q - OFF_W1) % NIN;
        *reinterpret_cast<__nv_bfloat16 *>(tc + TCP_W1 + core_off(o, i, NIN)) = __float2bfloat16_rn(p);
    } else if (q < OFF_W2) {
        reinterpret_cast<float *>(tc + TCP_B1)[q - OFF_B1] = p;
    } else if (q < OFF_B2) {
        const int o = (q - OFF_W2) / NH, i = (q - OFF_W2) % NH;
        *reinterpret_cast<__nv_bfloat16 *>(tc + TCP_W2 + core_off(o, i, NH)) = __float2bfloat16_rn(p);
    } else if (q < OFF_W3) {
        reinterpret_cast<float *>(tc + TCP_B2)[q - OFF_B2] = p;
    } else if (q < OFF_B3) {
        reinterpret_cast<float *>(tc + TCP_W3)[q - OFF_W3] = p;
    } else {
        reinterpret_cast<float *>(tc + TCP_B3)[0] = p;
    }
}

// Adam update of the FP32 master copy and refresh of the BF16 copies.
__global__ void k_mlp_adam(float *__restrict__ P, float *__restrict__ m, float *__restrict__ v,
                           const float *__restrict__ grad, float lr, float b1, float b2, float eps, float c1,
                           float c2, __nv_bfloat16 *W1, __nv_bfloat16 *W2, __nv_bfloat16 *W2T,
                           unsigned char *TC) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= NPARAM) return;
    const float gq = grad[q];
    const float mq = b1 * m[q] + (1.f - b1) * gq;
    const float vq = b2 * v[q] + (1.f - b2) * gq * gq;
    m[q] = mq;
    v[q] = vq;
    const float p = P[q] - lr * (mq * c1) / (sqrtf(vq * c2) + eps);
    P[q] = p;
    tc_pack_param(TC, q, p);
    const __nv_bfloat16 pb = __float2bfloat16_rn(p);
    if (q < OFF_B1) W1[frag_w1((q - OFF_W1) / NIN, (q - OFF_W1) % NIN)] = pb;
    else if (q >= OFF_W2 && q < OFF_B2) {
        const int r = q - OFF_W2, o = r / NH, i = r % NH;
        W2[frag_w2(o, i)] = pb;
        W2T[i * NH + o] = pb;
    }
}

__global__ void k_mlp_refresh(const float *__restrict__ P, __nv_bfloat16 *W1, __nv_bfloat16 *W2, __nv_bfloat16 *W2T,
                              unsigned char *TC) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= NPARAM) return;
    tc_pack_param(TC, q, P[q]);
    const __nv_bfloat16 pb = __float2bfloat16_rn(P[q]);
    if (q < OFF_B1) W1[frag_w1((q - OFF_W1) / NIN, (q - OFF_W1) % NIN)] = pb;
    else if (q >= OFF_W2 && q < OFF_B2) {
        const int r = q - OFF_W2, o = r / NH, i = r % NH;
        W2[frag_w2(o, i)] = pb;
        W2T[i * NH + o] = pb;
    }
}

// ---------------------------------------------------------------- features + indicator

// Modal energies of density and pressure of 16 elements per warp (np = 4).
// Lane L and L + 16 share element e = base + (L & 15): each loads the four
// variables at 8 of the 16 points (lower lane points 0-7, upper 8-15), then
// they swap halves so that the lower lane holds the density values and the
// upper lane the pressure values.  The lower lane's su is the plain
// modal-decay ratio of the density.  Lanes of elements past the end (valid
// false) must still take part in the exchange; they return zero features.
// The raw values a lane needs: the four variables at its 8 points.
template <class Real>
__device__ __forceinline__ void load_raw(const Real *__restrict__ u, size_t ne, size_t e, bool valid, bool pressure,
                                         float (&w)[8][4]) {
    const int q0 = pressure ? 8 : 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        if (valid) {
            Real v[4];
            frk::ld4(u + frk::e2d_index(e, q0 + k, 0, ne), v);
#pragma unroll
            for (int m = 0; m < 4; ++m) w[k][m] = (float)v[m];
        } else {
            w[k][0] = 1.f;
            w[k][1] = w[k][2] = w[k][3] = 0.f;
        }
    }
}


template <class Real>
__device__ __forceinline__ void element_features(const Real *__restrict__ u, size_t ne, size_t e, bool valid,
                                                 bool pressure, const IV1 &iv, float gm1, float (&feat)[16],
                                                 float &su) {
    float w[8][4];
    load_raw<Real>(u, ne, e, valid, pressure, w);
    features_from_raw(w, valid, pressure, iv, gm1, feat, su);
}

// One warp per 16 elements (the indicator kernel's tiling, so that training
// features and inference features are the same numbers).
template <class Real>
__global__ void __launch_bounds__(128) k_features(const Real *__restrict__ u, size_t ne, IV1 iv, float gm1,
                                                  float *__restrict__ feat) {
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const size_t e = (t >> 5) * 16 + (lane & 15);
    if ((t >> 5) * 16 >= ne) return; // whole warp past the end
    const bool pr = lane >= 16, valid = e < ne;
    float f[16], su;
    element_features<Real>(u, ne, e, valid, pr, iv, gm1, f, su);
    if (!valid) return;
#pragma unroll
    for (int a = 0; a < 16; ++a) feat[e * NIN + (pr ? 16 : 0) + a] = f[a];
}


// Learned indicator + :l2 modal filter on a 2D Euler state (np = 4).  Per
// element: features -> MLP -> probability.  Where the probability is within
// `band` of `thr` the plain modal-decay test decides (fallback); otherwise the
// network does, except below the smooth floor (below_floor) where the element
// is smooth.  stats: [0] troubled, [1] network vs plain disagreements
// (misfires, judged by the plain test), [2] fallbacks.
// The learned indicator + :l2 filter over a 2D state (np = 4), persistent: a
// CTA of four warps takes groups of 64 consecutive elements; warp w holds
// elements 16 w .. 16 w + 15 of the group (lanes L and L + 16 share one).  The
// network runs on the tcgen05 tensor cores (mlp_tc_forward64, weights copied
// once per CTA); the decision takes the plain test as fallback and judge.  The
// next group's state values are loaded while the network runs.  A wait that
// times out sets ST_TIMEOUT in *status and ends the CTA's work.
template <class Real>
__global__ void __launch_bounds__(32 * WARPS, 4) k_mlp_indicator(MLPDev w, Real *__restrict__ u, Real *__restrict__ lo,
                                                            size_t ne, const Real *__restrict__ V,
                                                            const Real *__restrict__ iV, IV1 iv, float gm1,
                                                            float thr, float band, float S0, float kappa, double lam,
                                                            int *__restrict__ flags, int *__restrict__ stats,
                                                            int *__restrict__ status) {
    static_assert(WARPS == 4, "the tcgen05 network runs on four warps");
    __shared__ __align__(128) unsigned char sm[TCS_BYTES];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t tmem = tc_begin(sm, w.TC, tid);
    const float *prob = reinterpret_cast<const float *>(sm + TCS_PROB) + 16 * warp;
    const size_t ngroups = (ne + 63) / 64;
    int n_trouble = 0, n_mis = 0, n_fb = 0;
    const bool pr = lane >= 16;
    uint32_t phase = 0;
    float raw[8][4]; // this lane's values of the group being processed, loaded one group ahead
    size_t grp = blockIdx.x;
    if (grp < ngroups) {
        const size_t e = grp * 64 + 16 * warp + (lane & 15);
        load_raw<Real>(u, ne, e, e < ne, pr, raw);
    }
    for (; grp < ngroups; grp += gridDim.x) {
        const size_t e = grp * 64 + 16 * warp + (lane & 15);
        float feat[16], su = 0.f;
        features_from_raw(raw, e < ne, pr, iv, gm1, feat, su);
        store_features_tc(sm, 16 * warp + (lane & 15), pr ? 1 : 0, feat);
        if (grp + gridDim.x < ngroups) {
            const size_t en = (grp + gridDim.x) * 64 + 16 * warp + (lane & 15);
            load_raw<Real>(u, ne, en, en < ne, pr, raw);
        }
        if (!mlp_tc_forward64(sm, tmem, phase, tid)) break;
        bool bad = false;
        if (!pr && e < ne) {
            const bool plain = plain_troubled(su, S0, kappa);
            const float pm = below_floor(su, S0, kappa) ? 0.f : prob[lane];
            const bool fallback = fabsf(pm - thr) < band;
            const bool net = pm > thr;
            bad = fallback ? plain : net;
            n_fb += fallback;
            n_mis += (net != plain);
            n_trouble += bad;
            flags[e] = bad ? 1 : 0;
        }
        // :l2 modal filter of the troubled elements
        warp_filter_elements<Real>(__ballot_sync(0xffffffffu, bad), grp * 64 + 16 * warp, u, lo, ne, V, iV, lam);
    }
    if (tc_end(sm, tmem, phase, tid) && tid == 0) atomicOr(status, frk::ST_TIMEOUT);
    // warp-reduce the statistics, one atomic per warp
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        n_trouble += __shfl_xor_sync(0xffffffffu, n_trouble, off);
        n_mis += __shfl_xor_sync(0xffffffffu, n_mis, off);
        n_fb += __shfl_xor_sync(0xffffffffu, n_fb, off);
    }
    if (lane == 0) {
        if (n_trouble) atomicAdd(&stats[0], n_trouble);
        if (n_mis) atomicAdd(&stats[1], n_mis);
        if (n_fb) atomicAdd(&stats[2], n_fb);
    }
}

uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

} // namespace

// ---------------------------------------------------------------- host objects
struct frgpu_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    float *P = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *loss = nullptr;
    __nv_bfloat16 *W1 = nullptr, *W2 = nullptr, *W2T = nullptr;
    unsigned char *TC = nullptr; // packed for the tcgen05 path (TCP_* layout)
    long step = 0;
    long launches = 0;
    MLPDev dev() const { return MLPDev{P, W1, W2, W2T, TC}; }
};

static void mlp_free(frgpu_mlp *m) {
    if (!m) return;
    if (m->stream) cudaStreamSynchronize(m->stream);
    void *b[] = {m->P, m->m, m->v, m->grad, m->loss, m->W1, m->W2, m->W2T, m->TC};
    for (void *p : b)
        if (p) cudaFree(p);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
}

static int mlp_refresh(frgpu_mlp *m) {
    k_mlp_refresh<<<(NPARAM + 255) / 256, 256, 0, m->stream>>>(m->P, m->W1, m->W2, m->W2T, m->TC);
    FR_CUDA(cudaGetLastError());
    m->launches += 1;
    return FRGPU_OK;
}

// Device buffer sized for `count` elements of T, grown on demand (freed at exit of the call).
template <class T> struct DevBuf {
    T *p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    int alloc(size_t count) {
        FR_CUDA(cudaMalloc(&p, sizeof(T) * (count ? count : 1)));
        return FRGPU_OK;
    }
};

extern "C" {

FRGPU_API int frgpu_mlp_nparams(void) { return NPARAM; }

FRGPU_API int frgpu_mlp_create(int seed, frgpu_mlp **out) {
    if (!out) {
        fr_set_error("mlp_create: null output");
        return FRGPU_ERR_ARG;
    }
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        fr_set_error("mlp_create: no CUDA device");
        return FRGPU_ERR_CUDA;
    }
    auto *m = new frgpu_mlp();
    cudaGetDevice(&m->device);
    int rc = [&]() -> int {
        FR_CUDA(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
        FR_CUDA(cudaMalloc(&m->P, sizeof(float) * NPARAM));
        FR_CUDA(cudaMalloc(&m->m, sizeof(float) * NPARAM));
        FR_CUDA(cudaMalloc(&m->v, sizeof(float) * NPARAM));
        FR_CUDA(cudaMalloc(&m->grad, sizeof(float) * NPARAM));
        FR_CUDA(cudaMalloc(&m->loss, sizeof(float)));
        FR_CUDA(cudaMalloc(&m->W1, sizeof(__nv_bfloat16) * NH * NIN));
        FR_CUDA(cudaMalloc(&m->W2, sizeof(__nv_bfloat16) * NH * NH));
        FR_CUDA(cudaMalloc(&m->W2T, sizeof(__nv_bfloat16) * NH * NH));
        FR_CUDA(cudaMalloc(&m->TC, TCP_BYTES));
        FR_CUDA(cudaMemset(m->TC, 0, TCP_BYTES));
        FR_CUDA(cudaMemset(m->m, 0, sizeof(float) * NPARAM));
        FR_CUDA(cudaMemset(m->v, 0, sizeof(float) * NPARAM));
        // deterministic init: uniform(-a, a) with a = sqrt(6 / fan_in) (He-uniform), zero biases
        std::vector<float> h(NPARAM, 0.f);
        auto uni = [&](uint32_t k) { return (hash32(k ^ (uint32_t)seed * 0x9e3779b9U) >> 8) * (1.0f / 16777216.0f); };
        const float a1 = std::sqrt(6.f / NIN), a2 = std::sqrt(6.f / NH), a3 = std::sqrt(3.f / NH);
        for (int q = 0; q < NH * NIN; ++q) h[OFF_W1 + q] = (2.f * uni(q) - 1.f) * a1;
        for (int q = 0; q < NH * NH; ++q) h[OFF_W2 + q] = (2.f * uni(100000 + q) - 1.f) * a2;
        for (int q = 0; q < NH; ++q) h[OFF_W3 + q] = (2.f * uni(200000 + q) - 1.f) * a3;
        FR_CUDA(cudaMemcpy(m->P, h.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
        return mlp_refresh(m);
    }();
    if (rc) {
        mlp_free(m);
        return rc;
    }
    FR_CUDA(cudaStreamSynchronize(m->stream));
    *out = m;
    return FRGPU_OK;
}

FRGPU_API void frgpu_mlp_destroy(frgpu_mlp *m) { mlp_free(m); }

FRGPU_API int frgpu_mlp_get_params(const frgpu_mlp *m, float *params) {
    if (!m || !params) {
        fr_set_error("mlp_get_params: null argument");
        return FRGPU_ERR_ARG;
    }
    FR_CUDA(cudaStreamSynchronize(m->stream));
    FR_CUDA(cudaMemcpy(params, m->P, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
    return FRGPU_OK;
}

FRGPU_API int frgpu_mlp_set_params(frgpu_mlp *m, const float *params) {
    if (!m || !params) {
        fr_set_error("mlp_set_params: null argument");
        return FRGPU_ERR_ARG;
    }
    FR_CUDA(cudaMemcpyAsync(m->P, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice, m->stream));
    int rc = mlp_refresh(m);
    if (rc) return rc;
    FR_CUDA(cudaStreamSynchronize(m->stream));
    return FRGPU_OK;
}

FRGPU_API int frgpu_mlp_forward(frgpu_mlp *m, const float *x, long n, float *y) {
    if (!m || !x || !y || n < 0) {
        fr_set_error("mlp_forward: bad arguments");
        return FRGPU_ERR_ARG;
    }
    if (n == 0) return FRGPU_OK;
    DevBuf<float> dx, dy;
    DevBuf<int> dst;
    int rc;
    if ((rc = dx.alloc((size_t)n * NIN)) || (rc = dy.alloc(n)) || (rc = dst.alloc(1))) return rc;
    FR_CUDA(cudaMemsetAsync(dst.p, 0, sizeof(int), m->stream));
    FR_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(float) * n * NIN, cudaMemcpyHostToDevice, m->stream));
    // persistent: at most 4 CTAs per SM (64 tensor-memory columns each)
    const int grid = (int)std::min<long>((n + 63) / 64, 152 * 4);
    k_mlp_forward<<<grid, 32 * WARPS, 0, m->stream>>>(m->dev(), dx.p, n, dy.p, dst.p);
    FR_CUDA(cudaGetLastError());
    m->launches += 1;
    int st = 0;
    FR_CUDA(cudaMemcpyAsync(y, dy.p, sizeof(float) * n, cudaMemcpyDeviceToHost, m->stream));
    FR_CUDA(cudaMemcpyAsync(&st, dst.p, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
    FR_CUDA(cudaStreamSynchronize(m->stream));
    if (st) {
        fr_set_error("mlp_forward: a tensor-core wait timed out");
        return FRGPU_ERR_TIMEOUT;
    }
    return FRGPU_OK;
}

static int mlp_grad_launch(frgpu_mlp *m, const float *dX, const float *dT, const int *didx, long n, float inv_total) {
    FR_CUDA(cudaMemsetAsync(m->grad, 0, sizeof(float) * NPARAM, m->stream));
    FR_CUDA(cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream));
    const int grid = (int)std::min<long>((n + 16 * GWARPS - 1) / (16 * GWARPS), 152 * 4);
    k_mlp_grad<<<grid, 32 * GWARPS, 0, m->stream>>>(m->dev(), dX, dT, didx, n, inv_total, m->grad, m->loss);
    FR_CUDA(cudaGetLastError());
    m->launches += 1;
    return FRGPU_OK;
}

FRGPU_API int frgpu_mlp_loss_grad(frgpu_mlp *m, const float *x, const float *t, long n, float *loss, float *grad) {
    if (!m || !x || !t || n <= 0) {
        fr_set_error("mlp_loss_grad: bad arguments");
        return FRGPU_ERR_ARG;
    }
    DevBuf<float> dx, dt;
    int rc;
    if ((rc = dx.alloc((size_t)n * NIN)) || (rc = dt.alloc(n))) return rc;
    FR_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(float) * n * NIN, cudaMemcpyHostToDevice, m->stream));
    FR_CUDA(cudaMemcpyAsync(dt.p, t, sizeof(float) * n, cudaMemcpyHostToDevice, m->stream));
    if ((rc = mlp_grad_launch(m, dx.p, dt.p, nullptr, n, 1.0f / (float)n))) return rc;
    if (grad) FR_CUDA(cudaMemcpyAsync(grad, m->grad, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, m->stream));
    if (loss) FR_CUDA(cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    FR_CUDA(cudaStreamSynchronize(m->stream));
    return FRGPU_OK;
}

// Mini-batch Adam on (x, t).  Samples are visited in a per-epoch permutation
// drawn from `seed`; loss_out (optional) receives the mean loss of each epoch.
FRGPU_API int frgpu_mlp_train(frgpu_mlp *m, const float *x, const float *t, long n, int epochs, int batch, float lr,
                              int seed, float *loss_out) {
    if (!m || !x || !t || n <= 0 || epochs < 0 || batch <= 0 || !(lr > 0)) {
        fr_set_error("mlp_train: bad arguments");
        return FRGPU_ERR_ARG;
    }
    DevBuf<float> dx, dt;
    DevBuf<int> didx;
    int rc;
    if ((rc = dx.alloc((size_t)n * NIN)) || (rc = dt.alloc(n)) || (rc = didx.alloc(n))) return rc;
    FR_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(float) * n * NIN, cudaMemcpyHostToDevice, m->stream));
    FR_CUDA(cudaMemcpyAsync(dt.p, t, sizeof(float) * n, cudaMemcpyHostToDevice, m->stream));
    std::vector<int> perm(n);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int ep = 0; ep < epochs; ++ep) {
        for (long q = 0; q < n; ++q) perm[q] = (int)q;
        for (long q = n - 1; q > 0; --q) { // Fisher-Yates with a counter-based hash
            const long r = (long)(hash32((uint32_t)(q * 2654435761u) ^ hash32((uint32_t)(seed * 977 + ep))) % (uint32_t)(q + 1));
            std::swap(perm[q], perm[r]);
        }
        FR_CUDA(cudaMemcpyAsync(didx.p, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, m->stream));
        double ep_loss = 0;
        for (long s = 0; s < n; s += batch) {
            const long nb = std::min<long>(batch, n - s);
            if ((rc = mlp_grad_launch(m, dx.p, dt.p, didx.p + s, nb, 1.0f / (float)nb))) return rc;
            m->step += 1;
            const float c1 = 1.f / (1.f - std::pow(b1, (float)m->step));
            const float c2 = 1.f / (1.f - std::pow(b2, (float)m->step));
            k_mlp_adam<<<(NPARAM + 255) / 256, 256, 0, m->stream>>>(m->P, m->m, m->v, m->grad, lr, b1, b2, eps, c1,
                                                                     c2, m->W1, m->W2, m->W2T, m->TC);
            FR_CUDA(cudaGetLastError());
            m->launches += 1;
            if (loss_out) {
                float l = 0;
                FR_CUDA(cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
                FR_CUDA(cudaStreamSynchronize(m->stream));
                ep_loss += (double)l * nb;
            }
        }
        if (loss_out) loss_out[ep] = (float)(ep_loss / n);
        FR_CUDA(cudaStreamSynchronize(m->stream));
    }
    FR_CUDA(cudaStreamSynchronize(m->stream));
    return FRGPU_OK;
}

} // extern "C"

// ---- used by runtime.cu -------------------------------------------------------
fr_mlp_ptrs fr_mlp_device(const frgpu_mlp *m) { return fr_mlp_ptrs{m->P, m->W1, m->W2, m->W2T, m->TC}; }

// The 1D factor of the space's tensor inverse Vandermonde matrix:
// iV[(i,0),(k,0)] = iV1[i][k] iV1[0][0], and iV1[0][0] = w_0 / sqrt(2) > 0.
void fr_iv1_from_tensor(const frgpu_space &s, float *iv1) {
    const double *iV = s.iV.data();
    const double c = std::sqrt(iV[0]);
    for (int i = 0; i < 4; ++i)
        for (int k = 0; k < 4; ++k) iv1[4 * i + k] = (float)(iV[4 * i + 16 * k] / c);
}

static IV1 iv1_from_tensor(const frgpu_problem *p) {
    IV1 r;
    fr_iv1_from_tensor(p->sp, &r.m[0][0]);
    return r;
}

int fr_fused_indicator(const frgpu_problem *p) {
    const bool fusable = p->fuse_indicator && p->d.equation == FRGPU_EULER2D && p->d.precision == FRGPU_FP32K &&
                         p->sp.np == 4 && p->d_V && p->d_iV && !p->d_met;
    if (!fusable) return FRGPU_IND_NONE;
    if (p->indicator == FRGPU_IND_MLP && p->mlp) return FRGPU_IND_MLP;
    if (p->indicator == FRGPU_IND_PLAIN) return FRGPU_IND_PLAIN;
    return FRGPU_IND_NONE;
}

int fr_launch_features(frgpu_problem *p, float *d_feat) {
    if (p->d.equation != FRGPU_EULER2D || p->sp.np != 4) {
        fr_set_error("modal features: 2D Euler with deg = 3 (32 inputs)");
        return FRGPU_ERR_UNSUPPORTED;
    }
    const size_t ne = (size_t)p->sp.nx * p->sp.ny;
    const int grid = (int)(((ne + 15) / 16 * 32 + 127) / 128);
    const float gm1 = (float)(p->d.gamma - 1.0);
    if (p->d.precision == FRGPU_FP64)
        k_features<double><<<grid, 128, 0, p->stream>>>((const double *)fr_state_hi(p), ne, iv1_from_tensor(p), gm1,
                                                        d_feat);
    else
        k_features<float><<<grid, 128, 0, p->stream>>>((const float *)fr_state_hi(p), ne, iv1_from_tensor(p), gm1,
                                                       d_feat);
    FR_CUDA(cudaGetLastError());
    p->launches += 1;
    return FRGPU_OK;
}

int fr_launch_mlp_indicator(frgpu_problem *p, double lam, double S0, double kappa) {
    if (p->prepare_only) return FRGPU_OK;
    if (!p->mlp) {
        fr_set_error("learned indicator: no network bound to the problem (frgpu_problem_set_mlp)");
        return FRGPU_ERR_ARG;
    }
    if (p->d.equation != FRGPU_EULER2D || p->sp.np != 4) {
        fr_set_error("learned indicator: 2D Euler with deg = 3 (32 inputs)");
        return FRGPU_ERR_UNSUPPORTED;
    }
    const size_t ne = (size_t)p->sp.nx * p->sp.ny;
    const size_t ngroups = (ne + 63) / 64;
    // persistent: as many CTAs as fit at once (4 per SM at <= 128 registers per
    // thread; each holds 64 of the SM's 512 tensor-memory columns)
    int nsm = 152;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device);
    const int grid = (int)std::min<size_t>(ngroups, (size_t)nsm * 4);
    const float gm1 = (float)(p->d.gamma - 1.0);
    FR_CUDA(cudaMemsetAsync(p->d_count, 0, sizeof(int) * 4, p->stream));
    const MLPDev w = p->mlp->dev();
    const IV1 iv1 = iv1_from_tensor(p);
    if (p->d.precision == FRGPU_FP64)
        k_mlp_indicator<double><<<grid, 32 * WARPS, 0, p->stream>>>(
            w, (double *)fr_state_hi(p), nullptr, ne, (const double *)p->d_V, (const double *)p->d_iV, iv1,
            gm1, p->mlp_thr, p->mlp_band, (float)S0, (float)kappa, lam, p->d_flags, p->d_count, p->d_status);
    else
        k_mlp_indicator<float><<<grid, 32 * WARPS, 0, p->stream>>>(
            w, (float *)fr_state_hi(p), (float *)p->s3, ne, (const float *)p->d_V, (const float *)p->d_iV, iv1,
            gm1, p->mlp_thr, p->mlp_band, (float)S0, (float)kappa, lam, p->d_flags, p->d_count, p->d_status);
    FR_CUDA(cudaGetLastError());
    p->launches += 1;
    return FRGPU_OK;
}
