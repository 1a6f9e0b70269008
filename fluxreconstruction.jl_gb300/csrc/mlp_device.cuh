// mlp_device.cuh -- device side of the 32 -> 64 -> 64 -> 1 troubled-cell
// perceptron shared by the training / 2D indicator kernels (mlp.cu) and the
// ensemble's 1D indicator (ensemble_kernels.cuh): parameter layout, BF16
// mma.sync helpers, GELU, and the forward pass of one warp tile of 16 samples.
//
// Parameter vector (FP32 master copy), row-major [out][in]:
//   W1[64][32] b1[64] W2[64][64] b2[64] W3[64] b3[1]        (6337 values)
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "blackwell.cuh"
#include "fr_common.cuh"

namespace frmlp {

constexpr int NIN = 32, NH = 64;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NIN, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NH, NPARAM = OFF_B3 + 1;
constexpr int WARPS = 4;  // warps per CTA of the forward and indicator kernels
constexpr int GWARPS = 2; // warps per CTA of the gradient kernel (static shared memory < 48 KB)

struct MLPDev {
    const float *P;             // FP32 parameters
    const __nv_bfloat16 *W1;    // W1 [64][32] in fragment order (frag_w1)
    const __nv_bfloat16 *W2;    // W2 [64][64] in fragment order (frag_w2)
    const __nv_bfloat16 *W2T;   // [64][64]  row = input unit (backward pass)
    const unsigned char *TC;    // the network packed for the tcgen05 path (TCP_* layout)
};



// Fragment order of the BF16 weight copies: the m16n8k16 B fragments that lane
// (g = lane / 4, t = lane % 4) needs for output tile j (units 8j..8j+7) are
// contiguous, so one 128-bit load fetches two k-steps: word kk * 2 + h holds
// W[8j + g][16 kk + 8 h + 2 t], W[8j + g][16 kk + 8 h + 2 t + 1].
// Position of W1[o][i] (i < 32: 4 words per lane) and W2[o][i] (i < 64: 8 words).
__host__ __device__ __forceinline__ int frag_pos(int o, int i, int words) {
    const int j = o >> 3, g = o & 7, kk = i >> 4, r = i & 15, h = r >> 3, t = (r & 7) >> 1, e = r & 1;
    return ((j * 32 + 4 * g + t) * words + kk * 2 + h) * 2 + e;
}
__host__ __device__ __forceinline__ int frag_w1(int o, int i) { return frag_pos(o, i, 4); }
__host__ __device__ __forceinline__ int frag_w2(int o, int i) { return frag_pos(o, i, 8); }

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}
__device__ __forceinline__ uint32_t pack_bf16_raw(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    __nv_bfloat162 v;
    v.x = lo;
    v.y = hi;
    return *reinterpret_cast<uint32_t *>(&v);
}
__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16 *p) { return *reinterpret_cast<const uint32_t *>(p); }
// products that are never contracted into an FMA (the plain filter kernel is
// built without contraction)
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }

// D = A (16x16 bf16, row) * B (16x8 bf16, col) + C (f32)
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// GELU in its tanh form (Hendrycks and Gimpel, arXiv:1606.08415):
// gelu(x) = x/2 (1 + tanh(z)), z = sqrt(2/pi) (x + 0.044715 x^3), with the
// hardware tanh approximation (tanh.approx.f32).
__device__ __forceinline__ float tanh_fast(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
constexpr float GELU_C = 0.7978845608028654f, GELU_A = 0.044715f;
__device__ __forceinline__ float gelu(float x) {
    const float t = tanh_fast(GELU_C * fmaf(GELU_A * x, x * x, x));
    return 0.5f * x * (1.0f + t);
}
// gelu of two values as packed FP32 pairs: per lane the same operations (and
// roundings) as gelu(), half the arithmetic instructions
__device__ __forceinline__ float2 gelu2(float x0, float x1) {
    const float2 x = make_float2(x0, x1);
    const float2 xx = __fmul2_rn(x, x);
    const float2 ax = __fmul2_rn(make_float2(GELU_A, GELU_A), x);
    const float2 z = __fmul2_rn(make_float2(GELU_C, GELU_C), __ffma2_rn(ax, xx, x));
    const float2 t = make_float2(tanh_fast(z.x), tanh_fast(z.y));
    return __fmul2_rn(__fmul2_rn(make_float2(0.5f, 0.5f), x), __fadd2_rn(make_float2(1.0f, 1.0f), t));
}
__device__ __forceinline__ float dgelu(float x) {
    const float t = tanh_fast(GELU_C * fmaf(GELU_A * x, x * x, x));
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * GELU_C * fmaf(3.0f * GELU_A, x * x, 1.0f);
}

// Forward pass of one warp tile (16 samples).  xs: the tile's features in
// shared memory, bf16 [16][32].  Outputs per lane: pre-activations a1, a2 and
// activations h2 in the m16n8 accumulator layout (rows g and g+8, columns
// 8j + 2t and +1, g = lane/4, t = lane%4), layer-2 input fragments ah1, and
// the logits of rows g and g+8.
struct Fwd {
    float a1[8][4], a2[8][4];
    uint32_t ah1[4][4];
    float logit_g, logit_g8;
};

// Where the forward pass reads its weights from: global memory (training,
// evaluation) or a CTA's shared-memory copy (indicator).
struct MLPView {
    const float *b1, *b2, *w3, *b3;
    const __nv_bfloat16 *W1, *W2;
};
__device__ __forceinline__ MLPView global_view(const MLPDev &w) {
    return MLPView{w.P + OFF_B1, w.P + OFF_B2, w.P + OFF_W3, w.P + OFF_B3, w.W1, w.W2};
}

__device__ __forceinline__ void mlp_forward_tile(const MLPView &w, const __nv_bfloat16 *xs, Fwd &f) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t ax[2][4];
#pragma unroll
    for (int kk = 0; kk < 2; ++kk) {
        ax[kk][0] = ld_pair(xs + g * NIN + 16 * kk + 2 * t);
        ax[kk][1] = ld_pair(xs + (g + 8) * NIN + 16 * kk + 2 * t);
        ax[kk][2] = ld_pair(xs + g * NIN + 16 * kk + 8 + 2 * t);
        ax[kk][3] = ld_pair(xs + (g + 8) * NIN + 16 * kk + 8 + 2 * t);
    }
    const float *b1 = w.b1, *b2 = w.b2, *w3 = w.w3;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float c0 = b1[8 * j + 2 * t], c1 = b1[8 * j + 2 * t + 1];
        f.a1[j][0] = c0;
        f.a1[j][1] = c1;
        f.a1[j][2] = c0;
        f.a1[j][3] = c1;
        const uint4 b = reinterpret_cast<const uint4 *>(w.W1)[j * 32 + lane];
        mma16816(f.a1[j], ax[0], b.x, b.y);
        mma16816(f.a1[j], ax[1], b.z, b.w);
    }
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float *a = f.a1[2 * kk + (q >> 1)] + 2 * (q & 1);
            const float2 h = gelu2(a[0], a[1]);
            f.ah1[kk][q] = pack_bf16(h.x, h.y);
        }
    }
    float sg = 0.f, sg8 = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float c0 = b2[8 * j + 2 * t], c1 = b2[8 * j + 2 * t + 1];
        f.a2[j][0] = c0;
        f.a2[j][1] = c1;
        f.a2[j][2] = c0;
        f.a2[j][3] = c1;
        const uint4 *bp = reinterpret_cast<const uint4 *>(w.W2) + (j * 32 + lane) * 2;
        const uint4 b01 = bp[0], b23 = bp[1];
        mma16816(f.a2[j], f.ah1[0], b01.x, b01.y);
        mma16816(f.a2[j], f.ah1[1], b01.z, b01.w);
        mma16816(f.a2[j], f.ah1[2], b23.x, b23.y);
        mma16816(f.a2[j], f.ah1[3], b23.z, b23.w);
        const float w0 = w3[8 * j + 2 * t], w1 = w3[8 * j + 2 * t + 1];
        const float2 h01 = gelu2(f.a2[j][0], f.a2[j][1]), h23 = gelu2(f.a2[j][2], f.a2[j][3]);
        sg = fmaf(h01.x, w0, fmaf(h01.y, w1, sg));
        sg8 = fmaf(h23.x, w0, fmaf(h23.y, w1, sg8));
    }
    sg += __shfl_xor_sync(0xffffffffu, sg, 1);
    sg += __shfl_xor_sync(0xffffffffu, sg, 2);
    sg8 += __shfl_xor_sync(0xffffffffu, sg8, 1);
    sg8 += __shfl_xor_sync(0xffffffffu, sg8, 2);
    const float b3 = *w.b3;
    f.logit_g = sg + b3;
    f.logit_g8 = sg8 + b3;
}

// The 16 features of one lane as BF16 into row (16 values, 16-byte aligned)
// of a tile's feature matrix: two 128-bit shared-memory stores.
__device__ __forceinline__ void store_features_bf16(__nv_bfloat16 *row, const float (&feat)[16]) {
    uint4 *d = reinterpret_cast<uint4 *>(row);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const float *f = feat + 8 * h;
        d[h] = make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]), pack_bf16(f[6], f[7]));
    }
}

__device__ __forceinline__ float sigmoidf_(float z) { return 1.0f / (1.0f + expf(-z)); }

// Copy the BF16 weights and the FP32 biases / output weights to shared memory
// (W1: NH*NIN, W2: NH*NH bf16; b: 3*NH+1 floats) with the threads of a CTA;
// the caller synchronises.  W1 and W2 must be 16-byte aligned.
__device__ __forceinline__ void stage_weights(const MLPDev &w, __nv_bfloat16 *sW1, __nv_bfloat16 *sW2, float *sb) {
    const uint4 *g1 = reinterpret_cast<const uint4 *>(w.W1), *g2 = reinterpret_cast<const uint4 *>(w.W2);
    uint4 *d1 = reinterpret_cast<uint4 *>(sW1), *d2 = reinterpret_cast<uint4 *>(sW2);
    for (int q = threadIdx.x; q < NH * NIN / 8; q += blockDim.x) d1[q] = g1[q];
    for (int q = threadIdx.x; q < NH * NH / 8; q += blockDim.x) d2[q] = g2[q];
    for (int q = threadIdx.x; q < NH; q += blockDim.x) {
        sb[q] = w.P[OFF_B1 + q];
        sb[NH + q] = w.P[OFF_B2 + q];
        sb[2 * NH + q] = w.P[OFF_W3 + q];
    }
    if (threadIdx.x == 0) sb[3 * NH] = w.P[OFF_B3];
}
__device__ __forceinline__ MLPView smem_view(const __nv_bfloat16 *sW1, const __nv_bfloat16 *sW2, const float *sb) {
    return MLPView{sb, sb + NH, sb + 2 * NH, sb + 3 * NH, sW1, sW2};
}

// ---- the network on the 5th-generation tensor cores (tcgen05) ----------------
// The indicator kernels run the network on groups of 64 elements with four
// warps (128 threads).  Layer l is one M = 128, N = 64 tcgen05.mma chain
// (K = 32 for layer 1, 64 for layer 2, 16 per instruction), BF16 operands from
// shared memory, FP32 accumulator in 64 tensor-memory columns.  The 64 elements
// are rows 0-63 of the A operand and again rows 64-127, so that the four warps
// share the epilogue: warps 0-1 read rows 0-63 and take hidden units 0-31,
// warps 2-3 read the same elements in rows 64-127 and take units 32-63 (a warp
// reads the tensor-memory lanes of its own sub-partition).  Layer 1's epilogue
// (bias, GELU, BF16) writes the layer-2 A operand; layer 2's (bias, GELU, dot
// with w3) leaves half a logit per thread, and the halves meet in shared memory.
//
// Operands are K-major without swizzling: 8 x 8 BF16 core matrices of 128 bytes,
// adjacent along K 128 bytes apart and along M / N (K / 8) * 128 bytes apart.
__host__ __device__ constexpr int core_off(int r, int k, int K) {
    return (r >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}
// The packed network in global memory (bytes): W1 [64 x 32] and W2 [64 x 64]
// as K-major B operands (rows = output units), then FP32 b1, b2, w3 and b3.
constexpr int TCP_W1 = 0, TCP_W2 = TCP_W1 + NH * NIN * 2, TCP_B1 = TCP_W2 + NH * NH * 2, TCP_B2 = TCP_B1 + NH * 4,
              TCP_W3 = TCP_B2 + NH * 4, TCP_B3 = TCP_W3 + NH * 4, TCP_BYTES = TCP_B3 + 16;
// Shared memory of the tcgen05 network (bytes from a 128-byte aligned base).
constexpr int TCS_A1 = 0;                                       // [128][32] BF16, layer-1 A
constexpr int TCS_A2 = TCS_A1 + 128 * NIN * 2;                  // [128][64] BF16, layer-2 A
constexpr int TCS_P = TCS_A2 + 128 * NH * 2;                    // the packed network
constexpr int TCS_PART = TCS_P + (TCP_BYTES + 127) / 128 * 128; // [64] float half logits
constexpr int TCS_PROB = TCS_PART + 64 * 4;                     // [64] float probabilities
constexpr int TCS_BAR = TCS_PROB + 64 * 4;                      // mbarriers: [0] weights copied, [1] MMAs done
constexpr int TCS_TMEM = TCS_BAR + 16;                          // TMEM address, timeout flag
constexpr int TCS_BYTES = TCS_TMEM + 16;
constexpr uint32_t TC_COLS = 64; // tensor-memory columns (layer 2 reuses layer 1's)

// Set-up by the 128 threads (tid < 128): barriers, the bulk copy of the packed
// network, and the tensor-memory allocation (warp 0).  Returns the TMEM address.
__device__ __forceinline__ uint32_t tc_begin(unsigned char *sm, const unsigned char *pack, int tid) {
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + TCS_BAR);
    uint32_t *tm = reinterpret_cast<uint32_t *>(sm + TCS_TMEM);
    if (tid == 0) {
        bw::mbar_init(&bar[0], 1);
        bw::mbar_init(&bar[1], 1);
        tm[1] = 0;
        bw::mbar_arrive_expect_tx(&bar[0], TCP_BYTES);
        bw::bulk_load(sm + TCS_P, pack, TCP_BYTES, &bar[0]);
    }
    if (tid < 32) bw::tmem_alloc(tm, TC_COLS);
    bw::tc_fence_before();
    bw::bar_sync(1, 128);
    bw::tc_fence_after();
    if (!bw::mbar_wait(&bar[0], 0)) tm[1] = 1; // the weights never arrived
    return tm[0];
}

// End of the tcgen05 network's use: after a timeout, give the MMAs still in
// flight a bounded time to finish; free the tensor memory (warp 0).  Returns
// true when a wait timed out.
__device__ __forceinline__ bool tc_end(unsigned char *sm, uint32_t tmem, uint32_t phase, int tid) {
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + TCS_BAR);
    volatile uint32_t *tm = reinterpret_cast<uint32_t *>(sm + TCS_TMEM);
    bw::tc_fence_before();
    bw::bar_sync(1, 128);
    const bool timed_out = tm[1] != 0;
    if (timed_out && phase > 0) bw::mbar_wait(&bar[1], (phase - 1) & 1);
    bw::tc_fence_after();
    if (tid < 32) bw::tmem_dealloc(tmem, TC_COLS);
    return timed_out;
}

// The 16 features of one lane as BF16 into rows r and r + 64 of the layer-1 A
// operand: K columns 16 half .. 16 half + 15 (density half 0, pressure half 1).
__device__ __forceinline__ void store_features_tc(unsigned char *sm, int r, int half, const float (&feat)[16]) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const float *f = feat + 8 * h;
        const uint4 v = make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]),
                                   pack_bf16(f[6], f[7]));
        const int k = 16 * half + 8 * h;
        *reinterpret_cast<uint4 *>(sm + TCS_A1 + core_off(r, k, NIN)) = v;
        *reinterpret_cast<uint4 *>(sm + TCS_A1 + core_off(r + 64, k, NIN)) = v;
    }
}

// Forward pass of the 64 elements whose features are in A1 (all 128 threads
// call it).  Leaves sigmoid(logit) of row r in TCS_PROB[r]; `phase` counts
// the MMA-barrier phases used so far.  Returns false after a timed-out wait
// (the timeout flag is set).
__device__ __forceinline__ bool mlp_tc_forward64(unsigned char *sm, uint32_t tmem, uint32_t &phase, int tid) {
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + TCS_BAR);
    volatile uint32_t *flag = reinterpret_cast<uint32_t *>(sm + TCS_TMEM) + 1;
    const float *b1 = reinterpret_cast<const float *>(sm + TCS_P + TCP_B1);
    const float *b2 = reinterpret_cast<const float *>(sm + TCS_P + TCP_B2);
    const float *w3 = reinterpret_cast<const float *>(sm + TCS_P + TCP_W3);
    float *part = reinterpret_cast<float *>(sm + TCS_PART), *prob = reinterpret_cast<float *>(sm + TCS_PROB);
    const uint32_t a1 = bw::smem_addr(sm + TCS_A1), a2 = bw::smem_addr(sm + TCS_A2);
    const uint32_t w1 = bw::smem_addr(sm + TCS_P + TCP_W1), w2 = bw::smem_addr(sm + TCS_P + TCP_W2);
    constexpr uint32_t ID = bw::idesc_bf16_f32(128, NH);
    const int warp = tid >> 5, lane = tid & 31;
    const int r = (32 * warp + lane) & 63, cb = warp < 2 ? 0 : 32;
    const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
    // ---- layer 1: D = A1 W1^T --------------------------------------------------
    bw::fence_async_smem(); // A1 (written by this thread) -> the MMA's async proxy
    bw::tc_fence_before();
    bw::bar_sync(1, 128);
    if (*flag) return false;
    if (tid == 0) {
        bw::tc_fence_after();
#pragma unroll
        for (int s = 0; s < NIN / 16; ++s)
            bw::mma_bf16(tmem, bw::smem_desc_kmajor(a1 + 256 * s, 128, NIN / 8 * 128),
                         bw::smem_desc_kmajor(w1 + 256 * s, 128, NIN / 8 * 128), ID, s > 0);
        bw::mma_commit(&bar[1]);
    }
    if (!bw::mbar_wait(&bar[1], phase & 1)) *flag = 1;
    ++phase;
    bw::tc_fence_after();
    float v[32];
    bw::tmem_ld32(trow + cb, v);
    // h1 = gelu(a1 + b1) as BF16 into rows r and r + 64, K columns cb .. cb + 31 of A2
#pragma unroll
    for (int c = 0; c < 32; c += 8) {
        uint32_t q[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            const float2 g = gelu2(v[c + 2 * h] + b1[cb + c + 2 * h], v[c + 2 * h + 1] + b1[cb + c + 2 * h + 1]);
            q[h] = pack_bf16(g.x, g.y);
        }
        const uint4 o = make_uint4(q[0], q[1], q[2], q[3]);
        *reinterpret_cast<uint4 *>(sm + TCS_A2 + core_off(r, cb + c, NH)) = o;
        *reinterpret_cast<uint4 *>(sm + TCS_A2 + core_off(r + 64, cb + c, NH)) = o;
    }
    // ---- layer 2: D = A2 W2^T, over the same columns once every thread has read them
    bw::fence_async_smem();
    bw::tc_fence_before();
    bw::bar_sync(1, 128);
    if (*flag) return false;
    if (tid == 0) {
        bw::tc_fence_after();
#pragma unroll
        for (int s = 0; s < NH / 16; ++s)
            bw::mma_bf16(tmem, bw::smem_desc_kmajor(a2 + 256 * s, 128, NH / 8 * 128),
                         bw::smem_desc_kmajor(w2 + 256 * s, 128, NH / 8 * 128), ID, s > 0);
        bw::mma_commit(&bar[1]);
    }
    if (!bw::mbar_wait(&bar[1], phase & 1)) *flag = 1;
    ++phase;
    bw::tc_fence_after();
    bw::tmem_ld32(trow + cb, v);
    float sg = 0.f;
#pragma unroll
    for (int c = 0; c < 32; c += 2) {
        const float2 g = gelu2(v[c] + b2[cb + c], v[c + 1] + b2[cb + c + 1]);
        sg = fmaf(g.x, w3[cb + c], fmaf(g.y, w3[cb + c + 1], sg));
    }
    if (warp >= 2) part[r] = sg;
    bw::tc_fence_before();
    bw::bar_sync(1, 128);
    if (warp < 2) prob[r] = 1.0f / (1.0f + expf(-(sg + part[r] + *reinterpret_cast<const float *>(sm + TCS_P + TCP_B3))));
    bw::bar_sync(1, 128);
    return *flag == 0;
}

// ---- features and decisions of the 2D indicator (np = 4) ------------------
// 1D inverse Vandermonde matrix of deg 3 (iV1[i][k]); the tensor inverse of
// FRPSpace2D (src/struct.jl:196-205) factors as iV[(i,j)][(k,l)] = iV1[i][k] iV1[j][l].
struct IV1 {
    float m[4][4];
};

// Normalised modal energies of one field from its 16 point values v[k + 4 l]:
// feat[a] = clamp(log10(u_hat_a^2 / sum u_hat^2 + 1e-16), -16, 0) / 8 + 1 (0 when
// !valid), and su = u_hat_15^2 / sum u_hat^2 (the plain test's ratio).
__device__ __forceinline__ void modal_features16(const float (&v)[16], bool valid, const IV1 &iv, float (&feat)[16],
                                                 float &su) {
    // modal coefficients by sum factorisation: t[i][l] = sum_k iV1[i][k] v[k + 4 l],
    // u_hat[4 i + j] = sum_l iV1[j][l] t[i][l]
    float t[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            float s = iv.m[i][0] * v[4 * l];
#pragma unroll
            for (int k = 1; k < 4; ++k) s = fmaf(iv.m[i][k], v[k + 4 * l], s);
            t[i][l] = s;
        }
    float tot = 0.f;
    float en[16];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float s = iv.m[j][0] * t[i][0];
#pragma unroll
            for (int l = 1; l < 4; ++l) s = fmaf(iv.m[j][l], t[i][l], s);
            en[4 * i + j] = s * s;
            tot += s * s;
        }
    su = en[15] / tot;
    const float itot = 1.0f / tot;
#pragma unroll
    for (int a = 0; a < 16; ++a) {
        float x = __log2f(en[a] * itot + 1e-16f) * 0.30102999566398120f; // log10 through the hardware log2
        x = fminf(fmaxf(x, -16.f), 0.f);
        feat[a] = valid ? x * 0.125f + 1.0f : 0.f;
    }
}

// Pressure of a conserved 2D Euler state, as the indicator's features see it.
__device__ __forceinline__ float feature_pressure(float w0, float w1, float w2, float w3, float gm1) {
    const float ri = __fdividef(1.0f, w0);
    return gm1 * (w3 - 0.5f * (w1 * (w1 * ri) + w2 * (w2 * ri)));
}

// Features of the element shared by lanes L and L + 16 of a warp: each holds the
// four variables w[k][m] at 8 of its 16 points (the lower lane points 0-7, the
// upper 8-15, in the order q = k + 4 l); they swap halves so that the lower lane
// gets the density features, the upper lane the pressure features.  Lanes of
// elements past the end (valid false) take part in the exchange.
__device__ __forceinline__ void features_from_raw(const float (&w)[8][4], bool valid, bool pressure, const IV1 &iv,
                                                  float gm1, float (&feat)[16], float &su) {
    float v[16];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const float w0 = w[k][0], w1 = w[k][1], w2 = w[k][2], w3 = w[k][3];
        const float pk = feature_pressure(w0, w1, w2, w3, gm1);
        const float recv = __shfl_xor_sync(0xffffffffu, pressure ? w0 : pk, 16);
        v[k] = pressure ? recv : w0;     // density (lower) / pressure (upper) at point k
        v[8 + k] = pressure ? pk : recv; // ... at point 8 + k
    }
    modal_features16(v, valid, iv, feat, su);
}

// Where the modal decay leaves no doubt, below the plain test's sigma = 1 region
// (Se = log10 su < S0 - kappa: smooth, with more than a decade of margin to the
// plain decision at Se = S0 - 0.87 kappa), the learned indicator takes the element
// as smooth without consulting the network; the network decides everywhere else.
__device__ __forceinline__ bool below_floor(float su, float S0, float kappa) { return log10f(su) < S0 - kappa; }

// The plain modal-decay test (shock_detector, src/dissipation.jl:13-23) in FP32.
__device__ __forceinline__ bool plain_troubled(float su, float S0, float kappa) {
    const float Se = log10f(su);
    float sigma;
    if (Se < S0 - kappa)
        sigma = 1.f;
    else if (S0 - kappa <= Se && Se < S0 + kappa)
        sigma = 0.5f * (1.f - sinf(1.5707963267948966f * (Se - S0) / kappa));
    else
        sigma = 0.f;
    return sigma < 0.99f;
}

// :l2 modal filter of the elements ebase + b for the bits b set in todo (b < 16;
// the same mask on every lane), one element at a time by the whole warp: lane =
// 16 (variable pair) + mode a.  State in the 2D device layout (np = 4, 16
// points, 4 variables); lo (FP32K low part, may be null) is cleared where u is
// filtered.
// Every output is the same ascending FMA chain as the plain filter kernel's.
template <class Real>
__device__ __forceinline__ void warp_filter_elements(unsigned todo, size_t ebase, Real *u, Real *lo, size_t ne,
                                                     const Real *V, const Real *iV, double lam) {
    const int lane = threadIdx.x & 31, a = lane & 15, half = lane & 16;
    const Real den = Real(1) + mul_rn(Real(lam), Real((double)((a + 1) * (a + 1) * a * a)));
    while (todo) {
        const int src = __ffs(todo) - 1;
        todo &= todo - 1;
        const size_t et = ebase + src;
        for (int mp = 0; mp < 4; mp += 2) {
            const int m = mp + (half >> 4);
            const size_t at = frk::e2d_index(et, a, m, ne);
            const Real xa = u[at];
            Real s = iV[a] * __shfl_sync(0xffffffffu, xa, half);
#pragma unroll
            for (int b = 1; b < 16; ++b)
                s = frk::fmaR<Real>(iV[a + 16 * b], __shfl_sync(0xffffffffu, xa, half + b), s);
            const Real ha = s / den;
            Real r = V[a] * __shfl_sync(0xffffffffu, ha, half);
#pragma unroll
            for (int b = 1; b < 16; ++b)
                r = frk::fmaR<Real>(V[a + 16 * b], __shfl_sync(0xffffffffu, ha, half + b), r);
            u[at] = r;
            if (lo) lo[at] = Real(0);
        }
    }
}

} // namespace frmlp
