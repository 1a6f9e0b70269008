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

namespace frmlp {

constexpr int NIN = 32, NH = 64;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NIN, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NH, NPARAM = OFF_B3 + 1;
constexpr int WARPS = 4;  // warps per CTA of the forward and indicator kernels
constexpr int GWARPS = 2; // warps per CTA of the gradient kernel (static shared memory < 48 KB)

struct MLPDev {
    const float *P;             // FP32 parameters
    const __nv_bfloat16 *W1;    // [64][32]
    const __nv_bfloat16 *W2;    // [64][64]  row = output unit
    const __nv_bfloat16 *W2T;   // [64][64]  row = input unit
};

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
        const __nv_bfloat16 *row = w.W1 + (8 * j + g) * NIN;
#pragma unroll
        for (int kk = 0; kk < 2; ++kk) mma16816(f.a1[j], ax[kk], ld_pair(row + 16 * kk + 2 * t), ld_pair(row + 16 * kk + 8 + 2 * t));
    }
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
        f.ah1[kk][0] = pack_bf16(gelu(f.a1[2 * kk][0]), gelu(f.a1[2 * kk][1]));
        f.ah1[kk][1] = pack_bf16(gelu(f.a1[2 * kk][2]), gelu(f.a1[2 * kk][3]));
        f.ah1[kk][2] = pack_bf16(gelu(f.a1[2 * kk + 1][0]), gelu(f.a1[2 * kk + 1][1]));
        f.ah1[kk][3] = pack_bf16(gelu(f.a1[2 * kk + 1][2]), gelu(f.a1[2 * kk + 1][3]));
    }
    float sg = 0.f, sg8 = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float c0 = b2[8 * j + 2 * t], c1 = b2[8 * j + 2 * t + 1];
        f.a2[j][0] = c0;
        f.a2[j][1] = c1;
        f.a2[j][2] = c0;
        f.a2[j][3] = c1;
        const __nv_bfloat16 *row = w.W2 + (8 * j + g) * NH;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
            mma16816(f.a2[j], f.ah1[kk], ld_pair(row + 16 * kk + 2 * t), ld_pair(row + 16 * kk + 8 + 2 * t));
        const float w0 = w3[8 * j + 2 * t], w1 = w3[8 * j + 2 * t + 1];
        sg = fmaf(gelu(f.a2[j][0]), w0, fmaf(gelu(f.a2[j][1]), w1, sg));
        sg8 = fmaf(gelu(f.a2[j][2]), w0, fmaf(gelu(f.a2[j][3]), w1, sg8));
    }
    sg += __shfl_xor_sync(0xffffffffu, sg, 1);
    sg += __shfl_xor_sync(0xffffffffu, sg, 2);
    sg8 += __shfl_xor_sync(0xffffffffu, sg8, 1);
    sg8 += __shfl_xor_sync(0xffffffffu, sg8, 2);
    const float b3 = *w.b3;
    f.logit_g = sg + b3;
    f.logit_g8 = sg8 + b3;
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

} // namespace frmlp
