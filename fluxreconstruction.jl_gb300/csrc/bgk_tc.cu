// bgk_tc.cu -- FP32 1D1V BGK residual + SSPRK3 stage (mol! of example/bgk_wave.jl:69-129)
// with the transport term on the tensor cores.
//
// For a fixed velocity v the kinetic upwind transport of element i is linear
// in the point values of elements i-1, i, i+1:
//   v > 0:  du_m = -v [ sum_k (D_mk - dgl_m ll_k) u_k(i)/J_i + sum_k dgl_m lr_k u_k(i-1)/J_(i-1) ]
//   v <= 0: du_m = -v [ sum_k (D_mk - dgr_m lr_k) u_k(i)/J_i + sum_k dgr_m ll_k u_k(i+1)/J_(i+1) ]
// (the interface flux is the right trace of the upwind neighbour, heaviside(v) at
// bgk_wave.jl:26,103-107, and the correction of :122-128).  A tile of EB
// consecutive elements (EB * np <= 16 output rows) is therefore one block-banded
// [16 x 8 KS] operator A (per velocity sign, the same for every tile) times the
// [8 KS x 8] panel of u / J of elements i0-1 .. i0+EB at 8 velocities: an
// m16n8k8 TF32 MMA chain.  FP32 accuracy is kept with the three-term TF32 split
//   A B ~= Ab Bb + Ab Bs + As Bb,  X = Xb + Xs,  Xb = tf32(X), Xs = tf32(X - Xb)
// (the split product of Ootomo and Yokota, "Recovering single precision accuracy
// from Tensor Cores while surpassing the FP32 theoretical peak performance", 2022).
// The A fragments of both signs, split, are built once per problem on the host.
// A second form (k_bgk1d_umma, FRGPU_OPT_BGK_TENSOR = 2) runs the same split
// product on the 5th-generation tensor cores, 128 velocities per CTA; it adds
// the same terms in the same order and gives the same bits, but on the 512-
// velocity workload it has 4x fewer, longer-lived CTAs whose load -> MMA ->
// epilogue chain the SM cannot overlap, and takes 74 against 52 us per step.
//
// The BGK collision term (M - u)/tau needs the moments (rho, rho U, E) of every
// (element, point) over all velocities and conserve_prim at gamma = 3
// (bgk_wave.jl:76-81).  A first kernel computes them, one warp per (element,
// point) row with double-float partial sums, and stores (rho, U, lambda).  The
// transport kernel then runs one warp per tile of EB elements x 8 velocities.
//
// Layout: internal u[(i * np + k) * nvel + v] (velocity fastest).
#include <cmath>
#include <cstring>
#include <vector>

#include "blackwell.cuh"
#include "fr_stage.cuh"
#include "frgpu_internal.h"

using namespace frk;

namespace {

constexpr int TCW = 4; // warps per CTA of the transport kernel (each one 8-velocity tile)
constexpr int MW = 8;  // warps per CTA of the moments kernel (each one row)

// Tile geometry for np points per element (host and device).
struct BTile {
    int EB, ROWS, KR, KS;
};
__host__ __device__ constexpr BTile btile(int np) {
    return BTile{16 / np, (16 / np) * np, (16 / np + 2) * np, ((16 / np + 2) * np + 7) / 8};
}
constexpr int KS_MAX = 4;                        // np = 5: KR = 25 -> 4 k-steps
constexpr int FRAG_WORDS = 2 * 2 * KS_MAX * 32 * 4; // [sign][big/small][ks][lane][4]

__device__ __forceinline__ uint32_t tf32_of(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// D += A (16x8, row) * B (8x8, col), TF32 in, FP32 accumulate
__device__ __forceinline__ void mma1688(float (&d)[4], const uint4 &a, uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a.x), "r"(a.y), "r"(a.z), "r"(a.w), "r"(b0), "r"(b1));
}

__device__ __forceinline__ int wrapn(int i, int n) { return ((i % n) + n) % n; }

// Knuth's TwoSum accumulation of x into the pair (s, e).
__device__ __forceinline__ void acc2(float &s, float &e, float x) {
    const float t = __fadd_rn(s, x);
    const float bp = __fsub_rn(t, s);
    e = __fadd_rn(e, __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(x, bp)));
    s = t;
}

// ---- moments -> (rho, U, lambda) per (element, point) row -------------------
template <int NP>
__global__ void __launch_bounds__(32 * MW) k_bgk_moments(const float *__restrict__ uin, const float *__restrict__ din,
                                                        const float *__restrict__ velo, const float *__restrict__ w,
                                                        int ne, int nv, float *__restrict__ prim, int *status,
                                                        int closure, double a_adv) {
    FR_PDL_ENTRY();
    const int row = blockIdx.x * MW + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (row >= ne * NP) return; // whole warp
    const size_t base = (size_t)row * nv;
    float s0 = 0.f, e0 = 0.f, s1 = 0.f, e1 = 0.f, s2 = 0.f, e2 = 0.f;
#pragma unroll 4
    for (int v = lane; v < nv; v += 32) {
        const float x = ld_state(uin, din, base + v);
        const float vel = __ldg(velo + v), wx = __ldg(w + v) * x;
        acc2(s0, e0, wx);
        acc2(s1, e1, wx * vel);
        acc2(s2, e2, (wx * vel) * vel);
    }
    double m0 = (double)s0 + (double)e0, m1 = (double)s1 + (double)e1, m2 = (double)s2 + (double)e2;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        m0 += __shfl_xor_sync(0xffffffffu, m0, off);
        m1 += __shfl_xor_sync(0xffffffffu, m1, off);
        m2 += __shfl_xor_sync(0xffffffffu, m2, off);
    }
    if (lane == 0) {
        // closure 0: conserve_prim(w, gamma = 3), 1D: U = m/rho, lambda = rho / (4 (E - m^2 / (2 rho))),
        // E = m2 / 2; closure 1: prim = [rho, a, 1]
        const double U = closure ? a_adv : m1 / m0;
        const double lam = closure ? 1.0 : 0.25 * m0 / (0.5 * m2 - 0.5 * m1 * U);
        prim[3 * row] = (float)m0;
        prim[3 * row + 1] = (float)U;
        prim[3 * row + 2] = (float)lam;
        if (!(m0 > 0.0) || !(lam > 0.0)) atomicOr(status, ST_UNPHYSICAL);
    }
}

// ---- transport on the tensor cores + relaxation + stage ----------------------
struct TCArgs {
    int ne, nvel;
    const float *uin, *din, *un;
    float *out, *ul;
    const double *dtp;
    const float *J;
    const float *velo;
    const float *prim;
    const uint4 *frag; // [sign][big/small][ks][lane] (4 words each)
    const uint32_t *uop; // tcgen05 B operands: [sign][big/small][UN x K core layout]
    float tau;
    int *status;
};

// ---- the same tile product on the 5th-generation tensor cores (tcgen05) ------
// One CTA of 128 threads per tile of EB elements x UM = 128 velocities, the
// product transposed so that velocities run along M:
//   D[v][r] = sum_kk P[v][kk] A[r][kk],  P[v][kk] = u_k(e) / J_e (e = i0 + kk / np - 1, k = kk % np),
// one tcgen05.mma.kind::tf32 chain per velocity sign present in the tile (M = 128,
// N = UN = 16 tile rows, K = 8 per instruction over the tile's 8 KS source rows),
// with the three-term split P A ~ Pb As + Ps Ab + Pb Ab; FP32 accumulators in
// tensor-memory columns 16 s .. 16 s + 15.  Thread t owns velocity v0 + t: it
// builds row t of P (big and small parts) in shared memory, and reads back row t
// of D (its warp's own tensor-memory lanes) for the epilogue.  Operands are
// K-major without swizzling: 8 x 4 TF32 core matrices of 128 bytes, adjacent
// along K 128 bytes apart and along M / N (K / 4) * 128 bytes apart.
constexpr int UM = 128, UN = 16, UK_MAX = 8 * KS_MAX;
constexpr int UT = 4 * UM; // threads per CTA: four per velocity in the epilogue
constexpr int UOP_WORDS = 4 * UN * UK_MAX;
__host__ __device__ constexpr int ucore(int r, int k, int K) {
    return (r >> 3) * (K / 4) * 32 + (k >> 2) * 32 + (r & 7) * 4 + (k & 3); // 4-byte words
}

template <int NP, int STAGE>
__global__ void __launch_bounds__(UT) k_bgk1d_umma(const TCArgs a) {
    FR_PDL_ENTRY();
    constexpr BTile T = btile(NP);
    constexpr int K = 8 * T.KS;
    constexpr int RG = (T.ROWS + 3) / 4; // rows per warp group in the epilogue
    static_assert(T.ROWS <= UN && K <= UK_MAX, "tile larger than the tcgen05 operands");
    __shared__ __align__(1024) uint32_t s_pb[UM * K];
    __shared__ __align__(1024) uint32_t s_ps[UM * K];
    __shared__ __align__(128) uint32_t s_op[4 * UN * K];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ uint32_t s_tm;
    const int tid = threadIdx.x, warp = tid >> 5, grp = tid / UM;
    const int ne = a.ne, nv = a.nvel;
    const int i0 = blockIdx.x * T.EB;
    // P: thread (grp, t) builds the K chunks grp, grp + 4, ... of row t (velocity v0 + t)
    {
        const int t = tid % UM, v = blockIdx.y * UM + t;
        const bool v_ok = v < nv;
        for (int c = grp; c < K / 4; c += 4) {
            uint32_t hb[4], hs[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int k2 = 4 * c + j;
                float x = 0.f;
                if (v_ok && k2 < T.KR) {
                    const int e = wrapn(i0 + k2 / NP - 1, ne);
                    x = ld_state(a.uin, a.din, ((size_t)e * NP + k2 % NP) * nv + v) / __ldg(a.J + e);
                }
                hb[j] = tf32_of(x);
                hs[j] = tf32_of(x - __uint_as_float(hb[j]));
            }
            *reinterpret_cast<uint4 *>(s_pb + ucore(t, 4 * c, K)) = make_uint4(hb[0], hb[1], hb[2], hb[3]);
            *reinterpret_cast<uint4 *>(s_ps + ucore(t, 4 * c, K)) = make_uint4(hs[0], hs[1], hs[2], hs[3]);
        }
    }
    for (int q = tid; q < 4 * UN * K; q += UT) s_op[q] = __ldg(a.uop + q);
    // the epilogue's velocity: warp w reads tensor-memory lanes 32 (w % 4) ..
    const int v = blockIdx.y * UM + 32 * (warp & 3) + (tid & 31);
    const bool v_ok = v < nv;
    const float vel = v_ok ? __ldg(a.velo + v) : 0.f;
    if (tid == 0) bw::mbar_init(&s_bar, 1);
    if (warp == 0) bw::tmem_alloc(&s_tm, 32);
    bw::fence_async_smem(); // P and the operator (written by this thread) -> the MMA's async proxy
    bw::tc_fence_before();
    const int any_pos = __syncthreads_or(v_ok && vel > 0.f);
    const int any_neg = __syncthreads_or(v_ok && !(vel > 0.f));
    bw::tc_fence_after();
    const uint32_t tmem = s_tm;
    if (tid == 0) {
        constexpr uint32_t ID = bw::idesc_tf32_f32(UM, UN);
        constexpr uint32_t SBO = (K / 4) * 128;
        const uint32_t pb = bw::smem_addr(s_pb), ps = bw::smem_addr(s_ps), op = bw::smem_addr(s_op);
#pragma unroll
        for (int sg = 0; sg < 2; ++sg) {
            if (!(sg == 1 ? any_pos : any_neg)) continue;
            const uint32_t d = tmem + 16 * sg;
            const uint32_t ob = op + (uint32_t)((sg * 2 + 0) * UN * K * 4), os = op + (uint32_t)((sg * 2 + 1) * UN * K * 4);
#pragma unroll
            for (int ks = 0; ks < T.KS; ++ks) {
                const uint32_t off = 256 * ks; // two core matrices (K = 8) per instruction
                bw::mma_tf32(d, bw::smem_desc_kmajor(pb + off, 128, SBO), bw::smem_desc_kmajor(os + off, 128, SBO), ID,
                             ks > 0);
                bw::mma_tf32(d, bw::smem_desc_kmajor(ps + off, 128, SBO), bw::smem_desc_kmajor(ob + off, 128, SBO), ID,
                             true);
                bw::mma_tf32(d, bw::smem_desc_kmajor(pb + off, 128, SBO), bw::smem_desc_kmajor(ob + off, 128, SBO), ID,
                             true);
            }
        }
        bw::mma_commit(&s_bar);
    }
    const bool done = bw::mbar_wait(&s_bar, 0);
    bw::tc_fence_after();
    int bad = 0;
    if (done) {
        float acc[32];
        bw::tmem_ld32(tmem + ((uint32_t)(32 * (warp & 3)) << 16), acc);
        const float dt = (float)(*a.dtp);
        const float pi_inv = 0.31830988618379067154f, itau = 1.0f / a.tau;
        const int sg = vel > 0.f ? 1 : 0;
#pragma unroll
        for (int q = 0; q < RG; ++q) {
            const int r = RG * (warp >> 2) + q;
            const int e = i0 + r / NP, m = r % NP;
            if (r >= T.ROWS || e >= ne || !v_ok) continue;
            const float tr = sg ? acc[16 + r] : acc[r];
            const size_t idx = ((size_t)e * NP + m) * nv + v;
            const float u = ld_state(a.uin, a.din, idx);
            const float *pr = a.prim + 3 * ((size_t)e * NP + m);
            const float rho = __ldg(pr), U = __ldg(pr + 1), lam = __ldg(pr + 2);
            const float dv = vel - U;
            const float M = rho * sqrtf(lam * pi_inv) * expf(-lam * dv * dv);
            const float du = fmaf(-vel, tr, (M - u) * itau);
            const float res = stage_update<float, MODE_FP32K, STAGE>(du, u, dt, idx, a.un, a.uin, a.din, a.out, a.ul);
            if (!isfinite(res)) bad |= ST_NONFINITE;
        }
    } else {
        bad |= ST_TIMEOUT;
        bw::mbar_wait(&s_bar, 0); // a bounded second wait for the MMAs still in flight
    }
    bw::tc_fence_before();
    __syncthreads();
    bw::tc_fence_after();
    if (warp == 0) bw::tmem_dealloc(tmem, 32);
    if (bad) atomicOr(a.status, bad);
}

template <int NP, int STAGE>
__global__ void __launch_bounds__(32 * TCW) k_bgk1d_tc(const TCArgs a) {
    FR_PDL_ENTRY();
    constexpr BTile T = btile(NP);
    const int ne = a.ne, nv = a.nvel;
    const int i0 = blockIdx.x * T.EB;
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int n0 = (blockIdx.y * TCW + (threadIdx.x >> 5)) * 8;
    if (n0 >= nv) return; // whole warp
    const int vb = n0 + g; // this lane's B column
    const bool vb_ok = vb < nv;
    const float velb = vb_ok ? __ldg(a.velo + vb) : 0.f;
    const unsigned pos = __ballot_sync(0xffffffffu, !vb_ok || velb > 0.f);
    const unsigned neg = __ballot_sync(0xffffffffu, !vb_ok || !(velb > 0.f));
    const bool all_pos = pos == 0xffffffffu, all_neg = neg == 0xffffffffu;
    float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
    for (int ks = 0; ks < T.KS; ++ks) {
        uint32_t bb[2], bs[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int kk = 8 * ks + t + 4 * h;
            float x = 0.f;
            if (vb_ok && kk < T.KR) {
                const int e = wrapn(i0 + kk / NP - 1, ne);
                x = ld_state(a.uin, a.din, ((size_t)e * NP + kk % NP) * nv + vb) / __ldg(a.J + e);
            }
            bb[h] = tf32_of(x);
            bs[h] = tf32_of(x - __uint_as_float(bb[h]));
        }
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            if (s == 1 ? all_neg : all_pos) continue; // no column of this sign in the tile
            const uint4 ab = __ldg(a.frag + ((s * 2 + 0) * KS_MAX + ks) * 32 + lane);
            const uint4 as = __ldg(a.frag + ((s * 2 + 1) * KS_MAX + ks) * 32 + lane);
            mma1688(acc[s], as, bb[0], bb[1]);
            mma1688(acc[s], ab, bs[0], bs[1]);
            mma1688(acc[s], ab, bb[0], bb[1]);
        }
    }
    // epilogue: rows g, g+8; velocities n0 + 2t, n0 + 2t + 1
    const float dt = (float)(*a.dtp);
    const float pi_inv = 0.31830988618379067154f, itau = 1.0f / a.tau;
    int bad = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int r = g + 8 * (q >> 1), v = n0 + 2 * t + (q & 1);
        const int e = i0 + r / NP, m = r % NP;
        if (r >= T.ROWS || e >= ne || v >= nv) continue;
        const float vel = __ldg(a.velo + v);
        const float tr = vel > 0.f ? acc[1][q] : acc[0][q];
        const size_t idx = ((size_t)e * NP + m) * nv + v;
        const float u = ld_state(a.uin, a.din, idx);
        const float *pr = a.prim + 3 * ((size_t)e * NP + m);
        const float rho = __ldg(pr), U = __ldg(pr + 1), lam = __ldg(pr + 2);
        const float dv = vel - U;
        const float M = rho * sqrtf(lam * pi_inv) * expf(-lam * dv * dv);
        const float du = fmaf(-vel, tr, (M - u) * itau);
        const float res = stage_update<float, MODE_FP32K, STAGE>(du, u, dt, idx, a.un, a.uin, a.din, a.out, a.ul);
        if (!isfinite(res)) bad |= ST_NONFINITE;
    }
    if (bad) atomicOr(a.status, bad);
}

// TF32 rounding of x (round to nearest, ties away from zero, as cvt.rna.tf32.f32).
uint32_t tf32_host(float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    const uint32_t sign = b & 0x80000000u, mag = b & 0x7fffffffu;
    if (mag >= 0x7f800000u) return b; // inf / nan
    return sign | ((mag + 0x1000u) & 0xffffe000u);
}

template <int NP>
int launch_tc(frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    if (p->prepare_only) return FRGPU_OK;
    constexpr BTile T = btile(NP);
    const int ne = p->sp.nx, nv = p->d.nvel;
    const float *uin = (const float *)in, *dn = (const float *)din;
    FR_CUDA(fr_launch_opt(false, k_bgk_moments<NP>, (ne * NP + MW - 1) / MW, 32 * MW, 0, p->stream,
        uin, dn, (const float *)p->d_velo, (const float *)p->d_w, ne, nv, p->d_bgk_prim, p->d_status, p->bgk_closure,
        p->d.a));
    FR_CUDA(cudaGetLastError());
    TCArgs a;
    a.ne = ne;
    a.nvel = nv;
    a.uin = uin;
    a.din = dn;
    a.un = (const float *)p->s0;
    a.out = (float *)out;
    a.ul = (float *)p->s3;
    a.dtp = p->d_dt;
    a.J = (const float *)p->d_J;
    a.velo = (const float *)p->d_velo;
    a.prim = p->d_bgk_prim;
    a.frag = reinterpret_cast<const uint4 *>(p->d_bgk_frag);
    a.uop = p->d_bgk_frag + FRAG_WORDS;
    a.tau = (float)p->d.tau;
    a.status = p->d_status;
    if (p->bgk_tensor == 2) {
        const dim3 ug((ne + T.EB - 1) / T.EB, (nv + UM - 1) / UM);
        switch (stage) {
        case 0: FR_CUDA(fr_launch_opt(false, k_bgk1d_umma<NP, 0>, ug, UT, 0, p->stream, a)); break;
        case 1: FR_CUDA(fr_launch_opt(false, k_bgk1d_umma<NP, 1>, ug, UT, 0, p->stream, a)); break;
        case 2: FR_CUDA(fr_launch_opt(false, k_bgk1d_umma<NP, 2>, ug, UT, 0, p->stream, a)); break;
        case 3: FR_CUDA(fr_launch_opt(false, k_bgk1d_umma<NP, 3>, ug, UT, 0, p->stream, a)); break;
        default: fr_set_error("BGK residual: bad stage"); return FRGPU_ERR_ARG;
        }
        FR_CUDA(cudaGetLastError());
        p->launches += 2;
        return FRGPU_OK;
    }
    const dim3 grid((ne + T.EB - 1) / T.EB, (nv + 8 * TCW - 1) / (8 * TCW));
    switch (stage) {
    case 0: FR_CUDA(fr_launch_opt(false, k_bgk1d_tc<NP, 0>, grid, 32 * TCW, 0, p->stream, a)); break;
    case 1: FR_CUDA(fr_launch_opt(false, k_bgk1d_tc<NP, 1>, grid, 32 * TCW, 0, p->stream, a)); break;
    case 2: FR_CUDA(fr_launch_opt(false, k_bgk1d_tc<NP, 2>, grid, 32 * TCW, 0, p->stream, a)); break;
    case 3: FR_CUDA(fr_launch_opt(false, k_bgk1d_tc<NP, 3>, grid, 32 * TCW, 0, p->stream, a)); break;
    default: fr_set_error("BGK residual: bad stage"); return FRGPU_ERR_ARG;
    }
    FR_CUDA(cudaGetLastError());
    p->launches += 2;
    return FRGPU_OK;
}

} // namespace

// The J-free transport operator of a tile, per velocity sign s (1: v > 0, 0: v <= 0):
// row r = (el, m), source row kk = (es, k) with es = kk / np - 1 the element offset;
// Mc couples an element to itself, Mn to its upwind neighbour (left for v > 0,
// right for v <= 0).  Stored as the lanes' m16n8k8 A fragments:
// a0 = A[g][8ks+t], a1 = A[g+8][8ks+t], a2 = A[g][8ks+t+4], a3 = A[g+8][8ks+t+4],
// g = lane / 4, t = lane % 4, split into TF32 big and small parts.
int fr_bgk_tc_setup(frgpu_problem *p) {
    const frgpu_space &s = p->sp;
    const int np = s.np;
    const BTile T = btile(np);
    auto A = [&](int sg, int r, int kk) -> double {
        if (r >= T.ROWS || kk >= T.KR) return 0.0;
        const int el = r / np, m = r % np, es = kk / np - 1, k = kk % np;
        const int up = sg == 1 ? el - 1 : el + 1;
        const double D = s.dl[m + np * k];
        if (es == el) return sg == 1 ? D - s.dhl[m] * s.ll[k] : D - s.dhr[m] * s.lr[k];
        if (es == up) return sg == 1 ? s.dhl[m] * s.lr[k] : s.dhr[m] * s.ll[k];
        return 0.0;
    };
    std::vector<uint32_t> frag(FRAG_WORDS, 0u);
    for (int sg = 0; sg < 2; ++sg)
        for (int ks = 0; ks < T.KS; ++ks)
            for (int lane = 0; lane < 32; ++lane) {
                const int g = lane / 4, t = lane % 4;
                const int rr[4] = {g, g + 8, g, g + 8}, cc[4] = {8 * ks + t, 8 * ks + t, 8 * ks + t + 4, 8 * ks + t + 4};
                for (int q = 0; q < 4; ++q) {
                    const float x = (float)A(sg, rr[q], cc[q]);
                    const uint32_t big = tf32_host(x);
                    float bf;
                    std::memcpy(&bf, &big, 4);
                    frag[(((sg * 2 + 0) * KS_MAX + ks) * 32 + lane) * 4 + q] = big;
                    frag[(((sg * 2 + 1) * KS_MAX + ks) * 32 + lane) * 4 + q] = tf32_host(x - bf);
                }
            }
    // the tcgen05 B operands: rows r of the same operator, K-major core layout
    const int K = 8 * T.KS;
    frag.resize(FRAG_WORDS + UOP_WORDS, 0u);
    for (int sg = 0; sg < 2; ++sg)
        for (int r = 0; r < UN; ++r)
            for (int kk = 0; kk < K; ++kk) {
                const float x = (float)A(sg, r, kk);
                const uint32_t big = tf32_host(x);
                float bf;
                std::memcpy(&bf, &big, 4);
                frag[FRAG_WORDS + (sg * 2 + 0) * UN * K + ucore(r, kk, K)] = big;
                frag[FRAG_WORDS + (sg * 2 + 1) * UN * K + ucore(r, kk, K)] = tf32_host(x - bf);
            }
    FR_CUDA(cudaMalloc(&p->d_bgk_frag, sizeof(uint32_t) * frag.size()));
    FR_CUDA(cudaMemcpy(p->d_bgk_frag, frag.data(), sizeof(uint32_t) * frag.size(), cudaMemcpyHostToDevice));
    FR_CUDA(cudaMalloc(&p->d_bgk_prim, sizeof(float) * 3 * (size_t)s.nx * np));
    FR_CUDA(cudaMemset(p->d_bgk_prim, 0, sizeof(float) * 3 * (size_t)s.nx * np));
    return FRGPU_OK;
}

int fr_launch_bgk1d_tc(frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    switch (p->sp.np) {
    case 2: return launch_tc<2>(p, stage, in, din, out);
    case 3: return launch_tc<3>(p, stage, in, din, out);
    case 4: return launch_tc<4>(p, stage, in, din, out);
    case 5: return launch_tc<5>(p, stage, in, din, out);
    case 6: return launch_tc<6>(p, stage, in, din, out);
    }
    fr_set_error("BGK residual: polynomial degree must be 1..5");
    return FRGPU_ERR_UNSUPPORTED;
}
