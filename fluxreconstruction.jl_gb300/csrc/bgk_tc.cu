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
// [16 x 8 KS] operator (per velocity sign) times the [8 KS x 8] panel of point
// values of elements i0-1 .. i0+EB at 8 velocities: an m16n8k8 TF32 MMA chain.
// FP32 accuracy is kept with the three-term TF32 split
//   A B ~= Ab Bb + Ab Bs + As Bb,  X = Xb + Xs,  Xb = tf32(X), Xs = tf32(X - Xb)
// (the split product of Ootomo and Yokota, "Recovering single precision accuracy
// from Tensor Cores while surpassing the FP32 theoretical peak performance", 2022).
//
// The BGK collision term (M - u)/tau needs the moments (rho, rho U, E) of every
// (element, point) over all velocities, with conserve_prim at gamma = 3
// (bgk_wave.jl:76-81).  Each CTA recomputes them for its EB elements over all
// velocities (FP32 per lane, pairwise across the warp) before its MMA tiles;
// the state is small enough (a few MB) that the repeated reads hit L2.
//
// Layout: internal u[(i * np + k) * nvel + v] (velocity fastest).  CTA = EB
// elements x 128 velocities, 4 warps, each warp 4 n-tiles of 8 velocities.
#include <cmath>

#include "fr_stage.cuh"
#include "frgpu_internal.h"

using namespace frk;

namespace {

constexpr int TCW = 4;          // warps per CTA
constexpr int VT = 32 * TCW;    // velocities per CTA (4 n-tiles of 8 per warp)

template <int NP> struct BT {
    static constexpr int EB = 16 / NP;       // elements per tile
    static constexpr int ROWS = EB * NP;     // output rows used
    static constexpr int KR = (EB + 2) * NP; // source rows: elements i0-1 .. i0+EB
    static constexpr int KS = (KR + 7) / 8;  // k8 steps
};

// J-free transport blocks per velocity sign s (0: v <= 0, 1: v > 0):
// Mc[s] couples an element to itself, Mn[s] to its upwind neighbour
// (left for v > 0, right for v <= 0).
template <int NP> struct TCOps {
    float Mc[2][NP][NP], Mn[2][NP][NP];
};

template <int NP> struct TCArgs {
    int ne, nvel;
    const float *uin, *din, *un;
    float *out, *ul;
    const double *dtp;
    const float *J;
    const float *velo, *w;
    float tau;
    TCOps<NP> ops;
    int *status;
};

__device__ __forceinline__ uint32_t tf32_of(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ void split_tf32(float x, uint32_t &big, uint32_t &small) {
    big = tf32_of(x);
    small = tf32_of(x - __uint_as_float(big));
}

// D += A (16x8, row) * B (8x8, col), TF32 in, FP32 accumulate
__device__ __forceinline__ void mma1688(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ int wrapn(int i, int n) { return ((i % n) + n) % n; }

template <int NP, int STAGE>
__global__ void __launch_bounds__(32 * TCW) k_bgk1d_tc(const TCArgs<NP> a) {
    using T = BT<NP>;
    constexpr int KC = 8 * T::KS;
    __shared__ float sA[2][2][16][KC]; // [sign][big/small][row][source row]
    __shared__ float sprim[16][3];     // rho, U, lambda per output row
    const int ne = a.ne, nv = a.nvel;
    const int i0 = blockIdx.x * T::EB;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int bad = 0;

    // ---- the tile's operator (scaled by the source elements' 1/J), split into TF32 parts
    for (int q = threadIdx.x; q < 2 * 16 * KC; q += blockDim.x) {
        const int s = q / (16 * KC), r = (q / KC) % 16, kk = q % KC;
        float val = 0.f;
        if (r < T::ROWS && kk < T::KR) {
            const int el = r / NP, m = r % NP, es = kk / NP - 1, k = kk % NP;
            const int up = s == 1 ? el - 1 : el + 1; // upwind neighbour (local index)
            float c = 0.f;
            if (es == el)
                c = a.ops.Mc[s][m][k];
            else if (es == up)
                c = a.ops.Mn[s][m][k];
            if (c != 0.f) val = c / a.J[wrapn(i0 + es, ne)];
        }
        const float big = __uint_as_float(tf32_of(val));
        sA[s][0][r][kk] = big;
        sA[s][1][r][kk] = __uint_as_float(tf32_of(val - big));
    }

    // ---- moments of the tile's rows over all velocities -> primitive variables
    for (int r = warp; r < T::ROWS; r += TCW) {
        const int e = i0 + r / NP, k = r % NP;
        float m0 = 0.f, m1 = 0.f, m2 = 0.f;
        if (e < ne) {
            const size_t base = ((size_t)e * NP + k) * nv;
            for (int v = lane; v < nv; v += 32) {
                const float x = ld_state(a.uin, a.din, base + v);
                const float vel = __ldg(a.velo + v), wx = __ldg(a.w + v) * x;
                m0 += wx;
                m1 = fmaf(wx, vel, m1);
                m2 = fmaf(wx * vel, vel, m2);
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            m0 += __shfl_xor_sync(0xffffffffu, m0, off);
            m1 += __shfl_xor_sync(0xffffffffu, m1, off);
            m2 += __shfl_xor_sync(0xffffffffu, m2, off);
        }
        if (lane == 0) {
            // conserve_prim(w, gamma = 3), 1D: U = m/rho, lambda = rho / (4 (E - m^2 / (2 rho)))
            const double w0 = m0, w1 = m1, w2 = 0.5 * (double)m2;
            const double U = w1 / w0;
            const double lam = 0.25 * w0 / (w2 - 0.5 * w1 * U);
            sprim[r][0] = (float)w0;
            sprim[r][1] = (float)U;
            sprim[r][2] = (float)lam;
            if (e < ne && (!(w0 > 0.0) || !(lam > 0.0))) bad |= ST_UNPHYSICAL;
        }
    }
    __syncthreads();

    const int g = lane >> 2, t = lane & 3;
    // A fragments of both signs (rows g, g+8; source rows 8s + t, 8s + t + 4)
    uint32_t A[2][2][T::KS][4];
#pragma unroll
    for (int s = 0; s < 2; ++s)
#pragma unroll
        for (int p = 0; p < 2; ++p)
#pragma unroll
            for (int ks = 0; ks < T::KS; ++ks) {
                A[s][p][ks][0] = __float_as_uint(sA[s][p][g][8 * ks + t]);
                A[s][p][ks][1] = __float_as_uint(sA[s][p][g + 8][8 * ks + t]);
                A[s][p][ks][2] = __float_as_uint(sA[s][p][g][8 * ks + t + 4]);
                A[s][p][ks][3] = __float_as_uint(sA[s][p][g + 8][8 * ks + t + 4]);
            }
    // global (element, point) row offsets of this lane's B rows
    size_t brow[T::KS][2];
#pragma unroll
    for (int ks = 0; ks < T::KS; ++ks)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int kk = 8 * ks + t + 4 * h;
            brow[ks][h] = kk < T::KR ? ((size_t)wrapn(i0 + kk / NP - 1, ne) * NP + kk % NP) * nv : (size_t)-1;
        }
    const float dt = (float)(*a.dtp);
    const float pi_inv = 0.31830988618379067154f, itau = 1.0f / a.tau;

    for (int nt = 0; nt < 4; ++nt) {
        const int n0 = blockIdx.y * VT + warp * 32 + nt * 8;
        if (n0 >= nv) break;
        const int vb = n0 + g; // this lane's B column
        const bool vb_ok = vb < nv;
        const float velb = vb_ok ? __ldg(a.velo + vb) : 0.f;
        const unsigned pos = __ballot_sync(0xffffffffu, !vb_ok || velb > 0.f);
        const unsigned neg = __ballot_sync(0xffffffffu, !vb_ok || !(velb > 0.f));
        const bool all_pos = pos == 0xffffffffu, all_neg = neg == 0xffffffffu;
        float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
        for (int ks = 0; ks < T::KS; ++ks) {
            uint32_t bb[2], bs[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                float x = 0.f;
                if (vb_ok && brow[ks][h] != (size_t)-1) x = ld_state(a.uin, a.din, brow[ks][h] + vb);
                split_tf32(x, bb[h], bs[h]);
            }
            if (!all_neg) { // v > 0 operator
                mma1688(acc[1], A[1][1][ks], bb[0], bb[1]);
                mma1688(acc[1], A[1][0][ks], bs[0], bs[1]);
                mma1688(acc[1], A[1][0][ks], bb[0], bb[1]);
            }
            if (!all_pos) { // v <= 0 operator
                mma1688(acc[0], A[0][1][ks], bb[0], bb[1]);
                mma1688(acc[0], A[0][0][ks], bs[0], bs[1]);
                mma1688(acc[0], A[0][0][ks], bb[0], bb[1]);
            }
        }
        // epilogue: rows g, g+8; velocities n0 + 2t, n0 + 2t + 1
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int r = g + 8 * (q >> 1), v = n0 + 2 * t + (q & 1);
            const int e = i0 + r / NP, m = r % NP;
            if (r >= T::ROWS || e >= ne || v >= nv) continue;
            const float vel = __ldg(a.velo + v);
            const float tr = vel > 0.f ? acc[1][q] : acc[0][q];
            const size_t idx = ((size_t)e * NP + m) * nv + v;
            const float u = ld_state(a.uin, a.din, idx);
            const float rho = sprim[r][0], U = sprim[r][1], lam = sprim[r][2];
            const float dv = vel - U;
            const float M = rho * sqrtf(lam * pi_inv) * expf(-lam * dv * dv);
            const float du = fmaf(-vel, tr, (M - u) * itau);
            const float res = stage_update<float, MODE_FP32K, STAGE>(du, u, dt, idx, a.un, a.uin, a.din, a.out, a.ul);
            if (!isfinite(res)) bad |= ST_NONFINITE;
        }
    }
    if (bad) atomicOr(a.status, bad);
}

template <int NP> TCOps<NP> make_tc_ops(const frgpu_space &s) {
    TCOps<NP> o;
    for (int m = 0; m < NP; ++m)
        for (int k = 0; k < NP; ++k) {
            const double D = s.dl[m + NP * k];
            o.Mc[1][m][k] = (float)(D - s.dhl[m] * s.ll[k]);
            o.Mn[1][m][k] = (float)(s.dhl[m] * s.lr[k]);
            o.Mc[0][m][k] = (float)(D - s.dhr[m] * s.lr[k]);
            o.Mn[0][m][k] = (float)(s.dhr[m] * s.ll[k]);
        }
    return o;
}

template <int NP>
int launch_tc(frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    if (p->prepare_only) return FRGPU_OK;
    TCArgs<NP> a;
    a.ne = p->sp.nx;
    a.nvel = p->d.nvel;
    a.uin = (const float *)in;
    a.din = (const float *)din;
    a.un = (const float *)p->s0;
    a.out = (float *)out;
    a.ul = (float *)p->s3;
    a.dtp = p->d_dt;
    a.J = (const float *)p->d_J;
    a.velo = (const float *)p->d_velo;
    a.w = (const float *)p->d_w;
    a.tau = (float)p->d.tau;
    a.ops = make_tc_ops<NP>(p->sp);
    a.status = p->d_status;
    const dim3 grid((a.ne + BT<NP>::EB - 1) / BT<NP>::EB, (a.nvel + VT - 1) / VT);
    switch (stage) {
    case 0: k_bgk1d_tc<NP, 0><<<grid, 32 * TCW, 0, p->stream>>>(a); break;
    case 1: k_bgk1d_tc<NP, 1><<<grid, 32 * TCW, 0, p->stream>>>(a); break;
    case 2: k_bgk1d_tc<NP, 2><<<grid, 32 * TCW, 0, p->stream>>>(a); break;
    case 3: k_bgk1d_tc<NP, 3><<<grid, 32 * TCW, 0, p->stream>>>(a); break;
    default: fr_set_error("BGK residual: bad stage"); return FRGPU_ERR_ARG;
    }
    FR_CUDA(cudaGetLastError());
    p->launches += 1;
    return FRGPU_OK;
}

} // namespace

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
