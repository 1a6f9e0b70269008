// euler2d.cu -- 2D Euler dispatch and the FP64 reductions (conserved sums, CFL).
#include <mutex>
#include <string>

#include "fr_common.cuh"
#include "frgpu_internal.h"

int fr_euler2d_fp64(frgpu_problem *p, int stage, const void *in, const void *din, void *out);
int fr_euler2d_fp32k(frgpu_problem *p, int stage, const void *in, const void *din, void *out);
int fr_euler2d_met_fp64(frgpu_problem *p, int stage, const void *in, const void *din, void *out);
int fr_euler2d_met_fp32k(frgpu_problem *p, int stage, const void *in, const void *din, void *out);

namespace {
// ---- FP64 reductions: conserved sums and CFL ---------------------------------
// Two passes with a fixed reduction order (no floating-point atomics), so the
// sums are deterministic run to run.
constexpr int RED_BLOCKS = FR_RED_BLOCKS;
constexpr int RED_THREADS = 256;

// Accumulator of a thread's partial sums.  FP64 form: plain double.  FP32K
// form (state hi + lo in FP32): a double-float pair (s, e) updated by Knuth's
// TwoSum, so the FP32 pipe carries an FP64-accurate sum over the thread's
// values; the cross-thread tree is FP64.
template <class Real> struct SumAcc;
template <> struct SumAcc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double hi, double lo) { s += hi + lo; }
    __device__ __forceinline__ double value() const { return s; }
};
template <> struct SumAcc<float> {
    float s = 0.f, e = 0.f;
    __device__ __forceinline__ void add(float hi, float lo) {
        const float t = __fadd_rn(s, hi);
        const float bp = __fsub_rn(t, s);
        const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(hi, bp));
        s = t;
        e = __fadd_rn(e, __fadd_rn(err, lo));
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)e; }
};

// Block (b, q) of a grid (eblocks, nq) reduces solution point q of the
// elements [b chunk, (b + 1) chunk) of a state in the 2D device layout (DEV)
// or in the reference's u[i, j, k, l, m] (arrays a caller passes to the
// allocation-free entry point): the unweighted sums of the four
// conserved variables (scaled by the quadrature weight wp[q] in FP64 at the
// end), the largest directional wave speed max(|u| + c, |v| + c) and the
// largest CFL rate (|u| + c)/dx + (|v| + c)/dy.  The wave speeds are
// evaluated in the state's precision.
// With a per-point inverse Jacobian met (a11, a12, a21, a22 in the device
// layout; general quadrilaterals, DEV only) every value is weighted by the
// point's det J = 1 / (a11 a22 - a12 a21), so that the sums are integrals over
// the physical elements (the caller then scales by 1, not by dx dy / 4), and
// the CFL rate is (lambda_r + lambda_s) / 2 with the contravariant speeds
// lambda_r = |a11 u + a12 v| + c |(a11, a12)|, lambda_s = |a21 u + a22 v| +
// c |(a21, a22)| (on a rectangle, (|u| + c)/dx + (|v| + c)/dy again).
// Final pass over the per-block partials: warp v (of 6) combines value v, each
// lane over a fixed strided subset of the blocks, then a fixed butterfly: the
// same order every call, so the result is deterministic.  Loads bypass L1
// (the partials were written by other SMs).
__device__ __forceinline__ double final_value(const double *__restrict__ part, int nblocks, int v) {
    const int lane = threadIdx.x & 31;
    double x = 0.0; // sums start at 0; the maxima are of non-negative speeds
    // a lane takes blocks lane, lane + 32, ... in ascending order; the loads of
    // a batch are all issued before the first of them is used
    constexpr int B = 20;
    for (int b0 = 0; b0 < nblocks; b0 += 32 * B) {
        double y[B];
#pragma unroll
        for (int k = 0; k < B; ++k) {
            const int b = b0 + lane + 32 * k;
            y[k] = b < nblocks ? __ldcg(part + b * 6 + v) : 0.0;
        }
#pragma unroll
        for (int k = 0; k < B; ++k)
            if (b0 + lane + 32 * k < nblocks) x = v < 4 ? x + y[k] : fmax(x, y[k]);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const double y = __shfl_xor_sync(0xffffffffu, x, off);
        x = v < 4 ? x + y : fmax(x, y);
    }
    return x;
}

// Warp tree of a thread's partials into red[v][warp] (fixed order: deterministic).
// FP64 form: FP64 sums and maxima.  FP32K form: the sums stay double-float pairs
// through the tree (TwoSum of the high parts, the low parts and the rounding
// errors added in FP32), the maxima FP32 (exact), and only lane 0 converts to
// FP64: the FP64 pipe (1/64 of the FP32 rate here) then carries one addition per
// warp instead of 30 per thread, which had made the FP64 tree the kernel's bound.
template <class Real>
__device__ __forceinline__ void warp_partials(const SumAcc<Real> (&acc)[4], Real smax, Real rmax,
                                              double (&red)[6][RED_THREADS / 32]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if constexpr (sizeof(Real) == 8) {
        double vals[6] = {acc[0].value(), acc[1].value(), acc[2].value(), acc[3].value(), smax, rmax};
#pragma unroll
        for (int v = 0; v < 6; ++v) {
            double x = vals[v];
            for (int off = 16; off > 0; off >>= 1) {
                double y = __shfl_down_sync(0xffffffffu, x, off);
                x = v < 4 ? x + y : fmax(x, y);
            }
            if (lane == 0) red[v][w] = x;
        }
    } else {
        float hs[4], he[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            hs[m] = acc[m].s;
            he[m] = acc[m].e;
        }
        float a = smax, b = rmax;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const float s2 = __shfl_down_sync(0xffffffffu, hs[m], off);
                const float e2 = __shfl_down_sync(0xffffffffu, he[m], off);
                const float t = __fadd_rn(hs[m], s2);
                const float bp = __fsub_rn(t, hs[m]);
                const float err = __fadd_rn(__fsub_rn(hs[m], __fsub_rn(t, bp)), __fsub_rn(s2, bp));
                hs[m] = t;
                he[m] = __fadd_rn(he[m], __fadd_rn(e2, err));
            }
            a = fmaxf(a, __shfl_down_sync(0xffffffffu, a, off));
            b = fmaxf(b, __shfl_down_sync(0xffffffffu, b, off));
        }
        if (lane == 0) {
#pragma unroll
            for (int m = 0; m < 4; ++m) red[m][w] = (double)hs[m] + (double)he[m];
            red[4][w] = a;
            red[5][w] = b;
        }
    }
}

template <class Real, bool DEV, bool MET = false>
__global__ void __launch_bounds__(RED_THREADS, sizeof(Real) == 4 ? 4 : 2) k_reduce2d_partial(const Real *__restrict__ u, const Real *__restrict__ lo,
                                                             size_t plane, int nq, const double *__restrict__ wp,
                                                             double gamma, double idx_, double idy_,
                                                             double *__restrict__ part,
                                                             const Real *__restrict__ met = nullptr,
                                                             unsigned *cnt = nullptr, double *fin = nullptr,
                                                             double *hfin = nullptr, const int *dstatus = nullptr,
                                                             int *hstatus = nullptr) {
    // part layout: [q * gridDim.x + b][6]: 4 sums, max directional speed, max CFL rate
    const int q = blockIdx.y;
    const size_t npts = plane * nq;
    const size_t chunk = (plane + gridDim.x - 1) / gridDim.x;
    const size_t e0 = (size_t)blockIdx.x * chunk, e1 = e0 + chunk < plane ? e0 + chunk : plane;
    const Real g = (Real)gamma, gm1 = (Real)(gamma - 1.0), ix = (Real)idx_, iy = (Real)idy_;
    SumAcc<Real> acc[4];
    Real smax = Real(0), rmax = Real(0);
    constexpr int UN = 2; // elements whose loads are issued together (4 measured slower: occupancy)
    for (size_t eb = e0 + threadIdx.x; eb < e1; eb += UN * blockDim.x) {
        Real W[UN][4], WL[UN][4], MT[UN][4];
#pragma unroll
        for (int t = 0; t < UN; ++t) {
            const size_t e = eb + (size_t)t * blockDim.x;
#pragma unroll
            for (int m = 0; m < 4; ++m) W[t][m] = WL[t][m] = MT[t][m] = Real(0);
            if (e >= e1) continue;
            if (DEV) {
                const size_t at = frk::e2d_index(e, q, 0, plane);
                frk::ldg4(u + at, W[t]);
                if (lo != nullptr) frk::ldg4(lo + at, WL[t]);
                if (MET) frk::ldg4(met + at, MT[t]);
            } else {
                const size_t tt = e + plane * q;
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    W[t][m] = u[tt + npts * m];
                    if (lo != nullptr) WL[t][m] = lo[tt + npts * m];
                }
            }
        }
        // the elements in ascending order, as one element per iteration would take them
#pragma unroll
        for (int t = 0; t < UN; ++t) {
            if (eb + (size_t)t * blockDim.x >= e1) break;
            Real *w = W[t], *wl = WL[t], *mt = MT[t];
            Real jac = Real(1);
            if (DEV && MET) jac = Real(1) / (mt[0] * mt[3] - mt[1] * mt[2]);
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                if (DEV && MET) acc[m].add(w[m] * jac, wl[m] * jac);
                else acc[m].add(w[m], wl[m]);
                w[m] += wl[m];
            }
            const Real rinv = frk::recipR<Real>(w[0]);
            const Real U = w[1] * rinv, V = w[2] * rinv;
            const Real p = gm1 * (w[3] - Real(0.5) * (w[1] * U + w[2] * V));
            const Real c = frk::sqrtP<Real>(g * p * rinv);
            const Real a = fabs(U) + c, bb = fabs(V) + c;
            smax = fmax(smax, fmax(a, bb));
            if (DEV && MET) {
                const Real lr = fabs(mt[0] * U + mt[1] * V) + c * frk::sqrtR<Real>(mt[0] * mt[0] + mt[1] * mt[1]);
                const Real ls = fabs(mt[2] * U + mt[3] * V) + c * frk::sqrtR<Real>(mt[2] * mt[2] + mt[3] * mt[3]);
                rmax = fmax(rmax, Real(0.5) * (lr + ls));
            } else {
                rmax = fmax(rmax, a * ix + bb * iy);
            }
        }
    }
    __shared__ double red[6][RED_THREADS / 32];
    warp_partials<Real>(acc, smax, rmax, red);
    __syncthreads();
    if (threadIdx.x < 6) {
        const int v = threadIdx.x;
        double x = red[v][0];
        for (int w = 1; w < RED_THREADS / 32; ++w) x = v < 4 ? x + red[v][w] : fmax(x, red[v][w]);
        part[((size_t)q * gridDim.x + blockIdx.x) * 6 + v] = v < 4 ? x * wp[q] : x;
    }
    if (cnt == nullptr) return;
    // the last block to finish combines every block's partials (the order of
    // the final pass is fixed, so the result does not depend on which block it is)
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(cnt, 1u) == gridDim.x * gridDim.y - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int v = threadIdx.x >> 5;
    if (v < 6) {
        const double x = final_value(part, (int)(gridDim.x * gridDim.y), v);
        if ((threadIdx.x & 31) == 0) {
            fin[v] = x;
            if (hfin) hfin[v] = x; // straight into the caller's page-locked host words
        }
    }
    if (threadIdx.x == 0) {
        if (hstatus) *hstatus = __ldcg(dstatus);
        *cnt = 0u; // ready for the next launch
    }
}

__global__ void __launch_bounds__(192) k_reduce_final(const double *__restrict__ part, int nblocks,
                                                      double *__restrict__ out) {
    const int v = threadIdx.x >> 5;
    const double x = final_value(part, nblocks, v);
    if ((threadIdx.x & 31) == 0) out[v] = x;
}

} // namespace

int fr_launch_euler2d(frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    if (p->d.flux == FRGPU_FLUX_CENTRAL) return fr_launch_central2d(p, stage, in, out);
    if (p->d_met) {
        if (p->d.precision == FRGPU_FP64) return fr_euler2d_met_fp64(p, stage, in, din, out);
        return fr_euler2d_met_fp32k(p, stage, in, din, out);
    }
    if (p->d.precision == FRGPU_FP64) return fr_euler2d_fp64(p, stage, in, din, out);
    return fr_euler2d_fp32k(p, stage, in, din, out);
}

// out (device, 6 doubles at p->d_red + RED_BLOCKS*6): sums[4], max speed, max CFL rate.
void fr_drop_reduce_graphs(frgpu_problem *p) {
    for (auto &g : p->red_graphs) {
        if (g.gexec) cudaGraphExecDestroy(g.gexec);
        g.gexec = nullptr;
        g.state = nullptr;
    }
}

// partial + final kernels, then the 6 results and the status word copied to
// the problem's page-locked host words
static int enqueue_reduce(frgpu_problem *p, const void *state, const void *lo, double cfl_dx, double cfl_dy) {
    const size_t plane = (size_t)p->sp.nx * p->sp.ny;
    const int np = p->sp.np;
    double *wp = p->d_red + FR_RED_WP;
    double *part = p->d_red;
    double *fin = p->d_red + FR_RED_FINAL;
    const int nq = np * np;
    const dim3 grid(RED_BLOCKS / nq, nq);
    // general quadrilaterals: weights det J and contravariant speeds from the metric
    // the spare final slot 7 holds the last-block counter (zeroed with d_red, reset by the kernel);
    // the results and the status word go to the page-locked host words from the kernel itself
    unsigned *cnt = reinterpret_cast<unsigned *>(fin + 7);
    frgpu_problem::host_words *hw = nullptr;
    FR_CUDA(cudaHostGetDevicePointer((void **)&hw, p->h_words, 0));
    const bool met = p->d_met != nullptr;
    if (p->d.precision == FRGPU_FP64) {
        auto k = met ? k_reduce2d_partial<double, true, true> : k_reduce2d_partial<double, true, false>;
        k<<<grid, RED_THREADS, 0, p->stream>>>((const double *)state, (const double *)lo, plane, nq, wp, p->d.gamma,
                                               cfl_dx, cfl_dy, part, (const double *)p->d_met, cnt, fin, hw->red,
                                               p->d_status, &hw->status);
    } else {
        auto k = met ? k_reduce2d_partial<float, true, true> : k_reduce2d_partial<float, true, false>;
        k<<<grid, RED_THREADS, 0, p->stream>>>((const float *)state, (const float *)lo, plane, nq, wp, p->d.gamma,
                                               cfl_dx, cfl_dy, part, (const float *)p->d_met, cnt, fin, hw->red,
                                               p->d_status, &hw->status);
    }
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}

int fr_launch_euler2d_reduce(frgpu_problem *p, const void *state, const void *lo, double *out_sums,
                             double *out_speed, double cfl_dx, double cfl_dy, int *status) {
    // the callers pass the rectangles' 1/dx, 1/dy: the graph of a state buffer
    // holds them as its kernel arguments
    if (cfl_dx != 1.0 / p->sp.dx || cfl_dy != 1.0 / p->sp.dy) {
        int rc = enqueue_reduce(p, state, lo, cfl_dx, cfl_dy);
        if (rc) return rc;
    } else {
        frgpu_problem::red_graph *g = nullptr;
        for (auto &r : p->red_graphs)
            if (r.gexec && r.state == state) g = &r;
        if (!g) {
            g = p->red_graphs[0].gexec ? &p->red_graphs[1] : &p->red_graphs[0];
            if (g->gexec) {
                FR_CUDA(cudaStreamSynchronize(p->stream));
                cudaGraphExecDestroy(g->gexec);
                g->gexec = nullptr;
            }
            cudaGraph_t graph = nullptr;
            FR_CUDA(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
            int rc = enqueue_reduce(p, state, lo, cfl_dx, cfl_dy);
            cudaError_t ce = cudaStreamEndCapture(p->stream, &graph);
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            if (ce != cudaSuccess) return fr_cuda_fail(ce, "cudaStreamEndCapture");
            ce = cudaGraphInstantiate(&g->gexec, graph, 0);
            cudaGraphDestroy(graph);
            if (ce != cudaSuccess) return fr_cuda_fail(ce, "cudaGraphInstantiate");
            g->state = state;
        }
        FR_CUDA(cudaGraphLaunch(g->gexec, p->stream));
    }
    p->launches += 1;
    FR_CUDA(cudaStreamSynchronize(p->stream));
    const double *h = p->h_words->red;
    if (status) *status = p->h_words->status;
    const double area = p->d_met ? 1.0 : p->sp.dx * p->sp.dy * 0.25;
    if (out_sums)
        for (int m = 0; m < 4; ++m) out_sums[m] = h[m] * area;
    if (out_speed) {
        out_speed[0] = h[4];
        out_speed[1] = h[5];
    }
    return FRGPU_OK;
}

// ---- allocation-free variant of the 2D reduction -----------------------------
// Some callers cannot let this library call cudaMalloc: hosts that own every
// device byte through their own pool (a Julia CUDA.jl or PyTorch caching
// allocator that must see all device memory), and processes that fix their
// device footprint at start-up.  frgpu_reduce2d_noalloc serves them: it runs
// the same partial/final reduction kernels as frgpu_reduce, but its partial
// sums live in the file-scope device array below instead of memory allocated
// per problem.  The array is 4096 x 6 doubles (192 KiB); one partial block
// covers one solution point q of up to NOALLOC_POINTS_PER_BLOCK = 16384
// elements, so a call needs ceil(nx * ny / 16384) * (deg+1)^2 <= 4096 blocks,
// and meshes that need more are rejected.  (That allows at most 67,108,864
// solution points nx * ny * (deg+1)^2, reached when nx * ny is a multiple of
// 16384; because of the rounding up, some smaller meshes are rejected too.)
// Every GPU that loads the library keeps the array until the process exits.
namespace {
constexpr int NOALLOC_MAX_BLOCKS = 4096;
constexpr long NOALLOC_POINTS_PER_BLOCK = (long)RED_THREADS * 64;
__device__ __align__(256) double g_noalloc_partials[NOALLOC_MAX_BLOCKS * 6];

// Device address of g_noalloc_partials, looked up once per device (host code
// cannot use the symbol itself: on the host it names a stand-in, not device memory).
void *g_noalloc_addr[FR_MAX_DEVICES] = {};
std::mutex g_noalloc_mu;

int noalloc_scratch(double **out) {
    int dev = 0;
    FR_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= FR_MAX_DEVICES) {
        fr_set_error("reduce2d_noalloc: device index out of range");
        return FRGPU_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_partials);
        if (e != cudaSuccess || ptr == nullptr) return fr_cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_partials)");
        g_noalloc_addr[dev] = ptr;
    }
    *out = (double *)g_noalloc_addr[dev];
    return FRGPU_OK;
}

// final pass of the allocation-free reduction: sums scaled by the element area
__global__ void __launch_bounds__(192) k_reduce_final_scaled(const double *__restrict__ part, int nblocks,
                                                             double scale, double *__restrict__ out) {
    const int v = threadIdx.x >> 5;
    const double x = final_value(part, nblocks, v);
    if ((threadIdx.x & 31) == 0) out[v] = v < 4 ? x * scale : x;
}
} // namespace

extern "C" FRGPU_API int frgpu_reduce2d_noalloc(const void *d_state, const void *d_lo, int precision, int nx, int ny,
                                                int deg, double dx, double dy, double gamma, const double *d_wp,
                                                double *d_out, void *stream) {
    if (!d_state || !d_wp || !d_out) {
        fr_set_error("reduce2d_noalloc: null device pointer");
        return FRGPU_ERR_ARG;
    }
    if (precision != FRGPU_FP64 && precision != FRGPU_FP32K) {
        fr_set_error("reduce2d_noalloc: unknown precision");
        return FRGPU_ERR_ARG;
    }
    if (precision == FRGPU_FP64 && d_lo) {
        fr_set_error("reduce2d_noalloc: d_lo must be NULL with FRGPU_FP64 (only the FP32K form has a low part)");
        return FRGPU_ERR_ARG;
    }
    if (nx < 1 || ny < 1 || deg < 1 || deg > 5 || !(dx > 0) || !(dy > 0) || !(gamma > 1)) {
        fr_set_error("reduce2d_noalloc: need nx, ny >= 1, 1 <= deg <= 5, dx, dy > 0 and gamma > 1");
        return FRGPU_ERR_ARG;
    }
    const int np = deg + 1;
    const size_t plane = (size_t)nx * ny;
    const size_t npts = plane * np * np;
    const long eblocks = (long)((plane + NOALLOC_POINTS_PER_BLOCK - 1) / NOALLOC_POINTS_PER_BLOCK);
    const long nblocks = eblocks * np * np;
    if (nblocks > NOALLOC_MAX_BLOCKS) {
        fr_set_error("reduce2d_noalloc: " + std::to_string(npts) + " solution points need " +
                     std::to_string(nblocks) + " partial blocks (ceil(nx*ny/" +
                     std::to_string(NOALLOC_POINTS_PER_BLOCK) + ") * (deg+1)^2), which exceed the maximum of " +
                     std::to_string(NOALLOC_MAX_BLOCKS) + " that the static scratch array holds");
        return FRGPU_ERR_ARG;
    }
    double *part = nullptr;
    int rc = noalloc_scratch(&part);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    // each partial block overwrites its own six slots, so the previous call's
    // contents never need clearing
    const dim3 grid((unsigned)eblocks, (unsigned)(np * np));
    if (precision == FRGPU_FP64)
        k_reduce2d_partial<double, false><<<grid, RED_THREADS, 0, st>>>(
            (const double *)d_state, (const double *)d_lo, plane, np * np, d_wp, gamma, 1.0 / dx, 1.0 / dy, part);
    else
        k_reduce2d_partial<float, false><<<grid, RED_THREADS, 0, st>>>(
            (const float *)d_state, (const float *)d_lo, plane, np * np, d_wp, gamma, 1.0 / dx, 1.0 / dy, part);
    FR_CUDA(cudaGetLastError());
    k_reduce_final_scaled<<<1, 192, 0, st>>>(part, (int)nblocks, dx * dy * 0.25, d_out);
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}
