// euler2d.cu -- 2D Euler dispatch and the FP64 reductions (conserved sums, CFL).
#include <mutex>
#include <string>

#include "fr_common.cuh"
#include "frgpu_internal.h"

int fr_euler2d_fp64(frgpu_problem *p, int stage, const void *in, const void *din, void *out);
int fr_euler2d_fp32k(frgpu_problem *p, int stage, const void *in, const void *din, void *out);

namespace {
// ---- FP64 reductions: conserved sums and CFL ---------------------------------
// Two passes with a fixed reduction order (no floating-point atomics), so the
// sums are deterministic run to run.
constexpr int RED_BLOCKS = FR_RED_BLOCKS;
constexpr int RED_THREADS = 256;

template <class Real>
__global__ void __launch_bounds__(RED_THREADS) k_reduce2d_partial(const Real *__restrict__ u, const Real *__restrict__ lo,
                                                             size_t plane, int np, const double *__restrict__ wp,
                                                             double gamma, double idx_, double idy_,
                                                             double *__restrict__ part) {
    // part layout: [block][6]: 4 sums, max directional speed, max CFL rate
    double s[4] = {0, 0, 0, 0}, smax = 0, rmax = 0;
    const int nq = np * np;
    const size_t npts = plane * nq;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < npts; t += (size_t)gridDim.x * blockDim.x) {
        const int q = (int)(t / plane);
        double w[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            double v = (double)u[t + npts * m];
            if (lo != nullptr) v += (double)lo[t + npts * m];
            w[m] = v;
            s[m] += wp[q] * v;
        }
        double U = w[1] / w[0], V = w[2] / w[0];
        double p = (gamma - 1.0) * (w[3] - 0.5 * (w[1] * U + w[2] * V));
        double c = sqrt(gamma * p / w[0]);
        double a = fabs(U) + c, b = fabs(V) + c;
        smax = fmax(smax, fmax(a, b));
        rmax = fmax(rmax, a * idx_ + b * idy_);
    }
    __shared__ double red[6][RED_THREADS / 32];
    double vals[6] = {s[0], s[1], s[2], s[3], smax, rmax};
#pragma unroll
    for (int v = 0; v < 6; ++v) {
        double x = vals[v];
        for (int off = 16; off > 0; off >>= 1) {
            double y = __shfl_down_sync(0xffffffffu, x, off);
            x = v < 4 ? x + y : fmax(x, y);
        }
        if ((threadIdx.x & 31) == 0) red[v][threadIdx.x >> 5] = x;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int v = threadIdx.x;
        double x = red[v][0];
        for (int w = 1; w < RED_THREADS / 32; ++w) x = v < 4 ? x + red[v][w] : fmax(x, red[v][w]);
        part[blockIdx.x * 6 + v] = x;
    }
}

__global__ void k_reduce_final(const double *__restrict__ part, int nblocks, double *__restrict__ out) {
    if (threadIdx.x < 6) {
        const int v = threadIdx.x;
        double x = part[v];
        for (int b = 1; b < nblocks; ++b) x = v < 4 ? x + part[b * 6 + v] : fmax(x, part[b * 6 + v]);
        out[v] = x;
    }
}

} // namespace

int fr_launch_euler2d(frgpu_problem *p, int stage, const void *in, const void *din, void *out) {
    if (p->d.precision == FRGPU_FP64) return fr_euler2d_fp64(p, stage, in, din, out);
    return fr_euler2d_fp32k(p, stage, in, din, out);
}

// out (device, 6 doubles at p->d_red + RED_BLOCKS*6): sums[4], max speed, max CFL rate.
int fr_launch_euler2d_reduce(frgpu_problem *p, const void *state, const void *lo, double *out_sums,
                             double *out_speed, double cfl_dx, double cfl_dy) {
    const size_t plane = (size_t)p->sp.nx * p->sp.ny;
    const int np = p->sp.np;
    double *wp = p->d_red + FR_RED_WP;
    double *part = p->d_red;
    double *fin = p->d_red + FR_RED_FINAL;
    if (p->d.precision == FRGPU_FP64)
        k_reduce2d_partial<double><<<RED_BLOCKS, RED_THREADS, 0, p->stream>>>((const double *)state, (const double *)lo,
                                                                           plane, np, wp, p->d.gamma, cfl_dx,
                                                                           cfl_dy, part);
    else
        k_reduce2d_partial<float><<<RED_BLOCKS, RED_THREADS, 0, p->stream>>>((const float *)state, (const float *)lo,
                                                                          plane, np, wp, p->d.gamma, cfl_dx, cfl_dy,
                                                                          part);
    FR_CUDA(cudaGetLastError());
    k_reduce_final<<<1, 32, 0, p->stream>>>(part, RED_BLOCKS, fin);
    FR_CUDA(cudaGetLastError());
    p->launches += 2;
    double h[6];
    FR_CUDA(cudaMemcpyAsync(h, fin, sizeof(h), cudaMemcpyDeviceToHost, p->stream));
    FR_CUDA(cudaStreamSynchronize(p->stream));
    const double area = p->sp.dx * p->sp.dy * 0.25;
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
// covers up to NOALLOC_POINTS_PER_BLOCK solution points, so a call accepts at
// most 4096 * 16384 = 67,108,864 solution points (nx * ny * (deg+1)^2) and
// rejects larger meshes.  Every GPU that loads the library keeps the array
// until the process exits.
namespace {
constexpr int NOALLOC_MAX_BLOCKS = 4096;
constexpr long NOALLOC_POINTS_PER_BLOCK = (long)RED_THREADS * 64;
constexpr int FR_MAX_DEVICES = 64;
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
__global__ void k_reduce_final_scaled(const double *__restrict__ part, int nblocks, double scale,
                                      double *__restrict__ out) {
    if (threadIdx.x < 6) {
        const int v = threadIdx.x;
        double x = part[v];
        for (int b = 1; b < nblocks; ++b) x = v < 4 ? x + part[b * 6 + v] : fmax(x, part[b * 6 + v]);
        out[v] = v < 4 ? x * scale : x;
    }
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
    if (nx < 1 || ny < 1 || deg < 1 || deg > 5 || !(dx > 0) || !(dy > 0) || !(gamma > 1)) {
        fr_set_error("reduce2d_noalloc: need nx, ny >= 1, 1 <= deg <= 5, dx, dy > 0 and gamma > 1");
        return FRGPU_ERR_ARG;
    }
    const int np = deg + 1;
    const size_t plane = (size_t)nx * ny;
    const size_t npts = plane * np * np;
    const long nblocks = (long)((npts + NOALLOC_POINTS_PER_BLOCK - 1) / NOALLOC_POINTS_PER_BLOCK);
    if (nblocks > NOALLOC_MAX_BLOCKS) {
        fr_set_error("reduce2d_noalloc: " + std::to_string(npts) + " solution points exceed the maximum of " +
                     std::to_string((long)NOALLOC_MAX_BLOCKS * NOALLOC_POINTS_PER_BLOCK) +
                     " that the static scratch array holds");
        return FRGPU_ERR_ARG;
    }
    double *part = nullptr;
    int rc = noalloc_scratch(&part);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    // each partial block overwrites its own six slots, so the previous call's
    // contents never need clearing
    if (precision == FRGPU_FP64)
        k_reduce2d_partial<double><<<(int)nblocks, RED_THREADS, 0, st>>>(
            (const double *)d_state, (const double *)d_lo, plane, np, d_wp, gamma, 1.0 / dx, 1.0 / dy, part);
    else
        k_reduce2d_partial<float><<<(int)nblocks, RED_THREADS, 0, st>>>(
            (const float *)d_state, (const float *)d_lo, plane, np, d_wp, gamma, 1.0 / dx, 1.0 / dy, part);
    FR_CUDA(cudaGetLastError());
    k_reduce_final_scaled<<<1, 32, 0, st>>>(part, (int)nblocks, dx * dy * 0.25, d_out);
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}
