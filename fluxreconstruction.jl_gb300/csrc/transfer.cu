// transfer.cu -- host state arrays (FP64, the reference's Julia layout) to and
// from the device state (internal layout, FP64 or the FP32 high/low pair).
//
// One cudaMemcpy moves the FP64 array into a device staging buffer; a kernel
// then checks it for non-finite values, splits it into the FP32 high part and
// the FP32 low part x - (double)hi (FP32K), and reorders the layouts that
// differ on the device: BGK f[i, v, k] -> u[(i * np + k) * nvel + v], and the
// 2D Euler u[i, j, k, l, m] -> the point-vector layout of e2d_index.
// Downloads run the reverse kernel (hi + lo in FP64) and one cudaMemcpy back.
// A page-locked (or registered) host array skips the staging copy: the kernels
// read or write it in place through its device mapping.  No per-element host
// loop.
#include <string>

#include "fr_common.cuh"
#include "frgpu_internal.h"

namespace {

enum { LAYOUT_SAME = 0, LAYOUT_BGK = 1, LAYOUT_E2D = 2 };

struct Layout {
    int kind;
    long ne, nv, np;
};

// device index of host index q (BGK q = i + ne (v + nv k)); the 1D equations
// keep the host layout, and 2D Euler has kernels of its own below
__device__ __forceinline__ long dev_index(const Layout &L, long q) {
    if (L.kind == LAYOUT_BGK) {
        const long i = q % L.ne, r = q / L.ne, v = r % L.nv, k = r / L.nv;
        return (i * L.np + k) * L.nv + v;
    }
    return q;
}

template <class Real>
__global__ void k_upload(const double *__restrict__ src, Real *__restrict__ hi, Real *__restrict__ lo, long n,
                         Layout L, unsigned long long *__restrict__ first_bad) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const double x = src[q];
        if (!isfinite(x)) atomicMin(first_bad, (unsigned long long)q);
        const long d = dev_index(L, q);
        if (sizeof(Real) == 8) {
            hi[d] = (Real)x;
        } else {
            const float h = (float)x;
            hi[d] = h;
            if (lo) lo[d] = (float)(x - (double)h);
        }
    }
}

// 2D Euler: one thread per (element, point) moves the point's 4 variables: 4
// coalesced FP64 reads of the host-order planes, one vector store per output.
// Grid (element blocks, points).
template <class Real>
__global__ void k_upload_e2d(const double *__restrict__ src, Real *__restrict__ hi, Real *__restrict__ lo, long ne,
                             long nq, unsigned long long *__restrict__ first_bad) {
    const long e = blockIdx.x * (long)blockDim.x + threadIdx.x, pt = blockIdx.y;
    if (e >= ne) return;
    Real h[4], l[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        const long s = e + ne * (pt + nq * m);
        const double x = src[s];
        if (!isfinite(x)) atomicMin(first_bad, (unsigned long long)s);
        h[m] = (Real)x;
        l[m] = (Real)(x - (double)h[m]);
    }
    const size_t at = frk::e2d_index((size_t)e, (int)pt, 0, (size_t)ne);
    frk::st4(hi + at, h);
    if (sizeof(Real) == 4 && lo) frk::st4(lo + at, l);
}

template <class Real>
__global__ void k_download_e2d(const Real *__restrict__ hi, const Real *__restrict__ lo, double *__restrict__ dst,
                               long ne, long nq) {
    const long e = blockIdx.x * (long)blockDim.x + threadIdx.x, pt = blockIdx.y;
    if (e >= ne) return;
    const size_t at = frk::e2d_index((size_t)e, (int)pt, 0, (size_t)ne);
    Real h[4], l[4] = {Real(0), Real(0), Real(0), Real(0)};
    frk::ldg4(hi + at, h);
    if (lo) frk::ldg4(lo + at, l);
#pragma unroll
    for (int m = 0; m < 4; ++m) dst[e + ne * (pt + nq * m)] = (double)h[m] + (double)l[m];
}

template <class Real>
__global__ void k_download(const Real *__restrict__ hi, const Real *__restrict__ lo, double *__restrict__ dst,
                           long n, Layout L) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const long d = dev_index(L, q);
        double x = (double)hi[d];
        if (lo) x += (double)lo[d];
        dst[q] = x;
    }
}

Layout layout_of(const frgpu_problem *p) {
    const int kind = p->d.equation == FRGPU_BGK1D ? LAYOUT_BGK : (p->d.equation == FRGPU_EULER2D ? LAYOUT_E2D : LAYOUT_SAME);
    const long ne = p->d.equation == FRGPU_EULER2D ? (long)p->sp.nx * p->sp.ny : (long)p->sp.nx;
    Layout L{kind, ne, p->d.nvel, p->sp.np};
    return L;
}

int stage_buffer(frgpu_problem *p) {
    if (!p->d_stage) {
        FR_CUDA(cudaMalloc(&p->d_stage, sizeof(double) * (size_t)p->ndof + sizeof(unsigned long long)));
    }
    return FRGPU_OK;
}

int grid_for(long n) {
    const long g = (n + 255) / 256;
    return (int)(g < 4 * 152 * 8 ? (g > 0 ? g : 1) : 4 * 152 * 8);
}

} // namespace

// Host u (FP64, reference layout) -> device hi (and lo for FP32K); rejects
// non-finite values with FRGPU_ERR_NONFINITE naming the first bad index.
// The device address of a page-locked (or registered) host array, or null for
// pageable memory: the conversion kernels then read or write the caller's
// array directly over the CPU-GPU link instead of through the staging copy.
static void *mapped(const void *host) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
        cudaGetLastError(); // a pageable pointer is no error here
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

int fr_put_state(frgpu_problem *p, const double *u, void *hi, void *lo) {
    int rc = stage_buffer(p);
    if (rc) return rc;
    double *stage = (double *)p->d_stage;
    unsigned long long *first_bad = reinterpret_cast<unsigned long long *>(stage + p->ndof);
    const unsigned long long none = ~0ull;
    const double *src = (const double *)mapped(u);
    if (!src) {
        FR_CUDA(cudaMemcpyAsync(stage, u, sizeof(double) * (size_t)p->ndof, cudaMemcpyHostToDevice, p->stream));
        src = stage;
    }
    FR_CUDA(cudaMemcpyAsync(first_bad, &none, sizeof(none), cudaMemcpyHostToDevice, p->stream));
    const Layout L = layout_of(p);
    if (L.kind == LAYOUT_E2D) {
        const long nq = L.np * L.np;
        const dim3 grid((unsigned)((L.ne + 255) / 256), (unsigned)nq);
        if (p->esize == 8)
            k_upload_e2d<double><<<grid, 256, 0, p->stream>>>(src, (double *)hi, nullptr, L.ne, nq, first_bad);
        else
            k_upload_e2d<float><<<grid, 256, 0, p->stream>>>(src, (float *)hi, (float *)lo, L.ne, nq, first_bad);
    } else if (p->esize == 8)
        k_upload<double><<<grid_for(p->ndof), 256, 0, p->stream>>>(src, (double *)hi, nullptr, p->ndof, L,
                                                                     first_bad);
    else
        k_upload<float><<<grid_for(p->ndof), 256, 0, p->stream>>>(src, (float *)hi, (float *)lo, p->ndof, L,
                                                                    first_bad);
    FR_CUDA(cudaGetLastError());
    unsigned long long bad = none;
    FR_CUDA(cudaMemcpyAsync(&bad, first_bad, sizeof(bad), cudaMemcpyDeviceToHost, p->stream));
    FR_CUDA(cudaStreamSynchronize(p->stream));
    if (bad != none) {
        fr_set_error("state upload: non-finite value at index " + std::to_string(bad));
        return FRGPU_ERR_NONFINITE;
    }
    return FRGPU_OK;
}

// Device hi (+ lo) -> host u (FP64, reference layout).
int fr_get_state(frgpu_problem *p, const void *hi, const void *lo, double *u) {
    int rc = stage_buffer(p);
    if (rc) return rc;
    double *dst = (double *)mapped(u);
    const bool direct = dst != nullptr;
    double *stage = direct ? dst : (double *)p->d_stage;
    const Layout L = layout_of(p);
    if (L.kind == LAYOUT_E2D) {
        const long nq = L.np * L.np;
        const dim3 grid((unsigned)((L.ne + 255) / 256), (unsigned)nq);
        if (p->esize == 8)
            k_download_e2d<double><<<grid, 256, 0, p->stream>>>((const double *)hi, nullptr, stage, L.ne, nq);
        else
            k_download_e2d<float><<<grid, 256, 0, p->stream>>>((const float *)hi, (const float *)lo, stage, L.ne, nq);
    } else if (p->esize == 8)
        k_download<double><<<grid_for(p->ndof), 256, 0, p->stream>>>((const double *)hi, nullptr, stage, p->ndof, L);
    else
        k_download<float><<<grid_for(p->ndof), 256, 0, p->stream>>>((const float *)hi, (const float *)lo, stage,
                                                                      p->ndof, L);
    FR_CUDA(cudaGetLastError());
    if (!direct)
        FR_CUDA(cudaMemcpyAsync(u, stage, sizeof(double) * (size_t)p->ndof, cudaMemcpyDeviceToHost, p->stream));
    FR_CUDA(cudaStreamSynchronize(p->stream));
    return FRGPU_OK;
}
