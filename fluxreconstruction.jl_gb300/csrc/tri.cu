// tri.cu -- flux reconstruction on unstructured triangles: the residual of
// linear advection u_t + a u_x + a u_y = 0 of dev/wave_triangle.jl:44-125 on
// the operators of TriFRPSpace (src/struct.jl:305-352), with explicit
// Runge-Kutta steps from erk.cu.
//
// Device layout: the state point-major, u[q * ncell + c] (the reference's
// column-major u[ncell, np] as it is); the cell geometry as 8 planes
// (J11, J21, J12, J22, iJ11, iJ21, iJ12, iJ22)[m * ncell + c]; per face f the
// neighbour cell nbc[f * ncell + c] (< 0: boundary face) and per flux point
// (f, k) the neighbour's flat flux point nbp[(f + 3 k) * ncell + c] =
// face' + 3 k'.  One thread per cell: loads of the own solution points and
// of the 3 neighbours' are coalesced across the warp for a mesh numbered
// row by row; the operators sit in shared memory and are read uniformly.
//
// Evaluation order (the oracle's fro_tri_rhs repeats it; this file is built
// with -fmad=false so that FP64 results are bit-identical): 2-vectors
// A x = fma(A12, x2, A11 x1); dot products ascending fma chains from the first
// product; the correction sum over flux points face-fastest.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fr_common.cuh"
#include "frgpu_internal.h"

namespace {

template <class Real> struct TriArgs {
    const Real *u;        // [np][ncell]
    Real *du;             // [np][ncell]
    const Real *ops;      // dl [2][np][np] (dl[j + np q + np np d]), lf [np][3 nfp], phi [np][3 nfp]
    const Real *geo;      // [8][ncell]
    const int *nbc;       // [3][ncell]
    const unsigned char *nbp; // [3 nfp][ncell]
    const unsigned char *active; // [ncell]: 1 where the cell is updated (cell type 0)
    int ncell;
    Real a;
};

template <class Real> __device__ __forceinline__ Real fmaT(Real x, Real y, Real z) { return frk::fmaR<Real>(x, y, z); }

// flux of the cell at its solution points: f = iJ (a u, a u)
template <class Real, int NP>
__device__ __forceinline__ void cell_flux(const TriArgs<Real> &a, unsigned c, Real (&u)[NP], Real (&f1)[NP],
                                          Real (&f2)[NP], Real (&Jc)[4]) {
    const unsigned n = (unsigned)a.ncell;
#pragma unroll
    for (int q = 0; q < NP; ++q) u[q] = __ldg(a.u + (unsigned)q * n + c);
#pragma unroll
    for (int m = 0; m < 4; ++m) Jc[m] = __ldg(a.geo + (unsigned)m * n + c);
    const Real i11 = __ldg(a.geo + 4 * n + c), i21 = __ldg(a.geo + 5 * n + c);
    const Real i12 = __ldg(a.geo + 6 * n + c), i22 = __ldg(a.geo + 7 * n + c);
#pragma unroll
    for (int q = 0; q < NP; ++q) {
        const Real fg = a.a * u[q], gg = a.a * u[q];
        f1[q] = fmaT<Real>(i12, gg, i11 * fg);
        f2[q] = fmaT<Real>(i22, gg, i21 * fg);
    }
}

// FP32: five 128-thread blocks per SM (96 registers, about 180 bytes of spill
// at p = 3) hide the neighbour gathers better than three blocks at the 152
// registers the unbounded build takes (386 against 545 us at 2 M cells, p = 3;
// six blocks at 80 registers spill more: 403 us).  FP64 (206 registers at
// p = 3) keeps two blocks: it is bound by the FP64 pipe, and capping its
// registers spills kilobytes.
template <class Real, int N>
__global__ void __launch_bounds__(128, sizeof(Real) == 4 ? 5 : 1) k_tri_rhs(const TriArgs<Real> a) {
    constexpr int NP = (N + 1) * (N + 2) / 2, NFP = 3 * (N + 1);
    constexpr int NOPS = 2 * NP * NP + 2 * NFP * NP;
    __shared__ Real s_ops[NOPS];
    for (int t = threadIdx.x; t < NOPS; t += blockDim.x) s_ops[t] = a.ops[t];
    __syncthreads();
    const Real *dl = s_ops, *lf = s_ops + 2 * NP * NP, *phi = lf + NFP * NP;
    const unsigned c = blockIdx.x * blockDim.x + threadIdx.x, n = (unsigned)a.ncell;
    if (c >= n) return;
    if (!a.active[c]) {
#pragma unroll
        for (int j = 0; j < NP; ++j) a.du[(unsigned)j * n + c] = Real(0);
        return;
    }
    Real u[NP], f1[NP], f2[NP], J[4];
    cell_flux<Real, NP>(a, c, u, f1, f2, J);
    const Real i11 = __ldg(a.geo + 4 * n + c), i21 = __ldg(a.geo + 5 * n + c);
    const Real i12 = __ldg(a.geo + 6 * n + c), i22 = __ldg(a.geo + 7 * n + c);
    // unit outward normals of the reference faces 1 -> 2, 2 -> 3, 3 -> 1
    const Real nrm[3][2] = {{Real(0), Real(-1)},
                            {Real(0.70710678118654752440), Real(0.70710678118654752440)},
                            {Real(-1), Real(0)}};
    Real d[NFP];
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        const int nb = __ldg(a.nbc + (unsigned)f * n + c);
        Real un[NP], g1[NP], g2[NP], K[4];
        if (nb >= 0) cell_flux<Real, NP>(a, (unsigned)nb, un, g1, g2, K);
#pragma unroll
        for (int k = 0; k < N + 1; ++k) {
            const int fp = f + 3 * k;
            Real uL = u[0] * lf[fp], a1 = f1[0] * lf[fp], a2 = f2[0] * lf[fp];
#pragma unroll
            for (int q = 1; q < NP; ++q) {
                const Real w = lf[fp + NFP * q];
                uL = fmaT<Real>(u[q], w, uL);
                a1 = fmaT<Real>(f1[q], w, a1);
                a2 = fmaT<Real>(f2[q], w, a2);
            }
            const Real fn_face = fmaT<Real>(a2, nrm[f][1], a1 * nrm[f][0]);
            Real fi1 = Real(0), fi2 = Real(0);
            if (nb >= 0) {
                const int p = __ldg(a.nbp + (unsigned)fp * n + c);
                Real uR = un[0] * lf[p], b1 = g1[0] * lf[p], b2 = g2[0] * lf[p];
#pragma unroll
                for (int q = 1; q < NP; ++q) {
                    const Real w = lf[p + NFP * q];
                    uR = fmaT<Real>(un[q], w, uR);
                    b1 = fmaT<Real>(g1[q], w, b1);
                    b2 = fmaT<Real>(g2[q], w, b2);
                }
                const Real fL1 = fmaT<Real>(J[2], a2, J[0] * a1), fL2 = fmaT<Real>(J[3], a2, J[1] * a1);
                const Real fR1 = fmaT<Real>(K[2], b2, K[0] * b1), fR2 = fmaT<Real>(K[3], b2, K[1] * b1);
                const Real jump = uL - uR, den = jump + Real(1e-6);
                const Real au1 = (fL1 - fR1) / den, au2 = (fL2 - fR2) / den;
                fi1 = Real(0.5) * (fL1 + fR1) - Real(0.5) * fabs(au1) * jump;
                fi2 = Real(0.5) * (fL2 + fR2) - Real(0.5) * fabs(au2) * jump;
            }
            const Real h1 = fmaT<Real>(i12, fi2, i11 * fi1), h2 = fmaT<Real>(i22, fi2, i21 * fi1);
            const Real fn_int = fmaT<Real>(h2, nrm[f][1], h1 * nrm[f][0]);
            d[fp] = fn_int - fn_face;
        }
    }
#pragma unroll
    for (int j = 0; j < NP; ++j) {
        Real r1 = f1[0] * dl[j], r2 = f2[0] * dl[j + NP * NP];
#pragma unroll
        for (int q = 1; q < NP; ++q) {
            r1 = fmaT<Real>(f1[q], dl[j + NP * q], r1);
            r2 = fmaT<Real>(f2[q], dl[j + NP * q + NP * NP], r2);
        }
        Real r3 = d[0] * phi[NFP * j];
#pragma unroll
        for (int t = 1; t < NFP; ++t) r3 = fmaT<Real>(d[t], phi[t + NFP * j], r3);
        a.du[(unsigned)j * n + c] = (-r1 - r2) + (-r3);
    }
}

// FP64 host values -> the state's precision; FP32 keeps the rounding residue in lo
template <class Real>
__global__ void __launch_bounds__(256) k_tri_from64(const double *__restrict__ in, Real *__restrict__ hi,
                                                     Real *__restrict__ lo, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const double v = in[q];
        const Real h = (Real)v;
        hi[q] = h;
        if (lo) lo[q] = (Real)(v - (double)h);
    }
}

template <class Real>
__global__ void __launch_bounds__(256) k_tri_to64(const Real *__restrict__ hi, const Real *__restrict__ lo,
                                                   double *__restrict__ out, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        out[q] = lo ? (double)hi[q] + (double)lo[q] : (double)hi[q];
}

int tri_grid(size_t n, int threads) {
    const size_t g = (n + threads - 1) / threads;
    return (int)(g < 152 * 16 ? (g > 0 ? g : 1) : 152 * 16);
}

} // namespace

struct frgpu_tri {
    int ncell = 0, deg = 0, np = 0, nfp = 0, precision = FRGPU_FP64;
    double a = 0;
    size_t esize = 8, ndof = 0;
    cudaStream_t stream = nullptr;
    void *u = nullptr, *lo = nullptr; // state (high part) and FP32 low part
    void *ops = nullptr, *geo = nullptr;
    int *nbc = nullptr;
    unsigned char *nbp = nullptr, *active = nullptr;
    double *d_host64 = nullptr;       // FP64 staging for host transfers
    char *kbuf = nullptr;             // ERK stage derivatives + stage input
    size_t kcap = 0;
    double *d_dt = nullptr;
    int *d_status = nullptr;
    long launches = 0;
    // cached graph of one ERK step
    std::vector<double> gA, gb;
    cudaGraphExec_t gexec = nullptr;
    long graph_launches = 0;
};

namespace {

#define TRI_REQ(cond, msg)                                                                                         \
    do {                                                                                                           \
        if (!(cond)) {                                                                                             \
            fr_set_error(msg);                                                                                     \
            return FRGPU_ERR_ARG;                                                                                  \
        }                                                                                                          \
    } while (0)

template <class Real, int N> int launch_rhs_n(frgpu_tri *t, const void *in, void *out) {
    TriArgs<Real> a;
    a.u = (const Real *)in;
    a.du = (Real *)out;
    a.ops = (const Real *)t->ops;
    a.geo = (const Real *)t->geo;
    a.nbc = t->nbc;
    a.nbp = t->nbp;
    a.active = t->active;
    a.ncell = t->ncell;
    a.a = (Real)t->a;
    k_tri_rhs<Real, N><<<(t->ncell + 127) / 128, 128, 0, t->stream>>>(a);
    FR_CUDA(cudaGetLastError());
    t->launches += 1;
    return FRGPU_OK;
}

template <class Real> int launch_rhs_t(frgpu_tri *t, const void *in, void *out) {
    switch (t->deg) {
    case 1: return launch_rhs_n<Real, 1>(t, in, out);
    case 2: return launch_rhs_n<Real, 2>(t, in, out);
    case 3: return launch_rhs_n<Real, 3>(t, in, out);
    default: break;
    }
    fr_set_error("triangles: degree not built (1..3)");
    return FRGPU_ERR_UNSUPPORTED;
}

int tri_residual(void *ctx, const void *in, void *out) {
    frgpu_tri *t = (frgpu_tri *)ctx;
    return t->precision == FRGPU_FP32K ? launch_rhs_t<float>(t, in, out) : launch_rhs_t<double>(t, in, out);
}

// host FP64 values -> device buffer dst (and lo) in the state's precision
int upload64(frgpu_tri *t, const double *h, void *dst, void *lo) {
    FR_CUDA(cudaMemcpyAsync(t->d_host64, h, sizeof(double) * t->ndof, cudaMemcpyHostToDevice, t->stream));
    if (t->precision == FRGPU_FP32K)
        k_tri_from64<float><<<tri_grid(t->ndof, 256), 256, 0, t->stream>>>(t->d_host64, (float *)dst, (float *)lo,
                                                                          t->ndof);
    else
        k_tri_from64<double><<<tri_grid(t->ndof, 256), 256, 0, t->stream>>>(t->d_host64, (double *)dst, nullptr,
                                                                           t->ndof);
    FR_CUDA(cudaGetLastError());
    return FRGPU_OK;
}

int download64(frgpu_tri *t, const void *src, const void *lo, double *h) {
    if (t->precision == FRGPU_FP32K)
        k_tri_to64<float><<<tri_grid(t->ndof, 256), 256, 0, t->stream>>>((const float *)src, (const float *)lo,
                                                                        t->d_host64, t->ndof);
    else
        k_tri_to64<double><<<tri_grid(t->ndof, 256), 256, 0, t->stream>>>((const double *)src, nullptr, t->d_host64,
                                                                         t->ndof);
    FR_CUDA(cudaGetLastError());
    FR_CUDA(cudaMemcpyAsync(h, t->d_host64, sizeof(double) * t->ndof, cudaMemcpyDeviceToHost, t->stream));
    FR_CUDA(cudaStreamSynchronize(t->stream));
    return FRGPU_OK;
}

int ensure_kbuf(frgpu_tri *t, int s) {
    const size_t need = (size_t)(s + 1) * t->ndof * t->esize;
    if (t->kcap >= need) return FRGPU_OK;
    if (t->kbuf) cudaFree(t->kbuf);
    t->kbuf = nullptr;
    t->kcap = 0;
    if (t->gexec) cudaGraphExecDestroy(t->gexec);
    t->gexec = nullptr;
    FR_CUDA(cudaMalloc(&t->kbuf, need));
    t->kcap = need;
    return FRGPU_OK;
}

template <class T> int upload_plain(void **dst, const T *h, size_t n) {
    FR_CUDA(cudaMalloc(dst, sizeof(T) * n));
    FR_CUDA(cudaMemcpy(*dst, h, sizeof(T) * n, cudaMemcpyHostToDevice));
    return FRGPU_OK;
}

// doubles -> device array in the state's precision
int upload_real(frgpu_tri *t, void **dst, const std::vector<double> &h) {
    if (t->esize == 8) return upload_plain<double>(dst, h.data(), h.size());
    try {
        std::vector<float> f(h.begin(), h.end());
        return upload_plain<float>(dst, f.data(), f.size());
    } catch (const std::exception &e) {
        fr_set_error(e.what());
        return FRGPU_ERR_ARG;
    }
}

void free_tri(frgpu_tri *t) {
    if (!t) return;
    if (t->gexec) cudaGraphExecDestroy(t->gexec);
    for (void *b : {(void *)t->u, t->lo, t->ops, t->geo, (void *)t->nbc, (void *)t->nbp, (void *)t->active,
                    (void *)t->d_host64, (void *)t->kbuf, (void *)t->d_dt, (void *)t->d_status})
        if (b) cudaFree(b);
    if (t->stream) cudaStreamDestroy(t->stream);
    delete t;
}

} // namespace

extern "C" {

FRGPU_API int frgpu_vandermonde_tri(int deg, const double *r, const double *s, int n, double *V, double *Vr,
                                    double *Vs) {
    TRI_REQ(deg >= 0 && deg <= 16 && n > 0 && r && s, "vandermonde_tri: bad arguments");
    try {
        frsetup::vandermonde_tri(deg, r, s, n, V, Vr, Vs);
    } catch (const std::exception &e) {
        fr_set_error(e.what());
        return FRGPU_ERR_ARG;
    }
    return FRGPU_OK;
}

FRGPU_API int frgpu_tri_operators(int deg, const double *r, const double *s, double *V, double *dl, double *lf,
                                  double *phi) {
    TRI_REQ(deg >= 1 && deg <= 16 && r && s, "tri_operators: bad arguments");
    try {
        frsetup::tri_operators(deg, r, s, V, dl, lf, phi);
    } catch (const std::exception &e) {
        fr_set_error(e.what());
        return FRGPU_ERR_ARG;
    }
    return FRGPU_OK;
}

static int tri_create_impl(int ncell, int deg, int precision, double a, const double *dl, const double *lf,
                           const double *phi, const double *J, const double *iJ, const int *nb_cell,
                           const int *nb_face, const int *nb_point, const int *cell_type, frgpu_tri **out) {
    TRI_REQ(out, "tri_create: null output handle");
    *out = nullptr;
    TRI_REQ(ncell > 0 && ncell <= (1 << 26), "tri_create: ncell must be in 1..2^26");
    TRI_REQ(deg >= 1 && deg <= 3, "tri_create: degree must be 1, 2 or 3");
    TRI_REQ(precision == FRGPU_FP64 || precision == FRGPU_FP32K, "tri_create: unknown precision");
    TRI_REQ(std::isfinite(a), "tri_create: non-finite advection speed");
    TRI_REQ(dl && lf && phi && J && iJ && nb_cell && nb_face && nb_point && cell_type, "tri_create: null array");
    const int np = (deg + 1) * (deg + 2) / 2, nfp = deg + 1, nf = 3 * nfp;
    const size_t nc = (size_t)ncell;
    // neighbours: one cell per face, faces 0..2, points 0..nfp-1, in range
    std::vector<int> nbc(3 * nc, -1);
    std::vector<unsigned char> nbp(nf * nc, 0), active(nc);
    for (size_t c = 0; c < nc; ++c) {
        active[c] = cell_type[c] == 0;
        for (int f = 0; f < 3; ++f)
            for (int k = 0; k < nfp; ++k) {
                const size_t i = c + nc * (f + 3 * (size_t)k);
                const int n = nb_cell[i];
                if (k == 0)
                    nbc[f * nc + c] = n < 0 ? -1 : n;
                else
                    TRI_REQ((n < 0 ? -1 : n) == nbc[f * nc + c], "tri_create: flux points of one face name different neighbour cells");
                if (n < 0) continue;
                TRI_REQ(n < ncell, "tri_create: neighbour cell out of range");
                TRI_REQ(nb_face[i] >= 0 && nb_face[i] < 3 && nb_point[i] >= 0 && nb_point[i] < nfp,
                        "tri_create: neighbour flux point out of range");
                nbp[(f + 3 * (size_t)k) * nc + c] = (unsigned char)(nb_face[i] + 3 * nb_point[i]);
            }
    }
    std::vector<double> ops;
    ops.insert(ops.end(), dl, dl + 2 * np * np);
    ops.insert(ops.end(), lf, lf + nf * np);
    ops.insert(ops.end(), phi, phi + nf * np);
    std::vector<double> geo(8 * nc);
    for (int m = 0; m < 4; ++m)
        for (size_t c = 0; c < nc; ++c) {
            geo[m * nc + c] = J[c + nc * m];
            geo[(4 + m) * nc + c] = iJ[c + nc * m];
        }
    for (double v : ops) TRI_REQ(std::isfinite(v), "tri_create: non-finite operator value");
    for (double v : geo) TRI_REQ(std::isfinite(v), "tri_create: non-finite Jacobian value");
    frgpu_tri *t = new frgpu_tri;
    t->ncell = ncell;
    t->deg = deg;
    t->np = np;
    t->nfp = nfp;
    t->precision = precision;
    t->a = a;
    t->esize = precision == FRGPU_FP32K ? 4 : 8;
    t->ndof = nc * np;
    int rc = FRGPU_OK;
    auto fail = [&](int r) {
        free_tri(t);
        return r;
    };
    if (cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(fr_cuda_fail(cudaGetLastError(), "tri_create: stream"));
    if ((rc = upload_real(t, &t->ops, ops)) || (rc = upload_real(t, &t->geo, geo)) ||
        (rc = upload_plain<int>((void **)&t->nbc, nbc.data(), nbc.size())) ||
        (rc = upload_plain<unsigned char>((void **)&t->nbp, nbp.data(), nbp.size())) ||
        (rc = upload_plain<unsigned char>((void **)&t->active, active.data(), active.size())))
        return fail(rc);
    cudaError_t e;
    if ((e = cudaMalloc(&t->u, t->ndof * t->esize)) != cudaSuccess ||
        (e = cudaMemset(t->u, 0, t->ndof * t->esize)) != cudaSuccess ||
        (e = cudaMalloc((void **)&t->d_host64, sizeof(double) * t->ndof)) != cudaSuccess ||
        (e = cudaMalloc((void **)&t->d_dt, sizeof(double))) != cudaSuccess ||
        (e = cudaMalloc((void **)&t->d_status, sizeof(int))) != cudaSuccess ||
        (e = cudaMemset(t->d_status, 0, sizeof(int))) != cudaSuccess)
        return fail(fr_cuda_fail(e, "tri_create: allocation"));
    if (precision == FRGPU_FP32K) {
        if ((e = cudaMalloc(&t->lo, t->ndof * t->esize)) != cudaSuccess ||
            (e = cudaMemset(t->lo, 0, t->ndof * t->esize)) != cudaSuccess)
            return fail(fr_cuda_fail(e, "tri_create: allocation"));
    }
    *out = t;
    return FRGPU_OK;
}

// host allocations may throw: no exception crosses the C ABI
FRGPU_API int frgpu_tri_create(int ncell, int deg, int precision, double a, const double *dl, const double *lf,
                               const double *phi, const double *J, const double *iJ, const int *nb_cell,
                               const int *nb_face, const int *nb_point, const int *cell_type, frgpu_tri **out) {
    try {
        return tri_create_impl(ncell, deg, precision, a, dl, lf, phi, J, iJ, nb_cell, nb_face, nb_point, cell_type,
                               out);
    } catch (const std::exception &e) {
        fr_set_error(std::string("tri_create: ") + e.what());
        return FRGPU_ERR_ARG;
    }
}

FRGPU_API int frgpu_tri_destroy(frgpu_tri *t) {
    if (t) {
        cudaStreamSynchronize(t->stream);
        free_tri(t);
    }
    return FRGPU_OK;
}

/* state u[ncell, np] (host FP64, column-major) */
FRGPU_API int frgpu_tri_set_state(frgpu_tri *t, const double *u) {
    TRI_REQ(t && u, "tri_set_state: null argument");
    for (size_t q = 0; q < t->ndof; ++q) TRI_REQ(std::isfinite(u[q]), "tri_set_state: non-finite value in the state");
    int rc = upload64(t, u, t->u, t->lo);
    if (rc) return rc;
    FR_CUDA(cudaStreamSynchronize(t->stream));
    return FRGPU_OK;
}

FRGPU_API int frgpu_tri_get_state(frgpu_tri *t, double *u) {
    TRI_REQ(t && u, "tri_get_state: null argument");
    return download64(t, t->u, t->lo, u);
}

/* du = L(u) for a host state: the dudt!(du, u, p, t) call of dev/wave_triangle.jl:44 */
FRGPU_API int frgpu_tri_rhs(frgpu_tri *t, double *du, const double *u) {
    TRI_REQ(t && du && u, "tri_rhs: null argument");
    int rc;
    if ((rc = ensure_kbuf(t, 1))) return rc;
    char *in = t->kbuf + t->ndof * t->esize;
    if ((rc = upload64(t, u, in, nullptr))) return rc;
    if ((rc = tri_residual(t, in, t->kbuf))) return rc;
    return download64(t, t->kbuf, nullptr, du);
}

/* The residual of the device state into a device scratch buffer, on the
 * object's stream, without a host round trip (for timing). */
FRGPU_API int frgpu_tri_rhs_device(frgpu_tri *t) {
    TRI_REQ(t, "tri_rhs_device: null argument");
    int rc;
    if ((rc = ensure_kbuf(t, 1))) return rc;
    return tri_residual(t, t->u, t->kbuf);
}

/* nsteps fixed steps of the explicit Runge-Kutta method (A, b) (row-major
 * s x s A, strictly lower triangular) on the device state: init(prob, alg;
 * dt, adaptive=false) + step! of OrdinaryDiffEq as dev/wave_triangle.jl:131-135
 * drives it (Euler: s = 1, A = 0, b = 1). */
static int tri_step_impl(frgpu_tri *t, int s, const double *A, const double *b, double dt, int nsteps) {
    TRI_REQ(t && A && b, "tri_step_erk: null argument");
    TRI_REQ(s >= 1 && s <= FR_ERK_MAXS, "tri_step_erk: stages must be in 1..16");
    TRI_REQ(nsteps >= 0, "tri_step_erk: negative step count");
    if (!(dt > 0.0) || !std::isfinite(dt)) {
        fr_set_error("tri_step_erk: dt must be positive and finite");
        return FRGPU_ERR_DT;
    }
    for (int i = 0; i < s; ++i)
        for (int j = 0; j < s; ++j) {
            TRI_REQ(std::isfinite(A[i * s + j]), "tri_step_erk: non-finite tableau entry");
            TRI_REQ(j < i || A[i * s + j] == 0.0, "tri_step_erk: the tableau must be explicit");
        }
    for (int j = 0; j < s; ++j) TRI_REQ(std::isfinite(b[j]), "tri_step_erk: non-finite weight");
    if (nsteps == 0) return FRGPU_OK;
    int rc;
    if ((rc = ensure_kbuf(t, s))) return rc;
    FR_CUDA(cudaMemcpyAsync(t->d_dt, &dt, sizeof(double), cudaMemcpyHostToDevice, t->stream));
    FR_CUDA(cudaStreamSynchronize(t->stream));
    std::vector<double> vA(A, A + (size_t)s * s), vb(b, b + s);
    if (!t->gexec || vA != t->gA || vb != t->gb) {
        if (t->gexec) cudaGraphExecDestroy(t->gexec);
        t->gexec = nullptr;
        fr_erk_raw r;
        r.stream = t->stream;
        r.s = s;
        r.A = vA.data();
        r.b = vb.data();
        r.n = t->ndof;
        r.f32 = t->precision == FRGPU_FP32K;
        r.u = t->u;
        r.lo = t->lo;
        r.kbuf = t->kbuf;
        r.esize = t->esize;
        r.d_dt = t->d_dt;
        r.d_status = t->d_status;
        r.prepare_only = false;
        long before = t->launches;
        r.launches = &t->launches;
        cudaGraph_t g;
        FR_CUDA(cudaStreamBeginCapture(t->stream, cudaStreamCaptureModeThreadLocal));
        rc = fr_erk_enqueue_raw(r, tri_residual, t);
        cudaError_t e = cudaStreamEndCapture(t->stream, &g);
        if (rc) {
            if (e == cudaSuccess) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return fr_cuda_fail(e, "tri_step_erk: capture");
        e = cudaGraphInstantiate(&t->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fr_cuda_fail(e, "tri_step_erk: instantiate");
        t->graph_launches = t->launches - before;
        t->launches = before;
        t->gA = vA;
        t->gb = vb;
    }
    for (int it = 0; it < nsteps; ++it) {
        FR_CUDA(cudaGraphLaunch(t->gexec, t->stream));
        t->launches += t->graph_launches;
    }
    int st = 0;
    FR_CUDA(cudaMemcpyAsync(&st, t->d_status, sizeof(int), cudaMemcpyDeviceToHost, t->stream));
    FR_CUDA(cudaStreamSynchronize(t->stream));
    if (st) {
        FR_CUDA(cudaMemset(t->d_status, 0, sizeof(int)));
        fr_set_error("tri_step_erk: non-finite value in the state");
        return FRGPU_ERR_NONFINITE;
    }
    return FRGPU_OK;
}

FRGPU_API int frgpu_tri_step_erk(frgpu_tri *t, int s, const double *A, const double *b, double dt, int nsteps) {
    try {
        return tri_step_impl(t, s, A, b, dt, nsteps);
    } catch (const std::exception &e) {
        fr_set_error(std::string("tri_step_erk: ") + e.what());
        return FRGPU_ERR_ARG;
    }
}

FRGPU_API int frgpu_tri_stream(frgpu_tri *t, void **stream) {
    TRI_REQ(t && stream, "tri_stream: null argument");
    *stream = (void *)t->stream;
    return FRGPU_OK;
}

/* kernels enqueued so far (graph replays count their kernels) */
FRGPU_API int frgpu_tri_launches(frgpu_tri *t, long long *n) {
    TRI_REQ(t && n, "tri_launches: null argument");
    *n = t->launches;
    return FRGPU_OK;
}

} // extern "C"
