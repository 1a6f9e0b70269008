// limiter.cu -- positivity-preserving limiter of src/dissipation.jl:38-216
// (Vandenhoeck & Lani 2019) on the device state, one thread per element.
//
// Euler forms (1D: dissipation.jl:61-121, 2D: :125-206): the weighted element
// mean u_mean (weights summing to 1), eps = min(1e-13, rho_mean, p_mean), the
// density scaling t1 = min((rho_mean - eps) / (rho_mean - rho_min + 1e-8), 1)
// with rho_min over the solution points and the face points, applied to the
// density; then every face point (state before the density scaling, as in the
// reference) and every solution point whose lambda = rho / (2 p) is below eps
// gives the t at which p(t (u - u_mean) + u_mean) = eps, and all variables are
// scaled by t2 = min(t_j, t0).  Where the reference calls min(tj, t0) in a form
// that throws, this takes the minimum; p(t) = eps is solved in closed form
// (p rho is quadratic in t; the root in [0, 1] nearest to 1) rather than by the
// reference's Newton iteration.  The 2D means cover all 4 variables (the
// reference's loop over axes(u, 2) does so only when np = 4).
// Scalar form (dissipation.jl:38-58): mean = sum(u w) / sum(w), theta over the
// two face traces and the solution points.
//
// FP64 applies the density formula to every element, as the reference does
// (t1 = 1 still rounds (u - mean) + mean), and is bit-identical to the oracle.
// FP32K decides on the high part, and rewrites an element (high part, low part
// cleared) only when a parameter is below 1, so untouched elements keep their
// compensated low part.
#include <string>

#include "fr_common.cuh"
#include "frgpu_internal.h"

using namespace frk;

namespace {

constexpr int LIM_MAXQ = FR_MAXNP * FR_MAXNP;

template <class Real> struct LimArgs {
    Real ll[FR_MAXNP], lr[FR_MAXNP];
    Real w[LIM_MAXQ]; // element quadrature weights (sum 1); scalar form: raw weights
    Real gamma, t0;
};

// conserve_prim's lambda = rho / (2 p) of a state of NV variables (FP64: IEEE
// divisions in the reference's order; FP32: the hardware reciprocal, 2 ulp)
template <class Real, int NV> __device__ __forceinline__ Real lim_lambda(const Real (&w)[4], Real g) {
    Real kin = fmaR<Real>(w[1], w[1], Real(0));
    if (NV == 4) kin = fmaR<Real>(w[2], w[2], kin);
    return divR<Real>(divR<Real>(Real(0.5) * w[0], g - Real(1)), w[NV - 1] - divR<Real>(Real(0.5) * kin, w[0]));
}

// root in [0, 1] nearest to 1 of a t^2 + b t + c; 1 when there is none
template <class Real> __device__ __forceinline__ Real lim_root(Real a, Real b, Real c) {
    Real r = Real(1);
    if (fabs(a) <= Real(sizeof(Real) == 8 ? 1e-300 : 1e-37)) {
        if (b != Real(0)) r = -c / b;
    } else {
        const Real disc = b * b - Real(4) * a * c;
        if (disc >= Real(0)) {
            const Real q = Real(-0.5) * (b + copysign(sqrt(disc), b));
            const Real r1 = q / a, r2 = q != Real(0) ? c / q : r1;
            const bool ok1 = r1 >= Real(0) && r1 <= Real(1), ok2 = r2 >= Real(0) && r2 <= Real(1);
            if (ok1 && ok2) r = r1 > r2 ? r1 : r2;
            else if (ok1) r = r1;
            else if (ok2) r = r2;
        }
    }
    return r < Real(0) ? Real(0) : (r > Real(1) ? Real(1) : r);
}

// t with p(t) = eps on the segment from the mean um to the state w:
// (gamma - 1)(2 E rho - |m|^2) - 2 eps rho = a t^2 + b t + c
template <class Real, int NV>
__device__ __forceinline__ Real lim_t(const Real (&w)[4], const Real (&um)[4], Real g, Real eps) {
    const Real gm1 = g - Real(1);
    constexpr int IE = NV - 1;
    const Real dr = w[0] - um[0], de = w[IE] - um[IE];
    Real dm2 = Real(0), mdm = Real(0), mm = Real(0);
#pragma unroll
    for (int v = 1; v < IE; ++v) {
        const Real dm = w[v] - um[v];
        dm2 = fmaR<Real>(dm, dm, dm2);
        mdm = fmaR<Real>(um[v], dm, mdm);
        mm = fmaR<Real>(um[v], um[v], mm);
    }
    const Real a = gm1 * (Real(2) * de * dr - dm2);
    const Real b = gm1 * (Real(2) * (um[IE] * dr + de * um[0]) - Real(2) * mdm) - Real(2) * eps * dr;
    const Real c = gm1 * (Real(2) * um[IE] * um[0] - mm) - Real(2) * eps * um[0];
    return lim_root<Real>(a, b, c);
}

// One Euler element of NQ solution points held in v[q][var] (NV variables);
// face point f is the trace along line (base fb[f], stride fs[f] in q) with
// weights fl[f] (ll or lr).  Returns 1 when scaled with a parameter below 1,
// 0 when not, -1 when t1 left (0, 1].
template <class Real, int NP, int NQ, int NV, int NF>
__device__ __forceinline__ int lim_element(Real (&v)[NQ][4], const LimArgs<Real> &a, const int (&fb)[NF],
                                           const int (&fs)[NF], const bool (&fr)[NF]) {
    const Real g = a.gamma;
    Real um[4] = {Real(0), Real(0), Real(0), Real(0)};
#pragma unroll
    for (int m = 0; m < NV; ++m) {
        Real s = v[0][m] * a.w[0];
#pragma unroll
        for (int q = 1; q < NQ; ++q) s = fmaR<Real>(v[q][m], a.w[q], s);
        um[m] = s;
    }
    const Real lm = lim_lambda<Real, NV>(um, g);
    const Real pm = Real(0.5) * um[0] * (Real(1) / lm);
    Real eps = Real(1e-13);
    if (um[0] < eps) eps = um[0];
    if (pm < eps) eps = pm;
    // density at the face points, before the density scaling
    Real rb[NF];
    Real rmin = Real(INFINITY);
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        const Real *wl = fr[f] ? a.lr : a.ll;
        Real s = v[fb[f]][0] * wl[0];
#pragma unroll
        for (int r = 1; r < NP; ++r) s = fmaR<Real>(v[fb[f] + r * fs[f]][0], wl[r], s);
        rb[f] = s;
        if (s < rmin) rmin = s;
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q)
        if (v[q][0] < rmin) rmin = v[q][0];
    // t1 < 1 exactly when rho_min < eps + 1e-8.  FP32 tests that directly: the
    // FP32 mean of a uniform density can exceed its point values by an ulp
    // (6e-8 at rho = 1), more than the formula's 1e-8 guard absorbs.
    Real t1 = Real(1);
    if (sizeof(Real) == 8 || !(rmin >= eps + Real(1e-8))) {
        t1 = (um[0] - eps) / (um[0] - rmin + Real(1e-8));
        if (t1 > Real(1)) t1 = Real(1);
    }
    if (!(t1 > Real(0))) return -1;
#pragma unroll
    for (int q = 0; q < NQ; ++q) v[q][0] = t1 * (v[q][0] - um[0]) + um[0];
    // energy: face points (stale density, unchanged other variables), then
    // solution points
    Real t2 = a.t0;
    bool found = false;
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        const Real *wl = fr[f] ? a.lr : a.ll;
        Real wf[4] = {rb[f], Real(0), Real(0), Real(0)};
#pragma unroll
        for (int m = 1; m < NV; ++m) {
            Real s = v[fb[f]][m] * wl[0];
#pragma unroll
            for (int r = 1; r < NP; ++r) s = fmaR<Real>(v[fb[f] + r * fs[f]][m], wl[r], s);
            wf[m] = s;
        }
        if (lim_lambda<Real, NV>(wf, g) < eps) {
            const Real t = lim_t<Real, NV>(wf, um, g, eps);
            if (t < t2) t2 = t;
            found = true;
        }
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q)
        if (lim_lambda<Real, NV>(v[q], g) < eps) {
            const Real t = lim_t<Real, NV>(v[q], um, g, eps);
            if (t < t2) t2 = t;
            found = true;
        }
    if (found)
#pragma unroll
        for (int m = 0; m < NV; ++m)
#pragma unroll
            for (int q = 0; q < NQ; ++q) v[q][m] = t2 * (v[q][m] - um[m]) + um[m];
    return (t1 < Real(1) || (found && t2 < Real(1))) ? 1 : 0;
}

// 2D Euler, state in the point-vector device layout.  Face points in the
// reference's order (dissipation.jl:143-161): for j = 0..np-1 the bottom face
// of column j (along s, ll), the right face of row j (along r, lr), the top
// face of column j (lr), the left face of row j (ll).
template <class Real, int NP, bool FP32K>
__global__ void __launch_bounds__(128) k_limiter2d(Real *__restrict__ u, Real *__restrict__ lo, size_t ne,
                                                   const LimArgs<Real> a, int *status, int *count) {
    constexpr int NQ = NP * NP, NF = 4 * NP;
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    Real v[NQ][4];
#pragma unroll
    for (int q = 0; q < NQ; ++q) ld4(u + e2d_index(e, q, 0, ne), v[q]);
    int fb[NF], fs[NF];
    bool fr[NF];
#pragma unroll
    for (int j = 0; j < NP; ++j) {
        fb[4 * j + 0] = j; fs[4 * j + 0] = NP; fr[4 * j + 0] = false;
        fb[4 * j + 1] = NP * j; fs[4 * j + 1] = 1; fr[4 * j + 1] = true;
        fb[4 * j + 2] = j; fs[4 * j + 2] = NP; fr[4 * j + 2] = true;
        fb[4 * j + 3] = NP * j; fs[4 * j + 3] = 1; fr[4 * j + 3] = false;
    }
    const int r = lim_element<Real, NP, NQ, 4, NF>(v, a, fb, fs, fr);
    if (r < 0) {
        atomicOr(status, ST_UNPHYSICAL);
        return;
    }
    if (FP32K && r == 0) return;
#pragma unroll
    for (int q = 0; q < NQ; ++q) st4(u + e2d_index(e, q, 0, ne), v[q]);
    if (FP32K && lo) {
        const Real z[4] = {Real(0), Real(0), Real(0), Real(0)};
#pragma unroll
        for (int q = 0; q < NQ; ++q) st4(lo + e2d_index(e, q, 0, ne), z);
    }
    if (r > 0) atomicAdd(count, 1);
}

// FP32K 2D form with np <= 4, four lanes per element: lane l holds row l
// (points k + np l).  Means, column-face traces and the minima are reduced
// across the lane quad with shuffles; lane l tests the faces of row l and of
// column l.  Same decisions as lim_element (sums in another order, FP32).
template <int NP>
__global__ void __launch_bounds__(128) k_limiter2d_rows(float *__restrict__ u, float *__restrict__ lo, size_t ne,
                                                        const LimArgs<float> a, int *status, int *count) {
    static_assert(NP <= 4, "four lanes per element");
    const unsigned FULL = 0xffffffffu;
    const int l = threadIdx.x & 3;
    const size_t e = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 2;
    const bool act = e < ne && l < NP;
    const float g = a.gamma;
    float v[NP][4];
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        v[k][0] = v[k][1] = v[k][2] = v[k][3] = 0.f;
        if (act) ld4(u + e2d_index(e, k + NP * l, 0, ne), v[k]);
    }
    auto qsum = [&](float x) {
        x += __shfl_xor_sync(FULL, x, 1);
        return x + __shfl_xor_sync(FULL, x, 2);
    };
    auto qmin = [&](float x) {
        x = fminf(x, __shfl_xor_sync(FULL, x, 1));
        return fminf(x, __shfl_xor_sync(FULL, x, 2));
    };
    // means
    float um[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < NP; ++k) s = fmaf(v[k][m], act ? a.w[k + NP * l] : 0.f, s);
        um[m] = qsum(s);
    }
    const float lm = lim_lambda<float, 4>(um, g);
    const float pm = 0.5f * um[0] * (1.f / lm);
    float eps = 1e-13f;
    if (um[0] < eps) eps = um[0];
    if (pm < eps) eps = pm;
    // face points before the density scaling: left / right of row l (own),
    // bottom / top of every column (quad sums), of which lane l keeps column l
    float fL[4], fR[4], fB[4], fT[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        float sl = 0.f, sr = 0.f;
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            sl = fmaf(v[k][m], a.ll[k], sl);
            sr = fmaf(v[k][m], a.lr[k], sr);
        }
        fL[m] = sl;
        fR[m] = sr;
        fB[m] = fT[m] = 0.f;
    }
    const float wl = act ? a.ll[l] : 0.f, wr = act ? a.lr[l] : 0.f;
    float rmin = INFINITY;
#pragma unroll
    for (int j = 0; j < NP; ++j)
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const float b = qsum(v[j][m] * wl), t = qsum(v[j][m] * wr);
            if (j == l) {
                fB[m] = b;
                fT[m] = t;
            }
            if (m == 0) rmin = fminf(rmin, fminf(b, t));
        }
    if (act) {
        rmin = fminf(rmin, fminf(fL[0], fR[0]));
#pragma unroll
        for (int k = 0; k < NP; ++k) rmin = fminf(rmin, v[k][0]);
    }
    rmin = qmin(rmin);
    float t1 = 1.f;
    if (!(rmin >= eps + 1e-8f)) { // see lim_element
        t1 = (um[0] - eps) / (um[0] - rmin + 1e-8f);
        if (t1 > 1.f) t1 = 1.f;
    }
    // every lane of the warp takes part in the shuffles below: a failed
    // element is flagged and left unchanged, not left early
    const bool failed = !(t1 > 0.f);
    if (failed) {
        if (act && l == 0) atomicOr(status, ST_UNPHYSICAL);
        t1 = 1.f;
    }
#pragma unroll
    for (int k = 0; k < NP; ++k) v[k][0] = t1 * (v[k][0] - um[0]) + um[0];
    float t2 = a.t0;
    float found = 0.f;
    if (act) {
        const float *faces[4] = {fL, fR, fB, fT};
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            float wf[4] = {faces[f][0], faces[f][1], faces[f][2], faces[f][3]};
            if (lim_lambda<float, 4>(wf, g) < eps) {
                t2 = fminf(t2, lim_t<float, 4>(wf, um, g, eps));
                found = 1.f;
            }
        }
#pragma unroll
        for (int k = 0; k < NP; ++k)
            if (lim_lambda<float, 4>(v[k], g) < eps) {
                t2 = fminf(t2, lim_t<float, 4>(v[k], um, g, eps));
                found = 1.f;
            }
    }
    t2 = qmin(t2);
    found = -qmin(-found);
    const bool fnd = found > 0.f;
    if (failed || !(t1 < 1.f || (fnd && t2 < 1.f))) return; // after the last shuffle
    if (fnd)
#pragma unroll
        for (int k = 0; k < NP; ++k)
#pragma unroll
            for (int m = 0; m < 4; ++m) v[k][m] = t2 * (v[k][m] - um[m]) + um[m];
    if (!act) return;
    const float z[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        st4(u + e2d_index(e, k + NP * l, 0, ne), v[k]);
        if (lo) st4(lo + e2d_index(e, k + NP * l, 0, ne), z);
    }
    if (l == 0) atomicAdd(count, 1);
}

// 1D Euler, u[e + ne (q + np m)]
template <class Real, int NP, bool FP32K>
__global__ void __launch_bounds__(128) k_limiter1d(Real *__restrict__ u, Real *__restrict__ lo, size_t ne,
                                                   const LimArgs<Real> a, int *status, int *count) {
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    Real v[NP][4];
#pragma unroll
    for (int q = 0; q < NP; ++q) {
#pragma unroll
        for (int m = 0; m < 3; ++m) v[q][m] = u[e + ne * (q + NP * m)];
        v[q][3] = Real(0);
    }
    const int fb[2] = {0, 0}, fs[2] = {1, 1};
    const bool fr[2] = {false, true};
    const int r = lim_element<Real, NP, NP, 3, 2>(v, a, fb, fs, fr);
    if (r < 0) {
        atomicOr(status, ST_UNPHYSICAL);
        return;
    }
    if (FP32K && r == 0) return;
#pragma unroll
    for (int q = 0; q < NP; ++q)
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            u[e + ne * (q + NP * m)] = v[q][m];
            if (FP32K && lo) lo[e + ne * (q + NP * m)] = Real(0);
        }
    if (r > 0) atomicAdd(count, 1);
}

// scalar (advection, Burgers), u[e + ne q]
template <class Real, int NP, bool FP32K>
__global__ void __launch_bounds__(128) k_limiter_scalar(Real *__restrict__ u, Real *__restrict__ lo, size_t ne,
                                                        const LimArgs<Real> a, int *status, int *count) {
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    Real v[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) v[q] = u[e + ne * q];
    Real sw = a.w[0];
#pragma unroll
    for (int q = 1; q < NP; ++q) sw += a.w[q];
    const Real um = dotw<Real, NP>(v, a.w) / sw;
    const Real ub0 = dotw<Real, NP>(v, a.ll), ub1 = dotw<Real, NP>(v, a.lr);
    Real eps = Real(1e-13);
    if (um < eps) eps = um;
    Real th = ub0 < ub1 ? ub0 : ub1;
#pragma unroll
    for (int q = 0; q < NP; ++q)
        if (v[q] < th) th = v[q];
    Real t = Real(1);
    if (sizeof(Real) == 8 || !(th >= eps + Real(1e-8))) { // see lim_element
        t = (um - eps) / (um - th + Real(1e-8));
        if (t > Real(1)) t = Real(1);
    }
    if (!(t > Real(0))) {
        atomicOr(status, ST_UNPHYSICAL);
        return;
    }
    if (FP32K && !(t < Real(1))) return;
#pragma unroll
    for (int q = 0; q < NP; ++q) {
        u[e + ne * q] = t * (v[q] - um) + um;
        if (FP32K && lo) lo[e + ne * q] = Real(0);
    }
    if (t < Real(1)) atomicAdd(count, 1);
}

template <class Real> LimArgs<Real> lim_args(const frgpu_problem *p, const std::vector<double> &w, double t0) {
    LimArgs<Real> a;
    for (int k = 0; k < FR_MAXNP; ++k) a.ll[k] = a.lr[k] = Real(0);
    for (int q = 0; q < LIM_MAXQ; ++q) a.w[q] = Real(0);
    for (int k = 0; k < p->sp.np; ++k) {
        a.ll[k] = (Real)p->sp.ll[k];
        a.lr[k] = (Real)p->sp.lr[k];
    }
    for (size_t q = 0; q < w.size(); ++q) a.w[q] = (Real)w[q];
    a.gamma = (Real)p->d.gamma;
    a.t0 = (Real)t0;
    return a;
}

template <class Real, bool FP32K> int launch_np(frgpu_problem *p, const std::vector<double> &w, double t0) {
    const int eq = p->d.equation;
    const size_t ne = eq == FRGPU_EULER2D ? (size_t)p->sp.nx * p->sp.ny : (size_t)p->sp.nx;
    Real *u = (Real *)fr_state_hi(p);
    Real *lo = FP32K ? (Real *)p->s3 : nullptr;
    const LimArgs<Real> a = lim_args<Real>(p, w, t0);
    const int grid = (int)((ne + 127) / 128);
    int *cnt = p->d_count + FR_COUNT_LIMITER;
#define FR_LIM(K, N) K<Real, N, FP32K><<<grid, 128, 0, p->stream>>>(u, lo, ne, a, p->d_status, cnt)
#define FR_LIM_NP(K)                                                                                               \
    switch (p->sp.np) {                                                                                            \
    case 2: FR_LIM(K, 2); break;                                                                                   \
    case 3: FR_LIM(K, 3); break;                                                                                   \
    case 4: FR_LIM(K, 4); break;                                                                                   \
    case 5: FR_LIM(K, 5); break;                                                                                   \
    case 6: FR_LIM(K, 6); break;                                                                                   \
    default: fr_set_error("positive_limiter: polynomial degree must be 1..5"); return FRGPU_ERR_UNSUPPORTED;      \
    }
    if (eq == FRGPU_EULER2D) {
        if constexpr (FP32K) {
            if (p->sp.np <= 4) {
                const int g4 = (int)((4 * ne + 127) / 128);
                switch (p->sp.np) {
                case 2: k_limiter2d_rows<2><<<g4, 128, 0, p->stream>>>(u, lo, ne, a, p->d_status, cnt); break;
                case 3: k_limiter2d_rows<3><<<g4, 128, 0, p->stream>>>(u, lo, ne, a, p->d_status, cnt); break;
                default: k_limiter2d_rows<4><<<g4, 128, 0, p->stream>>>(u, lo, ne, a, p->d_status, cnt); break;
                }
                FR_CUDA(cudaGetLastError());
                p->launches += 1;
                return FRGPU_OK;
            }
        }
        FR_LIM_NP(k_limiter2d)
    } else if (eq == FRGPU_EULER1D) {
        FR_LIM_NP(k_limiter1d)
    } else {
        FR_LIM_NP(k_limiter_scalar)
    }
#undef FR_LIM_NP
#undef FR_LIM
    FR_CUDA(cudaGetLastError());
    p->launches += 1;
    return FRGPU_OK;
}

} // namespace

// Enqueue the limiter on the problem's current state (stream-ordered, no
// synchronisation).  d_count[FR_COUNT_LIMITER] counts the limited elements;
// it is cleared here.
int fr_launch_limiter(frgpu_problem *p, const std::vector<double> &w, double t0) {
    const int eq = p->d.equation;
    if (eq == FRGPU_BGK1D) {
        fr_set_error("positive_limiter: not defined for the kinetic equation");
        return FRGPU_ERR_UNSUPPORTED;
    }
    if (p->prepare_only) return FRGPU_OK;
    FR_CUDA(cudaMemsetAsync(p->d_count + FR_COUNT_LIMITER, 0, sizeof(int), p->stream));
    if (p->d.precision == FRGPU_FP64) return launch_np<double, false>(p, w, t0);
    return launch_np<float, true>(p, w, t0);
}

// Element weights of the limiter: the caller's (np or np^2 values), or the
// space's Gauss weights normalised to sum 1 (the scalar form keeps the raw
// weights: it divides by their sum itself).  The Euler forms expect weights
// that sum to 1, as the reference's callers pass them.
int fr_limiter_weights(const frgpu_problem *p, const double *weights, std::vector<double> &w) {
    const int np = p->sp.np;
    const size_t n = p->d.equation == FRGPU_EULER2D ? (size_t)np * np : (size_t)np;
    w.assign(n, 0.0);
    if (weights) {
        for (size_t q = 0; q < n; ++q) w[q] = weights[q];
    } else {
        if (p->sp.wp.size() != n) {
            fr_set_error("positive_limiter: the space has no quadrature weights; pass them");
            return FRGPU_ERR_ARG;
        }
        // Gauss weights sum to 2 on [-1, 1] (4 on the square), and the reference
        // passes ps.wp ./ 4 in 2D
        const double s = p->d.equation == FRGPU_EULER2D ? 4.0 : 2.0;
        const bool scalar = p->d.equation == FRGPU_ADVECTION || p->d.equation == FRGPU_BURGERS;
        for (size_t q = 0; q < n; ++q) w[q] = scalar ? p->sp.wp[q] : p->sp.wp[q] / s;
    }
    return FRGPU_OK;
}
