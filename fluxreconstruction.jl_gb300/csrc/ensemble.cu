// ensemble.cu -- host side of the batched 1D Burgers ensemble: instance
// layout, the config-4 generator (Philox-4x32-10), the work queues, the
// tile-shape autotuner and the persistent launch.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "ensemble_kernels.cuh"

int fr_ensemble_launch_f64(const void *args, int grid, size_t smem, cudaStream_t st);
int fr_ensemble_launch_f32(const void *args, int grid, size_t smem, cudaStream_t st);
int fr_ensemble_occupancy_f64(size_t smem, bool learned, int *blocks);
int fr_ensemble_occupancy_f32(size_t smem, bool learned, int *blocks);
int fr_ensemble_features_f64(const void *args, int n, const long *d_eoff, float *d_feat, int *d_labels,
                             cudaStream_t st);
int fr_ensemble_features_f32(const void *args, int n, const long *d_eoff, float *d_feat, int *d_labels,
                             cudaStream_t st);

namespace {

// Philox-4x32-10 counter-based generator (Salmon, Moraes, Dror and Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC 2011).
void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

// Uniforms in (0, 1) of block `j` of instance `inst` (key = instance id, seed).
void uniforms(uint32_t inst, uint32_t seed, uint32_t j, double u[4]) {
    const uint32_t ctr[4] = {j, 0u, 0u, 0u}, key[2] = {inst, seed};
    uint32_t o[4];
    philox4x32_10(ctr, key, o);
    for (int q = 0; q < 4; ++q) u[q] = ((o[q] >> 8) + 0.5) * (1.0 / 16777216.0);
}

} // namespace

struct frgpu_ensemble {
    int n = 0, precision = FRGPU_FP64;
    double x0 = 0, x1 = 1;
    std::vector<EnsInstance> inst;
    std::vector<int> ne, deg;
    long ndof = 0;
    size_t esize = 8;
    void *u = nullptr, *s1 = nullptr, *s2 = nullptr, *backup = nullptr, *ops = nullptr;
    EnsInstance *d_inst = nullptr;
    int *d_qc = nullptr, *d_qw = nullptr, *d_counters = nullptr, *d_steps = nullptr, *d_status = nullptr;
    int *d_failed = nullptr; // per instance: 0 or the step at which it turned non-finite
    double *d_dt = nullptr;
    cudaStream_t stream = nullptr;
    int thr[5] = {128, 128, 128, 128, 128}; // warp queue if ne <= thr[deg-1]
    std::vector<int> steps;
    std::vector<double> dts;
    float last_ms = 0;
    long launches = 0;
    // learned indicator (borrowed network; null = plain indicator)
    const frgpu_mlp *mlp = nullptr;
    float mlp_thr = 0.5f, mlp_band = 0.0f;
    unsigned long long *d_istats = nullptr; // troubled, misfires, fallbacks, judged (last run)
    long *d_eoff = nullptr;                 // first element of each instance in the flat element list
    long nelem = 0;
};

static void ens_free(frgpu_ensemble *e) {
    if (!e) return;
    if (e->stream) cudaStreamSynchronize(e->stream);
    void *b[] = {e->u,         e->s1,     e->s2,     e->backup,   e->ops,      e->d_inst,  e->d_qc,
                 e->d_qw,      e->d_counters, e->d_steps, e->d_status, e->d_dt, e->d_istats, e->d_eoff,
                 e->d_failed};
    for (void *p : b)
        if (p) cudaFree(p);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

template <class Real> static void fill_ops(EnsOps<Real> &o) {
    std::memset(&o, 0, sizeof(o));
    for (int deg = 1; deg <= 5; ++deg) {
        const int np = deg + 1, d = deg - 1;
        std::vector<double> x, w, l(np), dl(np * np), gl(np), gr(np), V(np * np), iV(np * np);
        frsetup::gauss_legendre(np, x, w);
        frsetup::lagrange_point(x.data(), np, -1.0, l.data());
        for (int k = 0; k < np; ++k) o.ll[d][k] = (Real)l[k];
        frsetup::lagrange_point(x.data(), np, 1.0, l.data());
        for (int k = 0; k < np; ++k) o.lr[d][k] = (Real)l[k];
        frsetup::dlagrange(x.data(), np, dl.data());
        frsetup::dcorrection(FRGPU_RADAU, deg, x.data(), np, gl.data(), gr.data());
        frsetup::vandermonde(deg, x.data(), np, V.data());
        frsetup::invert(np, V.data(), iV.data());
        for (int a = 0; a < np; ++a) {
            o.dgl[d][a] = (Real)gl[a];
            o.dgr[d][a] = (Real)gr[a];
            for (int b = 0; b < np; ++b) {
                o.D[d][a][b] = (Real)dl[a + np * b];
                o.V[d][a][b] = (Real)V[a + np * b];
                o.iV[d][a][b] = (Real)iV[a + np * b];
            }
        }
        o.expfac[d] = std::exp(0.875 * deg);
    }
}

template <class Real>
static EnsArgs<Real> ens_args(frgpu_ensemble *e, int n_cta, int n_warp, double t_end, double cfl, int filter) {
    EnsArgs<Real> a{};
    a.inst = e->d_inst;
    a.queue_cta = e->d_qc;
    a.queue_warp = e->d_qw;
    a.n_cta = n_cta;
    a.n_warp = n_warp;
    a.counters = e->d_counters;
    a.u = (Real *)e->u;
    a.s1 = (Real *)e->s1;
    a.s2 = (Real *)e->s2;
    a.ops = (const EnsOps<Real> *)e->ops;
    a.t_end = t_end;
    a.cfl = cfl;
    a.filter = filter;
    a.dt_out = e->d_dt;
    a.steps_out = e->d_steps;
    a.failed = e->d_failed;
    a.status = e->d_status;
    a.mlp = frmlp::MLPDev{nullptr, nullptr, nullptr, nullptr, nullptr};
    if (e->mlp) {
        const fr_mlp_ptrs m = fr_mlp_device(e->mlp);
        a.mlp = frmlp::MLPDev{m.P, (const __nv_bfloat16 *)m.W1, (const __nv_bfloat16 *)m.W2,
                              (const __nv_bfloat16 *)m.W2T, m.TC};
    }
    a.thr = e->mlp_thr;
    a.band = e->mlp_band;
    a.istats = e->d_istats;
    return a;
}

static int ens_launch(frgpu_ensemble *e, double t_end, double cfl, int filter) {
    // queues: small instances to warps, the rest to whole CTAs, costliest first
    std::vector<int> qc, qw;
    for (int i = 0; i < e->n; ++i) {
        const int lim = std::min(e->thr[e->deg[i] - 1], ENS_MAX_NE_WARP);
        (e->ne[i] <= lim ? qw : qc).push_back(i);
    }
    auto cost = [&](int i) { return (double)e->ne[i] * e->ne[i] * (e->deg[i] + 1) * (2 * e->deg[i] + 1); };
    auto by_cost = [&](int a, int b) { return cost(a) > cost(b); };
    std::sort(qc.begin(), qc.end(), by_cost);
    std::sort(qw.begin(), qw.end(), by_cost);
    if (!qc.empty()) FR_CUDA(cudaMemcpyAsync(e->d_qc, qc.data(), sizeof(int) * qc.size(), cudaMemcpyHostToDevice, e->stream));
    if (!qw.empty()) FR_CUDA(cudaMemcpyAsync(e->d_qw, qw.data(), sizeof(int) * qw.size(), cudaMemcpyHostToDevice, e->stream));
    FR_CUDA(cudaMemsetAsync(e->d_counters, 0, sizeof(int) * 2, e->stream));
    FR_CUDA(cudaMemsetAsync(e->d_istats, 0, sizeof(unsigned long long) * 4, e->stream));
    int dev = 0, sms = 0, blocks = 0;
    FR_CUDA(cudaGetDevice(&dev));
    FR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int rc;
    const size_t learned = (e->mlp && filter) ? ENS_MLP_SMEM : 0;
    const size_t smem = (e->precision == FRGPU_FP64 ? ens_smem_bytes<double>() : ens_smem_bytes<float>()) + learned;
    rc = e->precision == FRGPU_FP64 ? fr_ensemble_occupancy_f64(smem, learned != 0, &blocks)
                                    : fr_ensemble_occupancy_f32(smem, learned != 0, &blocks);
    if (rc) return rc;
    const int grid = sms * std::max(blocks, 1);
    if (e->precision == FRGPU_FP64) {
        EnsArgs<double> a = ens_args<double>(e, (int)qc.size(), (int)qw.size(), t_end, cfl, filter);
        if (!learned) a.mlp.P = nullptr;
        rc = fr_ensemble_launch_f64(&a, grid, smem, e->stream);
    } else {
        EnsArgs<float> a = ens_args<float>(e, (int)qc.size(), (int)qw.size(), t_end, cfl, filter);
        if (!learned) a.mlp.P = nullptr;
        rc = fr_ensemble_launch_f32(&a, grid, smem, e->stream);
    }
    e->launches += 1;
    return rc;
}

static int ens_finish(frgpu_ensemble *e) {
    int st = 0;
    e->steps.assign(e->n, 0);
    e->dts.assign(e->n, 0.0);
    FR_CUDA(cudaMemcpyAsync(&st, e->d_status, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    FR_CUDA(cudaMemcpyAsync(e->steps.data(), e->d_steps, sizeof(int) * e->n, cudaMemcpyDeviceToHost, e->stream));
    FR_CUDA(cudaMemcpyAsync(e->dts.data(), e->d_dt, sizeof(double) * e->n, cudaMemcpyDeviceToHost, e->stream));
    FR_CUDA(cudaStreamSynchronize(e->stream));
    if (st) {
        FR_CUDA(cudaMemset(e->d_status, 0, sizeof(int)));
        fr_set_error("ensemble: non-finite value in an instance");
        return FRGPU_ERR_NONFINITE;
    }
    return FRGPU_OK;
}

extern "C" {

/* Sizes of the config-4 ensemble: ne log-uniform in [32, 2048] (rounded),
 * deg uniform in 1..5, drawn per instance id from Philox-4x32-10 with the seed. */
FRGPU_API int frgpu_ensemble_config4_sizes(int n, unsigned seed, int *ne, int *deg) {
    if (n < 1 || !ne || !deg) {
        fr_set_error("ensemble_config4_sizes: bad arguments");
        return FRGPU_ERR_ARG;
    }
    const double a = std::log(32.0), b = std::log(2048.0);
    for (int i = 0; i < n; ++i) {
        double u[4];
        uniforms((uint32_t)i, seed, 0u, u);
        ne[i] = std::min(2048, std::max(32, (int)std::lround(std::exp(a + u[0] * (b - a)))));
        deg[i] = 1 + std::min(4, (int)(5.0 * u[1]));
    }
    return FRGPU_OK;
}

FRGPU_API int frgpu_ensemble_create(int n, const int *ne, const int *deg, double x0, double x1, int precision,
                                    frgpu_ensemble **out) {
    if (!out) {
        fr_set_error("ensemble_create: null output");
        return FRGPU_ERR_ARG;
    }
    *out = nullptr;
    if (n < 1 || !ne || !deg || !(x1 > x0) || (precision != FRGPU_FP64 && precision != FRGPU_FP32K)) {
        fr_set_error("ensemble_create: bad arguments");
        return FRGPU_ERR_ARG;
    }
    for (int i = 0; i < n; ++i)
        if (ne[i] < 2 || ne[i] > ENS_MAX_NE_CTA || deg[i] < 1 || deg[i] > 5) {
            fr_set_error("ensemble_create: instance " + std::to_string(i) + " needs 2 <= ne <= 2048 and 1 <= deg <= 5");
            return FRGPU_ERR_ARG;
        }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        fr_set_error("ensemble_create: no CUDA device");
        return FRGPU_ERR_CUDA;
    }
    auto *e = new frgpu_ensemble();
    e->n = n;
    e->precision = precision;
    e->x0 = x0;
    e->x1 = x1;
    e->esize = precision == FRGPU_FP64 ? 8 : 4;
    e->ne.assign(ne, ne + n);
    e->deg.assign(deg, deg + n);
    long off = 0;
    for (int i = 0; i < n; ++i) {
        EnsInstance in;
        in.off = off;
        in.ne = ne[i];
        in.np = deg[i] + 1;
        in.dx = (x1 - x0) / ne[i];
        e->inst.push_back(in);
        off += (long)in.ne * in.np;
    }
    e->ndof = off;
    int rc = [&]() -> int {
        FR_CUDA(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
        const size_t bytes = e->esize * (size_t)e->ndof;
        FR_CUDA(cudaMalloc(&e->u, bytes));
        FR_CUDA(cudaMalloc(&e->s1, bytes));
        FR_CUDA(cudaMalloc(&e->s2, bytes));
        FR_CUDA(cudaMemset(e->u, 0, bytes));
        FR_CUDA(cudaMalloc(&e->d_inst, sizeof(EnsInstance) * n));
        FR_CUDA(cudaMemcpy(e->d_inst, e->inst.data(), sizeof(EnsInstance) * n, cudaMemcpyHostToDevice));
        FR_CUDA(cudaMalloc(&e->d_qc, sizeof(int) * n));
        FR_CUDA(cudaMalloc(&e->d_qw, sizeof(int) * n));
        FR_CUDA(cudaMalloc(&e->d_counters, sizeof(int) * 2));
        FR_CUDA(cudaMalloc(&e->d_steps, sizeof(int) * n));
        FR_CUDA(cudaMalloc(&e->d_dt, sizeof(double) * n));
        FR_CUDA(cudaMalloc(&e->d_status, sizeof(int)));
        FR_CUDA(cudaMemset(e->d_status, 0, sizeof(int)));
        FR_CUDA(cudaMalloc(&e->d_failed, sizeof(int) * n));
        FR_CUDA(cudaMemset(e->d_failed, 0, sizeof(int) * n));
        FR_CUDA(cudaMalloc(&e->d_istats, sizeof(unsigned long long) * 4));
        FR_CUDA(cudaMemset(e->d_istats, 0, sizeof(unsigned long long) * 4));
        std::vector<long> eoff(n);
        for (int i = 0; i < n; ++i) {
            eoff[i] = e->nelem;
            e->nelem += ne[i];
        }
        FR_CUDA(cudaMalloc(&e->d_eoff, sizeof(long) * n));
        FR_CUDA(cudaMemcpy(e->d_eoff, eoff.data(), sizeof(long) * n, cudaMemcpyHostToDevice));
        if (precision == FRGPU_FP64) {
            EnsOps<double> o;
            fill_ops(o);
            FR_CUDA(cudaMalloc(&e->ops, sizeof(o)));
            FR_CUDA(cudaMemcpy(e->ops, &o, sizeof(o), cudaMemcpyHostToDevice));
        } else {
            EnsOps<float> o;
            fill_ops(o);
            FR_CUDA(cudaMalloc(&e->ops, sizeof(o)));
            FR_CUDA(cudaMemcpy(e->ops, &o, sizeof(o), cudaMemcpyHostToDevice));
        }
        return FRGPU_OK;
    }();
    if (rc) {
        ens_free(e);
        return rc;
    }
    *out = e;
    return FRGPU_OK;
}

FRGPU_API void frgpu_ensemble_destroy(frgpu_ensemble *e) { ens_free(e); }

FRGPU_API long frgpu_ensemble_ndof(const frgpu_ensemble *e) { return e ? e->ndof : -1; }

/* Instance i's state u[ne_i, deg_i + 1] (Julia layout, FP64) in or out. */
FRGPU_API int frgpu_ensemble_set_state(frgpu_ensemble *e, int i, const double *u) {
    if (!e || !u || i < 0 || i >= e->n) {
        fr_set_error("ensemble_set_state: bad arguments");
        return FRGPU_ERR_ARG;
    }
    const long n = (long)e->inst[i].ne * e->inst[i].np;
    FR_CUDA(cudaMemset(e->d_failed + i, 0, sizeof(int)));
    if (e->esize == 8) {
        FR_CUDA(cudaMemcpy((double *)e->u + e->inst[i].off, u, sizeof(double) * n, cudaMemcpyHostToDevice));
    } else {
        std::vector<float> f(u, u + n);
        FR_CUDA(cudaMemcpy((float *)e->u + e->inst[i].off, f.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    }
    return FRGPU_OK;
}

FRGPU_API int frgpu_ensemble_get_state(frgpu_ensemble *e, int i, double *u) {
    if (!e || !u || i < 0 || i >= e->n) {
        fr_set_error("ensemble_get_state: bad arguments");
        return FRGPU_ERR_ARG;
    }
    FR_CUDA(cudaStreamSynchronize(e->stream));
    const long n = (long)e->inst[i].ne * e->inst[i].np;
    if (e->esize == 8) {
        FR_CUDA(cudaMemcpy(u, (double *)e->u + e->inst[i].off, sizeof(double) * n, cudaMemcpyDeviceToHost));
    } else {
        std::vector<float> f(n);
        FR_CUDA(cudaMemcpy(f.data(), (float *)e->u + e->inst[i].off, sizeof(float) * n, cudaMemcpyDeviceToHost));
        for (long q = 0; q < n; ++q) u[q] = f[q];
    }
    return FRGPU_OK;
}

/* Config-4 initial conditions: u0 = sum_{k=1..8} a_k sin(k x + phi_k) at the
 * solution points, a_k ~ N(0, sigma^2) (Box-Muller), phi_k ~ U[0, 2 pi), from
 * Philox-4x32-10 keyed by (instance id, seed). */
FRGPU_API int frgpu_ensemble_init_fourier(frgpu_ensemble *e, double sigma, unsigned seed) {
    if (!e) {
        fr_set_error("ensemble_init_fourier: null ensemble");
        return FRGPU_ERR_ARG;
    }
    const double twopi = 6.283185307179586476925286766559;
    std::vector<double> all((size_t)e->ndof);
    for (int i = 0; i < e->n; ++i) {
        double amp[8], ph[8], u[4];
        for (int j = 0; j < 2; ++j) {
            uniforms((uint32_t)i, seed, 1u + j, u);
            for (int q = 0; q < 2; ++q) {
                const double rad = std::sqrt(-2.0 * std::log(u[2 * q]));
                amp[4 * j + 2 * q] = sigma * rad * std::cos(twopi * u[2 * q + 1]);
                amp[4 * j + 2 * q + 1] = sigma * rad * std::sin(twopi * u[2 * q + 1]);
            }
        }
        for (int j = 0; j < 2; ++j) {
            uniforms((uint32_t)i, seed, 3u + j, u);
            for (int q = 0; q < 4; ++q) ph[4 * j + q] = twopi * u[q];
        }
        const EnsInstance &in = e->inst[i];
        std::vector<double> r, w;
        frsetup::gauss_legendre(in.np, r, w);
        for (int k = 0; k < in.np; ++k)
            for (int el = 0; el < in.ne; ++el) {
                const double xl = e->x0 + el * in.dx, xr = xl + in.dx;
                const double x = ((1.0 - r[k]) / 2.0) * xl + ((1.0 + r[k]) / 2.0) * xr;
                double v = 0;
                for (int m = 0; m < 8; ++m) v += amp[m] * std::sin((m + 1) * x + ph[m]);
                all[in.off + el + (long)in.ne * k] = v;
            }
    }
    FR_CUDA(cudaMemset(e->d_failed, 0, sizeof(int) * e->n));
    if (e->esize == 8) {
        FR_CUDA(cudaMemcpy(e->u, all.data(), sizeof(double) * e->ndof, cudaMemcpyHostToDevice));
    } else {
        std::vector<float> f(all.begin(), all.end());
        FR_CUDA(cudaMemcpy(e->u, f.data(), sizeof(float) * e->ndof, cudaMemcpyHostToDevice));
    }
    return FRGPU_OK;
}

/* Tile shapes: instances with ne <= thr[deg-1] run on one warp, the others on
 * a whole 256-thread CTA (ne <= 512 for warps). */
FRGPU_API int frgpu_ensemble_set_tiles(frgpu_ensemble *e, const int *thr) {
    if (!e || !thr) {
        fr_set_error("ensemble_set_tiles: bad arguments");
        return FRGPU_ERR_ARG;
    }
    for (int d = 0; d < 5; ++d) e->thr[d] = thr[d];
    return FRGPU_OK;
}

FRGPU_API int frgpu_ensemble_get_tiles(const frgpu_ensemble *e, int *thr) {
    if (!e || !thr) {
        fr_set_error("ensemble_get_tiles: bad arguments");
        return FRGPU_ERR_ARG;
    }
    for (int d = 0; d < 5; ++d) thr[d] = e->thr[d];
    return FRGPU_OK;
}

/* Advance every instance to t_end in one persistent launch (per-instance
 * CFL time step dt_i = cfl dx_i / ((2 deg_i + 1) max|u_i|), SSPRK3, the
 * modal-decay indicator + :l2 filter after every step when filter != 0). */
FRGPU_API int frgpu_ensemble_run(frgpu_ensemble *e, double t_end, double cfl, int filter) {
    if (!e || !(t_end > 0) || !(cfl > 0)) {
        fr_set_error("ensemble_run: bad arguments");
        return FRGPU_ERR_ARG;
    }
    cudaEvent_t a, b;
    FR_CUDA(cudaEventCreate(&a));
    FR_CUDA(cudaEventCreate(&b));
    FR_CUDA(cudaEventRecord(a, e->stream));
    int rc = ens_launch(e, t_end, cfl, filter);
    FR_CUDA(cudaEventRecord(b, e->stream));
    if (!rc) rc = ens_finish(e);
    cudaEventElapsedTime(&e->last_ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return rc;
}

/* After a run: total DOF-updates per RK stage (sum_i 3 ndof_i steps_i), the
 * largest step count, the kernel time (ms), and per-instance dt / steps (optional). */
FRGPU_API int frgpu_ensemble_stats(const frgpu_ensemble *e, double *dof_stage_updates, int *max_steps, float *ms,
                                   double *dt, int *steps) {
    if (!e) {
        fr_set_error("ensemble_stats: null ensemble");
        return FRGPU_ERR_ARG;
    }
    double tot = 0;
    int mx = 0;
    for (int i = 0; i < e->n && i < (int)e->steps.size(); ++i) {
        tot += 3.0 * e->inst[i].ne * e->inst[i].np * e->steps[i];
        mx = std::max(mx, e->steps[i]);
        if (dt) dt[i] = e->dts[i];
        if (steps) steps[i] = e->steps[i];
    }
    if (dof_stage_updates) *dof_stage_updates = tot;
    if (max_steps) *max_steps = mx;
    if (ms) *ms = e->last_ms;
    return FRGPU_OK;
}

/* Autotuner: coordinate descent over the per-degree warp/CTA thresholds
 * {0, 64, 128, 256, 512}, timing short runs of t_probe on the ensemble's own
 * state (restored after every probe).  The best thresholds are kept and
 * returned in thr (5 ints). */
FRGPU_API int frgpu_ensemble_tune(frgpu_ensemble *e, double t_probe, double cfl, int filter, int *thr) {
    if (!e || !(t_probe > 0) || !(cfl > 0)) {
        fr_set_error("ensemble_tune: bad arguments");
        return FRGPU_ERR_ARG;
    }
    const size_t bytes = e->esize * (size_t)e->ndof;
    if (!e->backup) FR_CUDA(cudaMalloc(&e->backup, bytes));
    FR_CUDA(cudaMemcpyAsync(e->backup, e->u, bytes, cudaMemcpyDeviceToDevice, e->stream));
    const int cand[5] = {0, 64, 128, 256, 512};
    auto probe = [&](float *ms) -> int {
        float best = 1e30f;
        for (int rep = 0; rep < 2; ++rep) {
            FR_CUDA(cudaMemcpyAsync(e->u, e->backup, bytes, cudaMemcpyDeviceToDevice, e->stream));
            int rc = frgpu_ensemble_run(e, t_probe, cfl, filter);
            if (rc) return rc;
            best = std::min(best, e->last_ms);
        }
        *ms = best;
        return FRGPU_OK;
    };
    for (int d = 0; d < 5; ++d) {
        int best_c = e->thr[d];
        float best_ms = 1e30f;
        for (int c : cand) {
            e->thr[d] = c;
            float ms;
            int rc = probe(&ms);
            if (rc) return rc;
            if (ms < best_ms) {
                best_ms = ms;
                best_c = c;
            }
        }
        e->thr[d] = best_c;
    }
    FR_CUDA(cudaMemcpyAsync(e->u, e->backup, bytes, cudaMemcpyDeviceToDevice, e->stream));
    FR_CUDA(cudaStreamSynchronize(e->stream));
    if (thr)
        for (int d = 0; d < 5; ++d) thr[d] = e->thr[d];
    return FRGPU_OK;
}

FRGPU_API long frgpu_ensemble_launches(const frgpu_ensemble *e) { return e ? e->launches : -1; }

/* Use the learned indicator (network m, probability threshold, fallback band)
 * in the post-step filter of frgpu_ensemble_run; m = NULL restores the plain
 * modal-decay indicator.  The network is borrowed and must outlive its use. */
FRGPU_API int frgpu_ensemble_set_mlp(frgpu_ensemble *e, const frgpu_mlp *m, double threshold, double band) {
    if (!e || !(threshold > 0 && threshold < 1) || !(band >= 0)) {
        fr_set_error("ensemble_set_mlp: bad arguments");
        return FRGPU_ERR_ARG;
    }
    e->mlp = m;
    e->mlp_thr = (float)threshold;
    e->mlp_band = (float)band;
    return FRGPU_OK;
}

/* Counts of the last run's learned indicator, summed over all steps and
 * instances: troubled, misfires (network != plain test), fallbacks, elements judged. */
FRGPU_API int frgpu_ensemble_indicator_stats(frgpu_ensemble *e, long long *stats) {
    if (!e || !stats) {
        fr_set_error("ensemble_indicator_stats: bad arguments");
        return FRGPU_ERR_ARG;
    }
    unsigned long long h[4];
    FR_CUDA(cudaMemcpyAsync(h, e->d_istats, sizeof(h), cudaMemcpyDeviceToHost, e->stream));
    FR_CUDA(cudaStreamSynchronize(e->stream));
    for (int c = 0; c < 4; ++c) stats[c] = (long long)h[c];
    return FRGPU_OK;
}

/* Instances stopped because their state turned non-finite (flags[i] = the
 * step, 1-based, after which instance i stopped; 0 = running normally).
 * Returns the number of stopped instances, or a negative error.  A stopped
 * instance stays stopped in later runs until its state is set again
 * (frgpu_ensemble_set_state / frgpu_ensemble_init_fourier). */
FRGPU_API int frgpu_ensemble_failed(frgpu_ensemble *e, int *flags) {
    if (!e) {
        fr_set_error("ensemble_failed: null ensemble");
        return FRGPU_ERR_ARG;
    }
    std::vector<int> f(e->n);
    FR_CUDA(cudaMemcpyAsync(f.data(), e->d_failed, sizeof(int) * e->n, cudaMemcpyDeviceToHost, e->stream));
    FR_CUDA(cudaStreamSynchronize(e->stream));
    int cnt = 0;
    for (int i = 0; i < e->n; ++i) {
        cnt += f[i] != 0;
        if (flags) flags[i] = f[i];
    }
    return cnt;
}

/* Number of elements over all instances (the rows of frgpu_ensemble_features). */
FRGPU_API long frgpu_ensemble_nelem(const frgpu_ensemble *e) { return e ? e->nelem : -1; }

/* Features (32 per element, as the learned indicator sees them) and the plain
 * modal-decay labels (1 = troubled) of every element of the current state,
 * instance by instance; n must equal frgpu_ensemble_nelem.  Host arrays. */
FRGPU_API int frgpu_ensemble_features(frgpu_ensemble *e, float *feat, int *labels, long n) {
    if (!e || !feat || !labels || n != e->nelem) {
        fr_set_error("ensemble_features: bad arguments (n must be the ensemble's element count)");
        return FRGPU_ERR_ARG;
    }
    float *d_feat = nullptr;
    int *d_lab = nullptr;
    int rc = [&]() -> int {
        FR_CUDA(cudaMalloc(&d_feat, sizeof(float) * 32 * (size_t)n));
        FR_CUDA(cudaMalloc(&d_lab, sizeof(int) * (size_t)n));
        int r;
        if (e->precision == FRGPU_FP64) {
            EnsArgs<double> a = ens_args<double>(e, 0, 0, 0.0, 0.0, 1);
            r = fr_ensemble_features_f64(&a, e->n, e->d_eoff, d_feat, d_lab, e->stream);
        } else {
            EnsArgs<float> a = ens_args<float>(e, 0, 0, 0.0, 0.0, 1);
            r = fr_ensemble_features_f32(&a, e->n, e->d_eoff, d_feat, d_lab, e->stream);
        }
        if (r) return r;
        FR_CUDA(cudaMemcpyAsync(feat, d_feat, sizeof(float) * 32 * (size_t)n, cudaMemcpyDeviceToHost, e->stream));
        FR_CUDA(cudaMemcpyAsync(labels, d_lab, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, e->stream));
        FR_CUDA(cudaStreamSynchronize(e->stream));
        return FRGPU_OK;
    }();
    if (d_feat) cudaFree(d_feat);
    if (d_lab) cudaFree(d_lab);
    e->launches += 1;
    return rc;
}

} // extern "C"
