// setup.cpp -- host-side construction of the flux-reconstruction operators
// (the L1/L2 layers of FluxReconstruction.jl: src/Polynomial/*.jl,
// src/Transform/transform.jl, src/struct.jl).  Computed once per space in
// extended precision and rounded to double.
#include <cmath>
#include <stdexcept>
#include <vector>

#include "frgpu_internal.h"

namespace frsetup {

using ld = long double;

// P_n(x) and P_n'(x) together from the Bonnet recurrence; the derivative uses
// P'_{k+1} = P'_{k-1} + (2k+1) P_k, which is regular at x = +-1.
static void legendre_pd(int n, ld x, ld &p, ld &dp) {
    ld p0 = 1, p1 = x, d0 = 0, d1 = 1;
    if (n == 0) { p = 1; dp = 0; return; }
    for (int k = 1; k < n; ++k) {
        ld p2 = ((2 * k + 1) * x * p1 - k * p0) / (k + 1);
        ld d2 = d0 + (2 * k + 1) * p1;
        p0 = p1; p1 = p2;
        d0 = d1; d1 = d2;
    }
    p = p1;
    dp = d1;
}

double dlegendre(int n, double x) {
    if (n <= 0) return 0.0;
    ld p, dp;
    legendre_pd(n, x, p, dp);
    return (double)dp;
}

// Gauss-Legendre rule of n points (FastGaussQuadrature.gausslegendre as used
// at src/Polynomial/poly_legendre.jl:6 and src/struct.jl:47): Newton's method
// on P_n in long double, nodes ascending.
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    const ld pi = 3.141592653589793238462643383279502884L;
    for (int i = 0; i < (n + 1) / 2; ++i) {
        ld z = std::cos(pi * (i + 0.75L) / (n + 0.5L)); // descending guess
        ld p, dp;
        for (int it = 0; it < 60; ++it) {
            legendre_pd(n, z, p, dp);
            ld dz = p / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-19L) break;
        }
        legendre_pd(n, z, p, dp);
        ld wt = 2 / ((1 - z * z) * dp * dp);
        x[n - 1 - i] = (double)z;
        x[i] = (double)(-z);
        w[n - 1 - i] = (double)wt;
        w[i] = (double)wt;
    }
    if (n % 2 == 1) x[n / 2] = 0.0;
}

// lagrange_point (src/Polynomial/poly_lagrange.jl:6-20)
void lagrange_point(const double *sp, int nsp, double x, double *l) {
    for (int k = 0; k < nsp; ++k) {
        ld t = 1;
        for (int j = 0; j < nsp; ++j)
            if (j != k) t *= ((ld)x - sp[j]) / ((ld)sp[k] - sp[j]);
        l[k] = (double)t;
    }
}

// dlagrange (src/Polynomial/poly_lagrange.jl:38-59): lpdm[m + nsp*k] = l_k'(r_m),
// l_k'(x) = sum_{l != k} 1/(x_k - x_l) prod_{j != k, l} (x - x_j)/(x_k - x_j).
void dlagrange(const double *sp, int nsp, double *lpdm) {
    for (int k = 0; k < nsp; ++k)
        for (int m = 0; m < nsp; ++m) {
            ld s = 0;
            for (int l = 0; l < nsp; ++l) {
                if (l == k) continue;
                ld t = 1 / ((ld)sp[k] - sp[l]);
                for (int j = 0; j < nsp; ++j)
                    if (j != k && j != l) t *= ((ld)sp[m] - sp[j]) / ((ld)sp[k] - sp[j]);
                s += t;
            }
            lpdm[m + nsp * k] = (double)s;
        }
}

// Correction-function derivatives (src/Polynomial/poly_legendre.jl:29-71).
// g_L' = (-1)^p (P_p' - y)/2, g_R' = (P_p' + y)/2 with y = P_{p+1}' (Radau),
// (p P_{p-1}' + (p+1) P_{p+1}')/(2p+1) (SD) or ((p+1) P_{p-1}' + p P_{p+1}')/(2p+1) (Huynh).
void dcorrection(int kind, int p, const double *x, int n, double *dgl, double *dgr) {
    const ld sgn = (p % 2 == 0) ? 1 : -1;
    for (int i = 0; i < n; ++i) {
        ld q, d, dp, dm = 0;
        legendre_pd(p, x[i], q, d);
        legendre_pd(p + 1, x[i], q, dp);
        if (p >= 1) legendre_pd(p - 1, x[i], q, dm);
        if (p - 1 == 0) dm = 0;
        ld y;
        if (kind == FRGPU_SD)
            y = (p * dm + (p + 1) * dp) / (2 * p + 1);
        else if (kind == FRGPU_HUYNH)
            y = ((p + 1) * dm + p * dp) / (2 * p + 1);
        else
            y = dp;
        dgl[i] = (double)(sgn * (d - y) / 2);
        dgr[i] = (double)((d + y) / 2);
    }
}

// Orthonormal Legendre polynomial sqrt((2n+1)/2) P_n(x): JacobiP(x, 0, 0, n)
// of src/Polynomial/poly_jacobi.jl:7-42.
double jacobi_orthonormal(int n, double x) {
    ld p, dp;
    legendre_pd(n, x, p, dp);
    return (double)(std::sqrt((2 * n + 1) / (ld)2) * p);
}

// vandermonde_matrix (src/Transform/transform.jl:18-26)
void vandermonde(int deg, const double *r, int n, double *V) {
    for (int j = 0; j <= deg; ++j)
        for (int i = 0; i < n; ++i) V[i + n * j] = jacobi_orthonormal(j, r[i]);
}

// vandermonde_matrix(Quad, ...) (src/Transform/transform.jl:55-68), mode
// sk = i*(deg+1) + j -> P~_i(r) P~_j(s)
void vandermonde_quad(int deg, const double *r, const double *s, int n, double *V) {
    int sk = 0;
    for (int i = 0; i <= deg; ++i)
        for (int j = 0; j <= deg; ++j, ++sk)
            for (int q = 0; q < n; ++q) V[q + n * sk] = jacobi_orthonormal(i, r[q]) * jacobi_orthonormal(j, s[q]);
}

// LU-free Gauss-Jordan inverse in long double with partial pivoting.
bool invert(int n, const double *A, double *Ainv) {
    std::vector<ld> M((size_t)n * 2 * n);
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) {
            M[(size_t)r * 2 * n + c] = A[r + (size_t)n * c];
            M[(size_t)r * 2 * n + n + c] = r == c ? 1 : 0;
        }
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(M[(size_t)r * 2 * n + c]) > std::fabs(M[(size_t)piv * 2 * n + c])) piv = r;
        if (M[(size_t)piv * 2 * n + c] == 0) return false;
        if (piv != c)
            for (int k = 0; k < 2 * n; ++k) std::swap(M[(size_t)c * 2 * n + k], M[(size_t)piv * 2 * n + k]);
        ld d = M[(size_t)c * 2 * n + c];
        for (int k = 0; k < 2 * n; ++k) M[(size_t)c * 2 * n + k] /= d;
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            ld f = M[(size_t)r * 2 * n + c];
            if (f == 0) continue;
            for (int k = 0; k < 2 * n; ++k) M[(size_t)r * 2 * n + k] -= f * M[(size_t)c * 2 * n + k];
        }
    }
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) Ainv[r + (size_t)n * c] = (double)M[(size_t)r * 2 * n + n + c];
    return true;
}

static void common_ops(frgpu_space &s) {
    const int np = s.np;
    gauss_legendre(np, s.xpl, s.w1);
    s.ll.resize(np);
    s.lr.resize(np);
    lagrange_point(s.xpl.data(), np, -1.0, s.ll.data());
    lagrange_point(s.xpl.data(), np, 1.0, s.lr.data());
    s.dl.resize((size_t)np * np);
    dlagrange(s.xpl.data(), np, s.dl.data());
}

// FRPSpace1D (src/struct.jl:40-85) on a uniform mesh of [x0, x1].
void build_1d(frgpu_space &s, int correction) {
    const int np = s.np;
    common_ops(s);
    s.dx = (s.x1 - s.x0) / s.nx;
    s.J.assign(s.nx, s.dx / 2);
    s.xc.resize(s.nx);
    for (int i = 0; i < s.nx; ++i) s.xc[i] = s.x0 + (i + 0.5) * s.dx;
    s.wp = s.w1;
    s.dhl.resize(np);
    s.dhr.resize(np);
    dcorrection(correction, s.deg, s.xpl.data(), np, s.dhl.data(), s.dhr.data());
    s.V.resize((size_t)np * np);
    s.iV.resize((size_t)np * np);
    vandermonde(s.deg, s.xpl.data(), np, s.V.data());
    if (!invert(np, s.V.data(), s.iV.data())) throw std::runtime_error("singular Vandermonde matrix");
}

// FRPSpace2D (src/struct.jl:130-242) on uniform rectangles; Radau correction
// as hard-coded at src/struct.jl:193; tensor Vandermonde on points flattened
// with r fastest (src/struct.jl:196-205).
void build_2d(frgpu_space &s) {
    const int np = s.np;
    common_ops(s);
    s.dx = (s.x1 - s.x0) / s.nx;
    s.dy = (s.y1 - s.y0) / s.ny;
    s.xc.resize(s.nx);
    s.yc.resize(s.ny);
    for (int i = 0; i < s.nx; ++i) s.xc[i] = s.x0 + (i + 0.5) * s.dx;
    for (int j = 0; j < s.ny; ++j) s.yc[j] = s.y0 + (j + 0.5) * s.dy;
    s.wp.resize((size_t)np * np);
    for (int l = 0; l < np; ++l)
        for (int k = 0; k < np; ++k) s.wp[k + np * l] = s.w1[k] * s.w1[l];
    s.dhl.resize(np);
    s.dhr.resize(np);
    dcorrection(FRGPU_RADAU, s.deg, s.xpl.data(), np, s.dhl.data(), s.dhr.data());
    const int n2 = np * np;
    std::vector<double> r(n2), q(n2);
    for (int l = 0; l < np; ++l)
        for (int k = 0; k < np; ++k) {
            r[k + np * l] = s.xpl[k];
            q[k + np * l] = s.xpl[l];
        }
    s.V.resize((size_t)n2 * n2);
    s.iV.resize((size_t)n2 * n2);
    vandermonde_quad(s.deg, r.data(), q.data(), n2, s.V.data());
    if (!invert(n2, s.V.data(), s.iV.data())) throw std::runtime_error("singular Vandermonde matrix");
}

// ---------------------------------------------------------------- triangles
// Orthonormal Jacobi polynomial P~_n^(alpha, 0)(x) (weight (1 - x)^alpha) from
// the classical three-term recurrence of P_n^(alpha, beta) and its norm
// h_n = 2^(alpha+beta+1) / (2n+alpha+beta+1) G(n+alpha+1) G(n+beta+1) / (G(n+alpha+beta+1) n!);
// the same functions JacobiP / dJacobiP of src/Polynomial/poly_jacobi.jl evaluate.
static ld jacobi_raw(int n, ld al, ld be, ld x) {
    if (n == 0) return 1;
    ld p0 = 1, p1 = (al + 1) + (al + be + 2) * (x - 1) / 2;
    for (int k = 2; k <= n; ++k) {
        const ld c = 2 * k + al + be;
        const ld p2 = ((c - 1) * (c * (c - 2) * x + al * al - be * be) * p1 - 2 * (k + al - 1) * (k + be - 1) * c * p0) /
                      (2 * k * (k + al + be) * (c - 2));
        p0 = p1;
        p1 = p2;
    }
    return p1;
}
static ld jacobi_norm(int n, ld al, ld be) {
    return std::pow((ld)2, al + be + 1) / (2 * n + al + be + 1) * std::tgamma(n + al + 1) * std::tgamma(n + be + 1) /
           (std::tgamma(n + al + be + 1) * std::tgamma((ld)n + 1));
}
static ld jacobi_on(int n, ld al, ld x) { return jacobi_raw(n, al, 0, x) / std::sqrt(jacobi_norm(n, al, 0)); }
// d/dx P_n^(al, 0) = (n + al + 1) / 2 P_{n-1}^(al+1, 1)
static ld djacobi_on(int n, ld al, ld x) {
    if (n == 0) return 0;
    return (n + al + 1) / 2 * jacobi_raw(n - 1, al + 1, 1, x) / std::sqrt(jacobi_norm(n, al, 0));
}

// The orthonormal simplex mode (i, j) of vandermonde_matrix(Tri, ...)
// (src/Transform/transform.jl:36-50, transform_triangle.jl:8-56) and its r and s
// derivatives at (r, s): psi = sqrt(2) P~_i(a) P~_j^(2i+1,0)(b) (1 - b)^i with
// a = 2 (1 + r) / (1 - s) - 1 (a = -1 at s = 1), b = s, by the chain rule
// da/dr = 2 / (1 - b), da/ds = (1 + a) / (1 - b).
static void simplex_mode(int i, int j, double r, double s, ld &v, ld &vr, ld &vs) {
    const ld a = s != 1.0 ? 2 * (1 + (ld)r) / (1 - (ld)s) - 1 : -1, b = s;
    const ld F = jacobi_on(i, 0, a), dF = djacobi_on(i, 0, a);
    const ld G = jacobi_on(j, 2 * i + 1, b), dG = djacobi_on(j, 2 * i + 1, b);
    const ld sq2 = std::sqrt((ld)2), om = 1 - b;
    const ld omi = std::pow(om, (ld)i), omi1 = i > 0 ? std::pow(om, (ld)(i - 1)) : 0;
    v = sq2 * F * G * omi;
    vr = i > 0 ? 2 * sq2 * dF * G * omi1 : 0;
    vs = sq2 * (F * dG * omi + (i > 0 ? (dF * (1 + a) - i * F) * G * omi1 : 0));
}

void vandermonde_tri(int deg, const double *r, const double *s, int n, double *V, double *Vr, double *Vs) {
    int sk = 0;
    for (int i = 0; i <= deg; ++i)
        for (int j = 0; j <= deg - i; ++j, ++sk)
            for (int q = 0; q < n; ++q) {
                ld v, vr, vs;
                simplex_mode(i, j, r[q], s[q], v, vr, vs);
                if (V) V[q + (size_t)n * sk] = (double)v;
                if (Vr) Vr[q + (size_t)n * sk] = (double)vr;
                if (Vs) Vs[q + (size_t)n * sk] = (double)vs;
            }
}

// Face flux points of the reference right triangle (triface_quadrature,
// src/Quadrature/quadrature.jl:86-106): Gauss-Legendre nodes x_k along face 1
// (r = x_k, s = -1), face 2 (r = x_{N-k}, s = x_k) and face 3 (r = -1, s = x_{N-k});
// weights w_k times the face lengths 1, sqrt(2), 1.
void triface_points(int deg, double *pr, double *ps, double *wf) {
    std::vector<double> x, w;
    gauss_legendre(deg + 1, x, w);
    const int m = deg + 1;
    for (int k = 0; k < m; ++k) {
        pr[0 + 3 * k] = x[k];
        ps[0 + 3 * k] = -1.0;
        pr[1 + 3 * k] = x[m - 1 - k];
        ps[1 + 3 * k] = x[k];
        pr[2 + 3 * k] = -1.0;
        ps[2 + 3 * k] = x[m - 1 - k];
        wf[0 + 3 * k] = w[k];
        wf[1 + 3 * k] = w[k] * std::sqrt(2.0);
        wf[2 + 3 * k] = w[k];
    }
}

// TriFRPSpace operators (src/struct.jl:305-352) at the np solution points (r, s):
// V; dl[i, q, d] = d l_q / d r_d at point i (dlagrange(V, Vr, Vs):
// V' \ Vr[i, :]); lf[f, k, q] = l_q at flux point (f, k) (V' \ psi_f);
// phi[f, k, i] = sum_m wf[f, k] psi_f[f, k, m] V[i, m] (correction_field,
// src/Polynomial/poly_triangle.jl:1-28).  Column-major outputs; any may be null.
void tri_operators(int deg, const double *r, const double *s, double *Vout, double *dl, double *lf, double *phi) {
    const int np = (deg + 1) * (deg + 2) / 2, m = deg + 1, nf = 3 * m;
    std::vector<double> V((size_t)np * np), Vr(V.size()), Vs(V.size()), iV(V.size());
    vandermonde_tri(deg, r, s, np, V.data(), Vr.data(), Vs.data());
    if (!invert(np, V.data(), iV.data())) throw std::runtime_error("singular triangle Vandermonde matrix");
    std::vector<double> pr(nf), ps(nf), wf(nf), Pf((size_t)nf * np);
    triface_points(deg, pr.data(), ps.data(), wf.data());
    vandermonde_tri(deg, pr.data(), ps.data(), nf, Pf.data(), nullptr, nullptr);
    if (Vout) std::copy(V.begin(), V.end(), Vout);
    for (int i = 0; i < np; ++i)
        for (int q = 0; q < np; ++q) {
            ld a = 0, b = 0;
            for (int t = 0; t < np; ++t) {
                a += (ld)Vr[i + (size_t)np * t] * iV[t + (size_t)np * q];
                b += (ld)Vs[i + (size_t)np * t] * iV[t + (size_t)np * q];
            }
            if (dl) {
                dl[i + (size_t)np * q] = (double)a;
                dl[i + (size_t)np * q + (size_t)np * np] = (double)b;
            }
        }
    for (int f = 0; f < nf; ++f) // f = face + 3 k, the flux point's flat index
        for (int q = 0; q < np; ++q) {
            ld a = 0, c = 0;
            for (int t = 0; t < np; ++t) {
                a += (ld)Pf[f + (size_t)nf * t] * iV[t + (size_t)np * q];
                c += (ld)wf[f] * Pf[f + (size_t)nf * t] * V[q + (size_t)np * t];
            }
            if (lf) lf[f + (size_t)nf * q] = (double)a;
            if (phi) phi[f + (size_t)nf * q] = (double)c;
        }
}

} // namespace frsetup
