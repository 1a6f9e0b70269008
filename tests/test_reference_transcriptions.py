"""Residuals of the reference transcribed loop for loop in numpy, against the
oracle's restatements (CPU only; the GPU tests compare the library with the
oracle):
* the kinetic mol! closures of example/bgk_wave.jl:69-129 and
  example/advection_kinetic.jl:73-128, with the scripts' own periodic face
  tables e2f / f2e (the conserve_prim(w, 3) closure and the density-only
  closure prim = [rho, a, 1]);
* the library's frode_advection! (config 1) and frode_euler! with their
  periodic and Dirichlet boundary functions;
* the indicator + :l2 filter loop of example/shock-vortex.jl:308-321;
* the scalar positive_limiter (src/dissipation.jl:38-58).
The 2D transcriptions sit beside their tests: tests/test_shock_vortex_script.py
(example/shock-vortex.jl) and tests/test_curve_euler.py (dev/curve_euler.jl)."""
import numpy as np
import pytest

from test_parity_gpu import oracle_space1d, oracle_space2d


def face_tables(nx):
    """e2f / f2e of the scripts (0-based): e2f[i] = (right face, left face) of
    element i, f2e[f] = (element right of face f, element left of it)."""
    nface = nx + 1
    e2f = np.zeros((nx, 2), dtype=int)
    for i in range(nx):
        if i == 0:
            e2f[i] = (i + 1, nface - 1)
        elif i == nx - 1:
            e2f[i] = (0, i)
        else:
            e2f[i] = (i + 1, i)
    f2e = np.zeros((nface, 2), dtype=int)
    for f in range(nface):
        if f == 0:
            f2e[f] = (f, nx - 1)
        elif f == nface - 1:
            f2e[f] = (0, f - 1)
        else:
            f2e[f] = (f, f - 1)
    return e2f, f2e


def bgk_wave_mol(u, dx, velo, weights, ll, lr, lpdm, dgl, dgr, tau):
    """example/bgk_wave.jl:69-129 (tau passed in; the script has 1e-2)."""
    ncell, nu, nsp = u.shape
    e2f, f2e = face_tables(ncell)
    delta = (velo > 0).astype(float)
    M = np.zeros_like(u)
    for i in range(ncell):
        for k in range(nsp):
            w = np.array([np.sum(weights * u[i, :, k]), np.sum(weights * velo * u[i, :, k]),
                          0.5 * np.sum(weights * velo ** 2 * u[i, :, k])])
            # conserve_prim(w, 3.0), 1D: U = m / rho, lambda = rho / (2 p), p = (gamma - 1)(E - m U / 2)
            U = w[1] / w[0]
            lam = 0.5 * w[0] / (3.0 - 1.0) / (w[2] - 0.5 * w[1] * U)
            M[i, :, k] = w[0] * np.sqrt(lam / np.pi) * np.exp(-lam * (velo - U) ** 2)
    f = np.zeros_like(u)
    for i in range(ncell):
        f[i] = velo[:, None] * u[i] / (0.5 * dx[i])
    f_face = np.zeros((ncell, nu, 2))
    for i in range(ncell):
        for j in range(nu):
            f_face[i, j, 0] = np.dot(f[i, j, :], ll)  # interp_face!: fdelta[1] = f . ll
            f_face[i, j, 1] = np.dot(f[i, j, :], lr)
    f_int = np.zeros((ncell + 1, nu))
    for fc in range(ncell + 1):
        f_int[fc] = f_face[f2e[fc, 0], :, 0] * (1.0 - delta) + f_face[f2e[fc, 1], :, 1] * delta
    du = np.zeros_like(u)
    for i in range(ncell):
        for j in range(nu):
            rhs1 = np.array([np.dot(f[i, j, :], lpdm[p, :]) for p in range(nsp)])  # poly_derivative!
            for p in range(nsp):
                du[i, j, p] = (-(rhs1[p] + (f_int[e2f[i, 1], j] - f_face[i, j, 0]) * dgl[p]
                                 + (f_int[e2f[i, 0], j] - f_face[i, j, 1]) * dgr[p])
                               + (M[i, j, p] - u[i, j, p]) / tau)
    return du


def advection_kinetic_mol(u, dx, velo, weights, a, ll, lr, lpdm, dgl, dgr, tau):
    """example/advection_kinetic.jl:73-128 (its f_face index 1 is the right
    trace, 2 the left one; the Maxwellian from the density alone)."""
    ncell, nu, nsp = u.shape
    e2f, f2e = face_tables(ncell)
    delta = (velo > 0).astype(float)
    M = np.zeros_like(u)
    for i in range(ncell):
        for k in range(nsp):
            rho = np.sum(u[i, :, k] * weights)
            prim = [rho, a, 1.0]
            M[i, :, k] = prim[0] * np.sqrt(prim[2] / np.pi) * np.exp(-prim[2] * (velo - prim[1]) ** 2)
    f = np.zeros_like(u)
    for i in range(ncell):
        f[i] = velo[:, None] * u[i] / (0.5 * dx[i])
    f_face = np.zeros((ncell, nu, 2))
    for i in range(ncell):
        for j in range(nu):
            for k in range(nsp):
                f_face[i, j, 0] += f[i, j, k] * lr[k]
                f_face[i, j, 1] += f[i, j, k] * ll[k]
    f_int = np.zeros((ncell + 1, nu))
    for fc in range(ncell + 1):
        f_int[fc] = f_face[f2e[fc, 0], :, 1] * (1.0 - delta) + f_face[f2e[fc, 1], :, 0] * delta
    rhs1 = np.zeros_like(u)
    for i in range(ncell):
        for j in range(nu):
            for p in range(nsp):
                for k in range(nsp):
                    rhs1[i, j, p] += f[i, j, k] * lpdm[p, k]
    du = np.zeros_like(u)
    for i in range(ncell):
        for j in range(nu):
            for p in range(nsp):
                du[i, j, p] = (-(rhs1[i, j, p] + (f_int[e2f[i, 1], j] - f_face[i, j, 1]) * dgl[p]
                                 + (f_int[e2f[i, 0], j] - f_face[i, j, 0]) * dgr[p])
                               + (M[i, j, p] - u[i, j, p]) / tau)
    return du


@pytest.mark.parametrize("script", ["bgk_wave", "advection_kinetic"])
def test_oracle_bgk_residual_is_the_script(frgpu, oracle, script):
    rng = np.random.default_rng(5)
    if script == "bgk_wave":
        nx, deg, nu, x0, x1, tau, closure, a = 20, 2, 100, 0.0, 1.0, 1e-2, 0, 1.0
        du_ = 10 / nu
        v = -5 + (np.arange(nu) + 0.5) * du_
    else:
        nx, deg, nu, x0, x1, tau, closure, a = 100, 2, 28, -1.0, 1.0, 0.002, 1, 1.0
        du_ = 10 / nu
        v = -5 + (np.arange(nu) + 0.5) * du_
    w = np.full(nu, du_)
    ps = frgpu.FRPSpace1D(x0, x1, nx, deg)
    po = oracle_space1d(ps, x0, x1, nx, deg)
    rho = 1 + 0.1 * np.sin(2 * np.pi * ps.xpg) + 0.01 * rng.standard_normal(ps.xpg.shape)
    u = np.zeros((nx, nu, deg + 1), order="F")
    for k in range(deg + 1):
        u[:, :, k] = rho[:, k, None] * np.sqrt(1 / np.pi) * np.exp(-(v[None, :] - 1.0) ** 2)
    u *= 1 + 0.01 * rng.standard_normal(u.shape)
    dx = np.full(nx, (x1 - x0) / nx)
    ops = (np.asarray(ps.ll), np.asarray(ps.lr), np.asarray(ps.dl), np.asarray(ps.dhl), np.asarray(ps.dhr))
    if script == "bgk_wave":
        ref = bgk_wave_mol(u, dx, v, w, *ops, tau)
    else:
        ref = advection_kinetic_mol(u, dx, v, w, a, *ops, tau)
    P = oracle.Problem(oracle.BGK1D, po, tau=tau, a=a, velo=v, weights=w, bgk_closure=closure)
    got = P.rhs(u)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def frode_advection(u, J, ll, lr, lpdm, dgl, dgr, a, bc):
    """frode_advection! (src/Equation/eq_advection.jl:55-77, the Matrix method)
    with advection_dflux!, advection_iflux!, scalar_rhs! and period_advection! /
    dirichlet_advection! (:103-175, src/Equation/eq_scalar.jl:1-12)."""
    ncell, nsp = u.shape
    f = a * u / J[:, None]
    u_face = np.stack([u @ ll, u @ lr], axis=1)
    f_face = np.stack([f @ ll, f @ lr], axis=1)
    f_int = np.zeros(ncell + 1)
    for i in range(1, ncell):
        au = (f_face[i, 0] - f_face[i - 1, 1]) / (u_face[i, 0] - u_face[i - 1, 1] + 1e-8)
        f_int[i] = 0.5 * (f_face[i, 0] + f_face[i - 1, 1]) - 0.5 * abs(au) * (u_face[i, 0] - u_face[i - 1, 1])
    rhs1 = f @ lpdm.T
    du = np.zeros_like(u)
    for p in range(nsp):
        for i in range(1, ncell - 1):
            du[i, p] = -(rhs1[i, p] + (f_int[i] - f_face[i, 0]) * dgl[p] + (f_int[i + 1] - f_face[i, 1]) * dgr[p])
    if bc == "period":
        au = (f_face[0, 0] - f_face[ncell - 1, 1]) / (u_face[0, 0] - u_face[ncell - 1, 1] + 1e-6)
        f_int[0] = 0.5 * (f_face[ncell - 1, 1] + f_face[0, 0]) - 0.5 * abs(au) * (u_face[0, 0] - u_face[ncell - 1, 1])
        f_int[ncell] = f_int[0]
        for p in range(nsp):
            for i in (0, ncell - 1):
                du[i, p] = -(rhs1[i, p] + (f_int[i] - f_face[i, 0]) * dgl[p]
                             + (f_int[i + 1] - f_face[i, 1]) * dgr[p])
    return du


@pytest.mark.parametrize("bc", ["period", "dirichlet"])
@pytest.mark.parametrize("deg", [1, 2, 4])
def test_oracle_advection_residual_is_frode_advection(frgpu, oracle, bc, deg):
    """Config 1's residual: the library's frode_advection! (periodic with the
    1e-6 face epsilon, or Dirichlet ends) against the oracle."""
    nx = 37
    ps = frgpu.FRPSpace1D(0, 1, nx, deg)
    po = oracle_space1d(ps, 0, 1, nx, deg)
    rng = np.random.default_rng(deg)
    u = np.asfortranarray(np.sin(2 * np.pi * ps.xpg) + 0.05 * rng.standard_normal(ps.xpg.shape))
    ref = frode_advection(u, np.full(nx, 0.5 / nx), np.asarray(ps.ll), np.asarray(ps.lr), np.asarray(ps.dl),
                          np.asarray(ps.dhl), np.asarray(ps.dhr), 1.0, bc)
    P = oracle.Problem(oracle.ADVECTION, po, a=1.0, bc=oracle.BC_PERIODIC if bc == "period" else oracle.BC_DIRICHLET)
    np.testing.assert_allclose(P.rhs(u), ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def hll_1d(wL, wR, g):
    """HLL with Davis wave speeds, 1D (the restatement of KitBase.flux_hll!)."""
    def parts(w):
        rho, m, E = w
        U = m / rho
        p = (g - 1) * (E - 0.5 * m * U)
        return np.array([m, m * U + p, (E + p) * U]), U, np.sqrt(g * p / rho)

    fL, uL, cL = parts(wL)
    fR, uR, cR = parts(wR)
    sl, sr = min(uL - cL, uR - cR), max(uL + cL, uR + cR)
    if sl >= 0:
        return fL
    if sr <= 0:
        return fR
    return (sr * fL - sl * fR + sl * sr * (wR - wL)) / (sr - sl)


def frode_euler(u, J, ll, lr, lpdm, dgl, dgr, g, bc):
    """frode_euler! (src/Equation/eq_euler.jl:29-73) with period_euler! /
    dirichlet_euler! (:75-98)."""
    ncell, nsp, _ = u.shape
    f = np.zeros_like(u)
    for j in range(nsp):
        for i in range(ncell):
            rho, m, E = u[i, j]
            U = m / rho
            p = (g - 1) * (E - 0.5 * m * U)
            f[i, j] = np.array([m, m * U + p, (E + p) * U]) / J[i]
    u_face = np.zeros((ncell, 2, 3))
    f_face = np.zeros((ncell, 2, 3))
    for k in range(3):
        u_face[:, 0, k] = u[:, :, k] @ ll
        f_face[:, 0, k] = f[:, :, k] @ ll
        u_face[:, 1, k] = u[:, :, k] @ lr
        f_face[:, 1, k] = f[:, :, k] @ lr
    f_int = np.zeros((ncell + 1, 3))
    for i in range(1, ncell):
        f_int[i] = hll_1d(u_face[i - 1, 1], u_face[i, 0], g)
    rhs1 = np.zeros_like(u)
    for k in range(3):
        rhs1[:, :, k] = f[:, :, k] @ lpdm.T
    du = np.zeros_like(u)

    def combine(i):
        for p in range(nsp):
            for k in range(3):
                du[i, p, k] = -(rhs1[i, p, k] + (f_int[i, k] / J[i] - f_face[i, 0, k]) * dgl[p]
                                + (f_int[i + 1, k] / J[i] - f_face[i, 1, k]) * dgr[p])

    for i in range(1, ncell - 1):
        combine(i)
    if bc == "period":
        f_int[0] = hll_1d(u_face[ncell - 1, 1], u_face[0, 0], g)
        f_int[ncell] = hll_1d(u_face[ncell - 1, 1], u_face[0, 0], g)
        for i in (0, ncell - 1):
            combine(i)
    return du


@pytest.mark.parametrize("bc", ["period", "dirichlet"])
@pytest.mark.parametrize("deg", [1, 2, 3])
def test_oracle_euler1d_residual_is_frode_euler(frgpu, oracle, bc, deg):
    """The 1D Euler residual of euler_highlevel.jl's FREulerProblem against the
    oracle (HLL restated, as in the 2D transcription)."""
    nx, g = 29, 1.4
    ps = frgpu.FRPSpace1D(0, 1, nx, deg)
    po = oracle_space1d(ps, 0, 1, nx, deg)
    x = np.asarray(ps.xpg)
    rng = np.random.default_rng(11 + deg)
    rho = 1 + 0.2 * np.sin(2 * np.pi * x) + 0.01 * rng.standard_normal(x.shape)
    U = 0.5 + 0.1 * np.cos(2 * np.pi * x)
    p = 1 + 0.1 * np.sin(4 * np.pi * x)
    u = np.zeros(x.shape + (3,), order="F")
    u[..., 0], u[..., 1], u[..., 2] = rho, rho * U, p / (g - 1) + 0.5 * rho * U * U
    ref = frode_euler(u, np.full(nx, 0.5 / nx), np.asarray(ps.ll), np.asarray(ps.lr), np.asarray(ps.dl),
                      np.asarray(ps.dhl), np.asarray(ps.dhr), g, bc)
    P = oracle.Problem(oracle.EULER1D, po, gamma=g, flux=oracle.FLUX_HLL,
                       bc=oracle.BC_PERIODIC if bc == "period" else oracle.BC_DIRICHLET)
    np.testing.assert_allclose(P.rhs(u), ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def script_filter_loop(u, V, iV, deg, lam=5e-4, kappa=9.0):
    """The indicator + filter loop of example/shock-vortex.jl:308-321 (its 1:3
    blocks are p = 2), with shock_detector (src/dissipation.jl:13-23) and
    KitBase's :l2 modal_filter! restated (u_q / (1 + lam q^2 (q + 1)^2) on the
    flat mode index)."""
    import math

    u = u.copy()
    flags = np.zeros(u.shape[:2], dtype=int)
    S0 = -3.0 * math.log10(deg)
    q = np.arange(u.shape[2] * u.shape[3])
    for i in range(u.shape[0]):
        for j in range(u.shape[1]):
            uh = iV @ u[i, j, :, :, 0].ravel(order="F")
            su = uh[-1] ** 2 / np.sum(uh ** 2)
            Se = math.log10(su) if su > 0 else -math.inf
            if Se < S0 - kappa:
                sigma = 1.0
            elif S0 - kappa <= Se < S0 + kappa:
                sigma = 0.5 * (1.0 - math.sin(0.5 * math.pi * (Se - S0) / kappa))
            else:
                sigma = 0.0
            if sigma < 0.99:
                flags[i, j] = 1
                for s in range(4):
                    uh = iV @ u[i, j, :, :, s].ravel(order="F")
                    uh = uh / (1 + lam * (q * q) * (q + 1) ** 2)
                    u[i, j, :, :, s] = (V @ uh).reshape(u.shape[2], u.shape[3], order="F")
    return u, flags


def test_oracle_filter_is_the_script_loop(frgpu, oracle):
    """The post-step filter of the shock-vortex script (p = 2, lambda = 5e-4,
    kappa = 9) on a state with smooth and discontinuous elements: the same
    elements flagged and the same filtered state as the oracle."""
    nx, ny, deg = 12, 7, 2
    ps = frgpu.FRPSpace2D(0, 2, nx, 0, 1, ny, deg)
    po = oracle_space2d(ps, 0, 2, nx, 0, 1, ny, deg)
    X, Y = ps.xpg[..., 0], ps.xpg[..., 1]
    rho = np.where(X < 0.7 + 0.3 * Y, 1.0, 1.6) + 0.05 * np.sin(5 * X) * np.cos(3 * Y)
    u = np.zeros(X.shape + (4,), order="F")
    u[..., 0], u[..., 1], u[..., 2], u[..., 3] = rho, 0.3 * rho, 0.1 * rho, 2.5 + 0.05 * rho
    ref, ref_flags = script_filter_loop(u, np.asarray(ps.V), np.asarray(ps.iV), deg)
    P = oracle.Problem(oracle.EULER2D, po, gamma=1.4, flux=oracle.FLUX_HLL)
    got, flags, n = P.filter2d(u, 5e-4, -3.0 * np.log10(deg), 9.0)
    assert 0 < n < nx * ny
    np.testing.assert_array_equal(flags, ref_flags)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13)


def positive_limiter_vector(u, weights, ll, lr):
    """positive_limiter(u::AbstractVector, weights, ll, lr) (src/dissipation.jl:38-58)."""
    u = u.copy()
    um = np.sum(u * weights) / np.sum(weights)
    ub = [np.dot(u, ll), np.dot(u, lr)]
    eps = min(1e-13, um)
    theta = min(min(ub), np.min(u))
    t = min((um - eps) / (um - theta + 1e-8), 1.0)
    assert 0 < t <= 1
    return t * (u - um) + um


def test_oracle_limiter_is_positive_limiter(frgpu, oracle):
    """The scalar positive_limiter against the oracle's restatement: elements
    whose traces dip below zero are pulled toward their mean, the others stay.
    (The Euler form cannot be run as the reference writes it once it acts: a
    negative density at a trace sends it into the energy corrector, whose
    `minimum(tj, t0)` (src/dissipation.jl:116, :199) has no method; the oracle
    restates the intended t2 = min(minimum(tj), t0).)"""
    nx, deg = 24, 3
    ps = frgpu.FRPSpace1D(0, 1, nx, deg)
    po = oracle_space1d(ps, 0, 1, nx, deg)
    ll, lr, w = np.asarray(ps.ll), np.asarray(ps.lr), np.asarray(ps.wp) / 2.0
    rng = np.random.default_rng(9)
    # per element a positive mean m with a linear slope A (up to 1.5 m): the
    # traces of the steeper elements go negative
    xi = np.asarray(ps.xpl)[None, :]
    m = rng.uniform(0.2, 1.0, (nx, 1))
    A = rng.uniform(0.0, 1.5, (nx, 1)) * m
    s = np.asfortranarray(m + A * xi)
    ref = np.stack([positive_limiter_vector(s[i], w, ll, lr) for i in range(nx)])
    got, _ = oracle.Problem(oracle.ADVECTION, po, a=1.0).positive_limiter(s, w)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-14)
    limited = np.abs(ref - s).max(axis=1) > 1e-12
    assert 0 < limited.sum() < nx
