"""Pin the CPU oracle: golden setup-math vectors, the reference's own identity
checks, analytic known answers for the residuals, convergence order and
conservation.  CPU only."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "setup_math.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.mark.parametrize("deg", [1, 2, 3, 4, 5])
def test_setup_math_matches_golden(oracle, gold, deg):
    x, w = oracle.gauss_legendre(deg + 1)
    np.testing.assert_allclose(x, gold[f"x{deg}"], rtol=0, atol=2e-16)
    np.testing.assert_allclose(w, gold[f"w{deg}"], rtol=0, atol=5e-16)
    xn, wn = np.polynomial.legendre.leggauss(deg + 1)
    np.testing.assert_allclose(x, xn, atol=1e-15)
    np.testing.assert_allclose(oracle.lagrange_point(x, -1.0), gold[f"ll{deg}"], atol=5e-15)
    np.testing.assert_allclose(oracle.lagrange_point(x, 1.0), gold[f"lr{deg}"], atol=5e-15)
    np.testing.assert_allclose(oracle.dlagrange(x), gold[f"dl{deg}"], atol=5e-14)
    for name in ("radau", "sd", "huynh"):
        gl, gr = oracle.dcorrection(name, deg, x)
        np.testing.assert_allclose(gl, gold[f"{name}_l{deg}"], atol=5e-14)
        np.testing.assert_allclose(gr, gold[f"{name}_r{deg}"], atol=5e-14)
    np.testing.assert_allclose(oracle.vandermonde_1d(deg, x), gold[f"V{deg}"], atol=5e-15)


@pytest.mark.parametrize("deg", [1, 2, 3, 4, 5])
def test_vandermonde_lagrange_identities(oracle, deg):
    """example/vandermonde_lagrange.jl:14,15,25: ll, lr and dl equal the
    Vandermonde-based construction V' \\ psi_f and V' \\ Vr."""
    ps = oracle.Space1D(0, 1, 100, deg)
    V = oracle.vandermonde_1d(deg, ps.xpl)
    psi = oracle.vandermonde_1d(deg, [-1.0, 1.0])
    lf = np.linalg.solve(V.T, psi.T).T
    np.testing.assert_allclose(lf[0], ps.ll, atol=1e-13)
    np.testing.assert_allclose(lf[1], ps.lr, atol=1e-13)
    Vr = oracle.dvandermonde_1d(deg, ps.xpl)
    dl = np.linalg.solve(V.T, Vr.T).T
    np.testing.assert_allclose(dl, ps.dl, atol=1e-12)
    # row sums of the differentiation matrix vanish, it differentiates x exactly,
    # Lagrange weights sum to one
    np.testing.assert_allclose(ps.dl.sum(axis=1), 0.0, atol=1e-12)
    np.testing.assert_allclose(ps.dl @ ps.xpl, 1.0, atol=1e-12)
    assert abs(ps.ll.sum() - 1) < 1e-14 and abs(ps.lr.sum() - 1) < 1e-14


@pytest.mark.parametrize("deg", [1, 2, 3, 4])
def test_correction_endpoint_values(oracle, deg):
    """g_L(-1) = 1, g_L(1) = 0 (and mirrored for g_R): integrate the nodal
    derivative polynomial (degree deg+... exact via quadrature on deg+2 points)."""
    xs, ws = np.polynomial.legendre.leggauss(deg + 3)
    gl, gr = oracle.dcorrection("radau", deg, xs)
    # int_{-1}^{1} g_L' = g_L(1) - g_L(-1) = -1
    assert abs(np.dot(ws, gl) + 1.0) < 1e-13
    assert abs(np.dot(ws, gr) - 1.0) < 1e-13


def test_shock_detector_cases(oracle):
    """src/dissipation.jl:13-23 on the inputs of test/runtests.jl:12-14."""
    assert oracle.shock_detector(-np.inf, 3) is False
    assert oracle.shock_detector(np.log10(0.1), 3) is True
    assert oracle.shock_detector(np.log10(1e5), 3) is True
    S0 = -3 * np.log10(3)
    assert oracle.shock_detector(S0 - 4.0 - 1e-9, 3) is False
    # sigma = 0.5(1 - sin(pi/2 (Se-S0)/k)) < 0.99 unless Se is close to S0 - k
    assert oracle.shock_detector(S0 - 3.9, 3) is False
    assert oracle.shock_detector(S0, 3) is True


def test_error_norms(oracle):
    """src/tools.jl:43-53 (dx inside the square for L2)."""
    rng = np.random.default_rng(0)
    u, ue = rng.random(7), rng.random(7)
    dx = 0.1
    assert abs(oracle.l1_error(u, ue, dx) - np.sum(np.abs(u - ue) * dx)) < 1e-15
    assert abs(oracle.l2_error(u, ue, dx) - np.sqrt(np.sum((np.abs(u - ue) * dx) ** 2))) < 1e-15
    assert abs(oracle.linf_error(u, ue, dx) - np.max(np.abs(u - ue) * dx)) < 1e-15


@pytest.mark.parametrize("deg", [1, 2, 3, 4])
def test_advection_residual_exact_for_polynomials(oracle, deg):
    """For a global polynomial of degree <= deg the face traces agree, the
    Roe flux is the physical flux, the corrections vanish and the residual is
    exactly -a u'(x) on interior elements."""
    ps = oracle.Space1D(-1, 1, 12, deg)
    c = np.random.default_rng(deg).standard_normal(deg + 1)
    u = np.polynomial.polynomial.polyval(ps.xpg, c)
    du_exact = -0.7 * np.polynomial.polynomial.polyval(ps.xpg, np.polynomial.polynomial.polyder(c))
    P = oracle.Problem(oracle.ADVECTION, ps, a=0.7, bc=oracle.BC_DIRICHLET)
    du = P.rhs(u)
    np.testing.assert_allclose(du[1:-1], du_exact[1:-1], atol=1e-11)
    assert np.all(du[0] == 0) and np.all(du[-1] == 0)


def test_euler2d_residual_exact_for_linear_density(oracle):
    """Uniform velocity and pressure make the Euler flux linear in density:
    for a density linear in x and y the residual is exact,
    d(rho)/dt = -(u rho_x + v rho_y)."""
    ps = oracle.Space2D(0, 1, 6, 0, 1, 5, 3)
    g, U, V, p = 1.4, 0.8, -0.3, 1.0
    X, Y = ps.xpg[..., 0], ps.xpg[..., 1]
    rho = 2.0 + 0.3 * X - 0.2 * Y
    u = np.zeros((6, 5, 4, 4, 4), order="F")
    u[..., 0] = rho
    u[..., 1] = rho * U
    u[..., 2] = rho * V
    u[..., 3] = p / (g - 1) + 0.5 * rho * (U * U + V * V)
    P = oracle.Problem(oracle.EULER2D, ps, flux=oracle.FLUX_HLL, gamma=g,
                       bcs=[oracle.BC_COPY] * 4)
    du = P.rhs(u)
    drho = -(U * 0.3 + V * -0.2)
    inner = (slice(1, -1), slice(1, -1))
    np.testing.assert_allclose(du[inner][..., 0], drho, atol=1e-11)
    np.testing.assert_allclose(du[inner][..., 1], drho * U, atol=1e-11)
    np.testing.assert_allclose(du[inner][..., 3], drho * 0.5 * (U * U + V * V), atol=1e-11)


def test_advection_sine_one_period(oracle):
    """Config 1 (periodic [0,1], 100 elements, p=2, Radau, SSPRK3 at CFL 0.1 to
    t=1): the wave returns to its initial condition up to the scheme error."""
    ps = oracle.Space1D(0, 1, 100, 2)
    u0 = np.sin(2 * np.pi * ps.xpg)
    P = oracle.Problem(oracle.ADVECTION, ps, a=1.0)
    dt = 0.1 * 0.01
    u1 = P.ssprk3(u0, dt, 1000)
    assert np.max(np.abs(u1 - u0)) < 5e-6
    # mass is conserved to round-off
    assert abs(np.sum(u1 @ ps.wp) - np.sum(u0 @ ps.wp)) < 1e-12


def test_euler1d_density_wave_convergence(oracle):
    """example/euler1d_convergence.jl:58-150 setup (p=3, gamma=5/3, density
    wave with u = p = 1): the error falls at about order p+1."""
    errs = []
    for ne in (8, 16, 32):
        ps = oracle.Space1D(0, 1, ne, 3)
        g = 5 / 3
        rho = 1 + 0.2 * np.sin(2 * np.pi * ps.xpg)
        u = np.zeros((ne, 4, 3), order="F")
        u[..., 0] = rho
        u[..., 1] = rho
        u[..., 2] = 1 / (g - 1) + 0.5 * rho
        P = oracle.Problem(oracle.EULER1D, ps, gamma=g, flux=oracle.FLUX_HLL)
        dt = 0.08 * (1 / ne) / 2.5
        n = int(round(0.2 / dt))
        dt = 0.2 / n
        u1 = P.ssprk3(u, dt, n)
        exact = 1 + 0.2 * np.sin(2 * np.pi * (ps.xpg - 0.2))
        errs.append(np.max(np.abs(u1[..., 0] - exact)))
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert np.all(rates > 3.3), (errs, rates)


def test_euler2d_conservation_periodic(oracle):
    ps = oracle.Space2D(0, 1, 8, 0, 1, 8, 2)
    g = 1.4
    X, Y = ps.xpg[..., 0], ps.xpg[..., 1]
    rho = 1 + 0.2 * np.sin(2 * np.pi * (X + Y))
    u = np.zeros((8, 8, 3, 3, 4), order="F")
    u[..., 0] = rho
    u[..., 1] = rho
    u[..., 2] = rho
    u[..., 3] = 1 / (g - 1) + rho
    P = oracle.Problem(oracle.EULER2D, ps, flux=oracle.FLUX_LF, gamma=g)
    s0 = P.conserved_sums2d(u)
    u1 = P.ssprk3(u, 2e-3, 20)
    np.testing.assert_allclose(P.conserved_sums2d(u1), s0, rtol=0, atol=1e-13)


def test_bgk_moments_conserved(oracle):
    """The BGK relaxation conserves mass; the transport is conservative."""
    ps = oracle.Space1D(0, 1, 16, 3)
    nv = 64
    dv = 16 / nv
    v = -8 + (np.arange(nv) + 0.5) * dv
    w = np.full(nv, dv)
    rho = 1 + 0.1 * np.sin(2 * np.pi * ps.xpg)
    f = np.zeros((16, nv, 4), order="F")
    for k in range(4):
        f[:, :, k] = rho[:, k, None] * np.sqrt(1 / np.pi) * np.exp(-(v[None, :] - 1) ** 2)
    P = oracle.Problem(oracle.BGK1D, ps, tau=1e-2, velo=v, weights=w)
    mass0 = np.einsum("ivk,v,k->", f, w, ps.wp)
    f1 = P.ssprk3(f, 1e-4, 20)
    mass1 = np.einsum("ivk,v,k->", f1, w, ps.wp)
    assert abs(mass1 - mass0) < 1e-12


def test_mlp_gradient_matches_finite_difference(oracle):
    rng = np.random.default_rng(1)
    nin, nh = 32, 64
    n_params = nh * nin + nh + nh * nh + nh + nh + 1
    P = rng.standard_normal(n_params) * 0.2
    x = rng.standard_normal((5, nin))
    t = (rng.random(5) > 0.5).astype(np.float64)
    loss, g = oracle.mlp_loss_grad(P, x, t)
    for idx in rng.choice(n_params, 12, replace=False):
        e = np.zeros(n_params)
        e[idx] = 1e-6
        lp, _ = oracle.mlp_loss_grad(P + e, x, t)
        lm, _ = oracle.mlp_loss_grad(P - e, x, t)
        assert abs((lp - lm) / 2e-6 - g[idx]) < 1e-7 * max(1, abs(g[idx]))


# ---- positivity-preserving limiter (src/dissipation.jl:38-216) -------------
def _euler2d_state(O, sp, seed, gamma=1.4):
    rng = np.random.default_rng(seed)
    shape = (sp.nx, sp.ny, sp.np, sp.np)
    rho = 1 + 0.1 * rng.standard_normal(shape)
    U, V = 0.3 * rng.standard_normal(shape), 0.2 * rng.standard_normal(shape)
    p = 1 + 0.1 * rng.standard_normal(shape)
    u = np.zeros(shape + (4,), order="F")
    u[..., 0], u[..., 1], u[..., 2] = rho, rho * U, rho * V
    u[..., 3] = p / (gamma - 1) + 0.5 * rho * (U ** 2 + V ** 2)
    return u


def _prim_p(w, gamma=1.4):
    return (gamma - 1) * (w[..., -1] - 0.5 * np.sum(w[..., 1:-1] ** 2, axis=-1) / w[..., 0])


def test_positive_limiter_reference_test_inputs(oracle):
    """The reference's own calls (test/runtests.jl:25-26) on constant states
    leave them unchanged."""
    O = oracle
    sp = O.Space1D(0, 1, 20, 5)
    u = np.ones((1, 6), order="F")
    out, n = O.Problem(O.ADVECTION, O.Space1D(0, 1, 1, 5)).positive_limiter(u, w=np.full(6, 1 / 6))
    assert n == 0 and np.array_equal(out, u)
    u3 = np.ones((1, 6, 3), order="F")
    out3, n3 = O.Problem(O.EULER1D, O.Space1D(0, 1, 1, 5), gamma=5 / 3).positive_limiter(u3, w=np.full(6, 1 / 6))
    assert n3 == 0 and np.array_equal(out3, u3)
    assert sp.np == 6


@pytest.mark.parametrize("deg", [2, 3])
def test_positive_limiter_2d_restores_positivity_and_keeps_means(oracle, deg):
    O = oracle
    sp = O.Space2D(0, 1, 5, 0, 1, 4, deg)
    pr = O.Problem(O.EULER2D, sp, gamma=1.4)
    u = _euler2d_state(O, sp, deg)
    u[1, 0, 1, 1, 0] = -0.3          # negative density at a solution point
    u[2, 1, 0, deg, 3] = 0.01        # energy too low: negative pressure
    u[4, 3, 2, 2, 3] = -0.5          # negative energy inside an element
    out, n = pr.positive_limiter(u)
    assert n == 3
    wq = np.asarray(sp.wp).ravel(order="F") / 4
    for i in range(sp.nx):
        for j in range(sp.ny):
            for m in range(4):
                before = u[i, j, :, :, m].ravel(order="F") @ wq
                after = out[i, j, :, :, m].ravel(order="F") @ wq
                assert abs(after - before) <= 1e-13 * max(1.0, abs(before))
    # positive density and pressure (pressure down to eps = 1e-13, up to the
    # round-off of E - |m|^2 / (2 rho) at O(1) energies)
    assert np.all(out[..., 0] > 0)
    assert np.all(_prim_p(out) >= -1e-13)
    # elements the limiter leaves alone move by round-off only ((u - mean) + mean)
    assert np.max(np.abs(out[0, 0] - u[0, 0])) < 1e-14


def test_positive_limiter_1d_forms(oracle):
    O = oracle
    sp = O.Space1D(0, 1, 6, 3)
    rng = np.random.default_rng(3)
    u = np.zeros((6, 4, 3), order="F")
    rho = 1 + 0.1 * rng.standard_normal((6, 4))
    u[..., 0], u[..., 1] = rho, 0.2 * rho
    u[..., 2] = 1 / 0.4 + 0.5 * rho * 0.04
    u[2, 1, 0] = -0.2
    u[4, 3, 2] = 0.0
    out, n = O.Problem(O.EULER1D, sp, gamma=1.4).positive_limiter(u)
    assert n == 2 and np.all(out[..., 0] > 0) and np.all(_prim_p(out) >= -1e-13)
    w = np.asarray(sp.wp) / 2
    assert np.allclose(np.einsum("iqm,q->im", out, w), np.einsum("iqm,q->im", u, w), rtol=0, atol=1e-13)
    s = 1 + 0.5 * np.sin(2 * np.pi * np.asarray(sp.xpg))
    s[3, 2] = -0.4
    outs, ns = O.Problem(O.ADVECTION, sp).positive_limiter(s)
    assert ns == 1 and outs[3].min() > 0 and np.allclose((outs[3] - s[3]) @ np.asarray(sp.wp), 0, atol=1e-14)


# ---- explicit Runge-Kutta tableaux (OrdinaryDiffEq's fixed-step methods) ----
def test_erk_tableaux_order_conditions():
    """The tableaux frgpu ships satisfy their order conditions (Tsit5: fifth
    order, all 17 conditions up to order 5; RK4: fourth; the two-stage methods:
    second), so a transcription error in a coefficient cannot pass."""
    import frgpu

    def conds(A, b, order):
        c = A.sum(1)
        out = [(b.sum(), 1.0), (b @ c, 1 / 2)]
        if order >= 3:
            out += [(b @ c ** 2, 1 / 3), (b @ A @ c, 1 / 6)]
        if order >= 4:
            out += [(b @ c ** 3, 1 / 4), (b @ (c * (A @ c)), 1 / 8), (b @ A @ c ** 2, 1 / 12), (b @ A @ A @ c, 1 / 24)]
        if order >= 5:
            out += [(b @ c ** 4, 1 / 5), (b @ (c ** 2 * (A @ c)), 1 / 10), (b @ (c * (A @ c ** 2)), 1 / 15),
                    (b @ (c * (A @ A @ c)), 1 / 30), (b @ (A @ c) ** 2, 1 / 20), (b @ A @ c ** 3, 1 / 20),
                    (b @ A @ (c * (A @ c)), 1 / 40), (b @ A @ A @ c ** 2, 1 / 60), (b @ A @ A @ A @ c, 1 / 120)]
        return out

    for alg, order in ((frgpu.Midpoint(), 2), (frgpu.Heun(), 2), (frgpu.Ralston(), 2), (frgpu.SSPRK22(), 2),
                       (frgpu.RK4(), 4), (frgpu.Tsit5(), 5)):
        for got, want in conds(alg.A, alg.b, order):
            assert abs(got - want) < 1e-13, (alg, got, want)
    with pytest.raises(ValueError):
        frgpu.ExplicitRK([[0, 1], [0, 0]], [0.5, 0.5])


def test_oracle_erk_reproduces_ssprk3_and_rk4(oracle):
    """fro_erk with the SSPRK33 tableau matches fro_ssprk3 to round-off, and one
    RK4 step matches the classical formula written out over the oracle's rhs."""
    O = oracle
    sp = O.Space1D(0, 1, 20, 3)
    pr = O.Problem(O.ADVECTION, sp, a=1.0)
    u0 = np.sin(2 * np.pi * np.asarray(sp.xpg))
    A = np.array([[0, 0, 0], [1, 0, 0], [0.25, 0.25, 0]])
    b = np.array([1 / 6, 1 / 6, 2 / 3])
    ua, ub = pr.ssprk3(u0, 1e-3, 10), pr.erk(u0, 1e-3, 10, A, b)
    assert np.max(np.abs(ua - ub)) < 1e-14
    A4 = np.array([[0, 0, 0, 0], [0.5, 0, 0, 0], [0, 0.5, 0, 0], [0, 0, 1, 0]])
    b4 = np.array([1, 2, 2, 1]) / 6
    dt = 2e-3
    k1 = pr.rhs(u0)
    k2 = pr.rhs(u0 + 0.5 * dt * k1)
    k3 = pr.rhs(u0 + 0.5 * dt * k2)
    k4 = pr.rhs(u0 + dt * k3)
    want = u0 + dt * (k1 + 2 * k2 + 2 * k3 + k4) / 6
    assert np.max(np.abs(pr.erk(u0, dt, 1, A4, b4) - want)) < 1e-13


def test_euler2d_metric_free_stream_and_diagonal(oracle):
    """The 2D residual with a per-point metric (dudt! of example/shock-vortex.jl
    with iJ[i, j][k, l]): a uniform state stays put on rectangles of different
    sizes (a diagonal metric constant within each element, varying between
    elements), and the rectangles' own diag(2/dx, 2/dy) gives the same bits as
    the uniform path.  (dudt! scales the interface fluxes by iJ11 and iJ22
    only, so with off-diagonal terms or a metric varying inside an element the
    formula it defines does not keep a uniform state; that is the reference's
    formula, reproduced as it is.)"""
    O = oracle
    sp = O.Space2D(0, 1, 5, 0, 1, 4, 3)
    pr = O.Problem(O.EULER2D, sp, gamma=1.4, flux=O.FLUX_HLL)
    shape = (5, 4, 4, 4)
    u = np.zeros(shape + (4,), order="F")
    u[..., 0], u[..., 1], u[..., 2], u[..., 3] = 1.2, 0.3, -0.2, 2.9
    iJ = np.zeros(shape + (2, 2), order="F")
    ix = 10.0 * (1 + 0.3 * np.arange(5))[:, None, None, None]
    iy = 8.0 * (1 + 0.2 * np.arange(4))[None, :, None, None]
    iJ[..., 0, 0], iJ[..., 1, 1] = ix + 0 * iJ[..., 0, 0], iy + 0 * iJ[..., 1, 1]
    pr.set_metric(iJ)
    assert np.max(np.abs(pr.rhs(u))) < 1e-12
    iJ[..., 0, 1] = 1.5          # off-diagonal: dudt!'s formula moves a uniform state
    pr.set_metric(iJ)
    assert np.max(np.abs(pr.rhs(u))) > 1e-3
    rng = np.random.default_rng(5)
    w = u + 0.05 * rng.standard_normal(u.shape)
    iJ[..., 0, 0], iJ[..., 1, 1], iJ[..., 0, 1], iJ[..., 1, 0] = sp.iJx, sp.iJy, 0.0, 0.0
    pr.set_metric(iJ)
    r_met = pr.rhs(w)
    pr.set_metric(None)
    assert np.array_equal(r_met, pr.rhs(w))


def parallelogram_metric(nx, ny, np_, dx, dy, s=0.3, t=-0.2):
    """Metric and unit face normals of the affine mesh x = X + s Y, y = Y + t X
    of nx x ny cells dx x dy (every element the same parallelogram):
    iJ = J^-1 with J = [[dx/2, s dy/2], [t dx/2, dy/2]], normals of the x faces
    along grad(xi) ~ (1, -s) and of the y faces along grad(eta) ~ (-t, 1)."""
    J = np.array([[dx / 2, s * dy / 2], [t * dx / 2, dy / 2]])
    iJ = np.zeros((nx, ny, np_, np_, 2, 2), order="F")
    iJ[...] = np.linalg.inv(J)
    n1 = np.zeros((nx + 1, ny, 2), order="F")
    n2 = np.zeros((nx, ny + 1, 2), order="F")
    n1[...] = np.array([1.0, -s]) / np.hypot(1.0, s)
    n2[...] = np.array([-t, 1.0]) / np.hypot(1.0, t)
    return iJ, n1, n2


@pytest.mark.parametrize("flux", ["lf", "hll"])
def test_euler2d_parallelogram_free_stream(oracle, flux):
    """Straight-sided quadrilaterals with face normals (dev/parallelogram.jl:
    interface fluxes solved along each face's unit normal and scaled by
    (iJ n)_1 on x faces, (iJ n)_2 on y faces): a uniform flow stays uniform on
    sheared parallelograms, which the normal-free formula does not manage."""
    O = oracle
    sp = O.Space2D(0, 1, 5, 0, 1, 4, 3)
    pr = O.Problem(O.EULER2D, sp, gamma=1.4, flux=O.FLUX_HLL if flux == "hll" else O.FLUX_LF)
    u = np.zeros((5, 4, 4, 4, 4), order="F")
    u[..., 0], u[..., 1], u[..., 2], u[..., 3] = 1.2, 0.3, -0.2, 2.9
    iJ, n1, n2 = parallelogram_metric(5, 4, 4, 0.2, 0.25)
    pr.set_metric(iJ, n1, n2)
    assert np.max(np.abs(pr.rhs(u))) < 1e-12
    pr.set_metric(iJ)
    assert np.max(np.abs(pr.rhs(u))) > 1e-3
    # the rotated solve with the axes as normals is the Cartesian x-face flux
    iJ[..., 0, 1] = iJ[..., 1, 0] = 0.0
    rng = np.random.default_rng(11)
    w = u + 0.05 * rng.standard_normal(u.shape)
    ax1 = np.zeros_like(n1)
    ax1[..., 0] = 1.0
    ax2 = np.zeros_like(n2)
    ax2[..., 1] = 1.0
    pr.set_metric(iJ, ax1, ax2)
    r_n = pr.rhs(w)
    pr.set_metric(iJ)
    assert np.max(np.abs(r_n - pr.rhs(w))) < 1e-12 * np.max(np.abs(r_n))
