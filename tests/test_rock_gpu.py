"""Stabilised explicit steps on the GPU (frgpu_step_rock, frgpu_spectral_radius)
against the oracle: the recurrence + finishing structure of OrdinaryDiffEq's
ROCK4 as example/advection_kinetic.jl:133-146 uses it, with the built-in RKC2
coefficients and with a ROCK-form coefficient set and an RK4 finishing
procedure; the spectral-radius estimate taken before every step; the
advection-kinetic problem (density-only BGK closure) it is run on."""
import numpy as np
import pytest

from test_parity_gpu import RTOL64, oracle_space1d, oracle_space2d, rel

pytestmark = pytest.mark.gpu

RK4_A = np.array([[0, 0, 0, 0], [0.5, 0, 0, 0], [0, 0.5, 0, 0], [0, 0, 1, 0]], dtype=float)
RK4_B = np.array([1 / 6, 1 / 3, 1 / 3, 1 / 6])


def rock_form():
    """A ROCK-form coefficient set (alpha = 1 + kappa, beta = -kappa, delta = 0)
    of six recurrence stages, with RK4 as the finishing procedure."""
    mu = np.array([0.21, 0.17, 0.15, 0.13, 0.12, 0.11])
    kappa = np.array([0.0, 0.31, 0.42, 0.47, 0.5, 0.52])
    al, be = 1 + kappa, -kappa
    al[0] = be[0] = 0.0
    return al, be, mu, np.zeros(6), RK4_A, RK4_B


def euler2d_pair(frgpu, oracle, precision="fp64", nx=16, ny=8, deg=3):
    ps = frgpu.FRPSpace2D(0, 2, nx, 0, 1, ny, deg)
    po = oracle_space2d(ps, 0, 2, nx, 0, 1, ny, deg)
    X, Y = ps.xpg[..., 0], ps.xpg[..., 1]
    u = np.zeros(X.shape + (4,), order="F")
    r = 1 + 0.2 * np.sin(np.pi * X) * np.cos(2 * np.pi * Y)
    u[..., 0], u[..., 1], u[..., 2] = r, r, 0.5 * r
    u[..., 3] = 1 / 0.4 + 0.5 * r * 1.25
    prob = frgpu.FREuler2DProblem(u, (0, 1), ps, 1.4, flux="hll", precision=precision)
    P = oracle.Problem(oracle.EULER2D, po, gamma=1.4, flux=oracle.FLUX_HLL, bc=oracle.BC_PERIODIC)
    return u, prob, P


def kinetic_pair(frgpu, oracle, tau, nx=100, deg=2, nu=28, precision="fp64"):
    """example/advection_kinetic.jl: x in [-1, 1] with 100 elements, p = 2, 28
    velocities on [-5, 5] (midpoint rule), a = 1, the density-only closure,
    starting from the equilibrium at rho = 1 - sin(pi x)."""
    ps = frgpu.FRPSpace1D(-1, 1, nx, deg)
    po = oracle_space1d(ps, -1, 1, nx, deg)
    du = 10 / nu
    v = -5 + (np.arange(nu) + 0.5) * du
    w = np.full(nu, du)
    rho0 = 1 - np.sin(np.pi * ps.xpg)
    f = np.zeros((nx, nu, deg + 1), order="F")
    for k in range(deg + 1):
        f[:, :, k] = rho0[:, k, None] * np.sqrt(1 / np.pi) * np.exp(-(v[None, :] - 1.0) ** 2)
    prob = frgpu.FRBGKProblem(f, (0, 0.5), ps, v, w, tau, precision=precision, closure="density", a=1.0)
    P = oracle.Problem(oracle.BGK1D, po, tau=tau, a=1.0, velo=v, weights=w, bgk_closure=1)
    return f, prob, P


def test_density_closure_residual_matches_oracle(frgpu, oracle):
    """FP64 within 1e-12 of the oracle.  FP32: the relaxation (M - u)/tau of a
    near-equilibrium state cancels, so the bound scales with max|u| / tau (a few
    FP32 roundings of M and u), not with the residual's own size."""
    tau = 2e-3
    f, prob, P = kinetic_pair(frgpu, oracle, tau)
    ref = P.rhs(f)
    assert rel(prob.rhs(f), ref) < RTOL64
    f32, prob32, _ = kinetic_pair(frgpu, oracle, tau, precision="fp32k")
    assert np.abs(prob32.rhs(f32) - ref).max() < 1e-6 * np.abs(f).max() / tau


@pytest.mark.parametrize("form", ["rkc2", "rock"])
def test_stabilised_step_fp64_bit_identical_on_euler2d(frgpu, oracle, form):
    """FP64 stabilised steps on the 2D Euler problem reproduce the oracle's
    fro_rock bit for bit (recurrence, finishing stages and update)."""
    u, prob, P = euler2d_pair(frgpu, oracle)
    if form == "rkc2":
        al, be, mu, de, _ = frgpu.rkc2_coefficients(7)
        A = b = None
    else:
        al, be, mu, de, A, b = rock_form()
    itg = frgpu.init(prob, dt=2e-3)
    itg.step_rock(al, be, mu, de, A, b, n=3)
    np.testing.assert_array_equal(itg.u, P.rock(u, 2e-3, 3, al, be, mu, de, A, b))


@pytest.mark.parametrize("form", ["rkc2", "rock"])
def test_stabilised_step_on_1d_problems(frgpu, oracle, form):
    """The 1D advection and the BGK problem (density closure) through the same
    recurrence, FP64, against the oracle."""
    if form == "rkc2":
        al, be, mu, de, _ = frgpu.rkc2_coefficients(5)
        A = b = None
    else:
        al, be, mu, de, A, b = rock_form()
    ps = frgpu.FRPSpace1D(0, 1, 40, 3)
    po = oracle_space1d(ps, 0, 1, 40, 3)
    u = np.asfortranarray(np.sin(2 * np.pi * ps.xpg))
    itg = frgpu.init(frgpu.FRAdvectionProblem(u, (0, 1), ps, 1.0), dt=1e-3)
    itg.step_rock(al, be, mu, de, A, b, n=4)
    assert rel(itg.u, oracle.Problem(oracle.ADVECTION, po, a=1.0).rock(u, 1e-3, 4, al, be, mu, de, A, b)) < RTOL64
    f, prob, P = kinetic_pair(frgpu, oracle, 1e-4, nx=20)
    itk = frgpu.init(prob, dt=5e-4)
    itk.step_rock(al, be, mu, de, A, b, n=4)
    assert rel(itk.u, P.rock(f, 5e-4, 4, al, be, mu, de, A, b)) < RTOL64


def test_stabilised_fp32k_close_to_fp64(frgpu, oracle):
    """FP32K: FP32 recurrence and residuals, the step's increment added to the
    high + low pair with the compensated sum."""
    u, prob, P = euler2d_pair(frgpu, oracle, precision="fp32k")
    al, be, mu, de, A, b = rock_form()
    itg = frgpu.init(prob, dt=2e-3)
    itg.step_rock(al, be, mu, de, A, b, n=10)
    assert rel(itg.u, P.rock(u, 2e-3, 10, al, be, mu, de, A, b)) < 2e-6


def test_spectral_radius_matches_oracle(frgpu, oracle):
    """The device power method takes the oracle's iterations to the same
    estimate (the norms differ only in summation order), cold and warm."""
    u, prob, P = euler2d_pair(frgpu, oracle)
    itg = frgpu.init(prob, dt=1e-3)
    r1, k1 = itg.spectral_radius(50)
    o1, ok1, d = P.spectral_radius(u, 50)
    assert k1 == ok1 and k1 > 0
    assert abs(r1 / o1 - 1) < 1e-8
    r2, k2 = itg.spectral_radius(50)
    o2, ok2, _ = P.spectral_radius(u, 50, d)
    assert k2 == ok2
    assert abs(r2 / o2 - 1) < 1e-8


@pytest.mark.parametrize("tau", [1e-4, 1e-5])
def test_rkc2_integrator_on_advection_kinetic(frgpu, oracle, tau):
    """init(prob, RKC2(); dt) on the advection-kinetic problem at the script's
    dt = 0.0005: each step takes the spectral radius, picks the stage count and
    steps, as the oracle does; where RK4 at this dt loses the solution (the
    relaxation eigenvalue -1/tau is far outside its stability interval), the
    stabilised steps stay bounded."""
    f, prob, P = kinetic_pair(frgpu, oracle, tau)
    dt, n = 5e-4, 60
    alg = frgpu.RKC2()
    itg = frgpu.init(prob, alg, dt=dt)
    itg.step(n)
    u, d = f.copy(order="F"), None
    stages = []
    for _ in range(n):
        r, _, d = P.spectral_radius(u, alg.maxiter, d)
        al, be, mu, de, _, _ = alg.coefficients(dt * r)
        stages.append(len(al))
        u = P.rock(u, dt, 1, al, be, mu, de)
    assert itg.stages == stages
    assert rel(itg.u, u) < 1e-10
    assert np.abs(itg.u).max() < 1.2
    rk4 = frgpu.init(kinetic_pair(frgpu, oracle, tau)[1], frgpu.RK4(), dt=dt)
    try:
        rk4.step(n)
        with np.errstate(invalid="ignore"):
            blown = not np.abs(rk4.u).max() < 1e6
    except frgpu.FRGPUError:  # non-finite values reported by the step
        blown = True
    assert blown


def test_step_rkc2_equals_the_host_driven_loop(frgpu, oracle):
    """frgpu_step_rkc2 (spectral radius, stage count and coefficients chosen in
    the library, n steps per call) against the same method driven step by step
    from the host (frgpu_spectral_radius, the Python stage choice and
    coefficients, frgpu_step_rock): the same stage counts and the same bits."""
    dt, n = 5e-4, 40
    a = frgpu.init(kinetic_pair(frgpu, oracle, 1e-4)[1], frgpu.RKC2(), dt=dt)
    a.step(n)
    rk = frgpu.RKC2()
    generic = frgpu.Stabilized(rk.coefficients, "RKC2 from the host", rk.maxiter)
    b = frgpu.init(kinetic_pair(frgpu, oracle, 1e-4)[1], generic, dt=dt)
    b.step(n)
    assert a.stages == b.stages and len(a.stages) == n
    assert np.array_equal(a.u, b.u)


def test_rock_graphs_follow_coefficients(frgpu, oracle):
    """Alternating coefficient sets replay their own captured graphs; the
    result equals stepping each set in turn on the oracle."""
    u, prob, P = euler2d_pair(frgpu, oracle)
    sets = [frgpu.rkc2_coefficients(s)[:4] for s in (3, 4, 3, 5, 4)]
    itg = frgpu.init(prob, dt=1e-3)
    ref = u
    for al, be, mu, de in sets:
        itg.step_rock(al, be, mu, de)
        ref = P.rock(ref, 1e-3, 1, al, be, mu, de)
    np.testing.assert_array_equal(itg.u, ref)


def test_fp32k_mixed_steps_follow_the_state(frgpu, oracle):
    """FP32K SSPRK3 steps move the high part between two buffers; the ERK and
    stabilised-step graphs captured before must follow it (a graph keyed on
    the buffer it updates), so a mixed sequence matches the oracle's."""
    u, prob, P = euler2d_pair(frgpu, oracle, precision="fp32k")
    al, be, mu, de, A, b = rock_form()
    rk4 = frgpu.RK4()  # four stages: the generic ERK graph (two-stage tableaux run fused)
    dt = 1e-3
    itg = frgpu.init(prob, dt=dt)
    ref = u
    for k in range(3):
        frgpu.Integrator.step(itg, 1)  # SSPRK3 (itg.alg is None)
        ref = P.ssprk3(ref, dt, 1)
        check = frgpu._lib.check
        check(frgpu._lib.lib().frgpu_step_erk(prob._h, 4, frgpu._lib.dptr(rk4.A), frgpu._lib.dptr(rk4.b), dt, 1))
        ref = P.erk(ref, dt, 1, rk4.A, rk4.b)
        itg.step_rock(al, be, mu, de, A, b, n=1)
        ref = P.rock(ref, dt, 1, al, be, mu, de, A, b)
    assert rel(itg.u, ref) < 2e-6
