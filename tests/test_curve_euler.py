"""dev/curve_euler.jl: 2D Euler on a polar grid of bilinear quadrilaterals (the
half annulus 1 <= r <= 6, 0 <= theta <= pi of KitBase.CSpace2D) with the
per-point inverse Jacobian, a central interaction flux with the fixed
dissipation 40 dt on the transformed-flux traces, and only the interior
elements updated.

CPU: the oracle's FRO_FLUX_CENTRAL residual against a literal numpy
transcription of the script's dudt! (lines 64-152, with its nx = size(u, 1) - 2
and ny = size(u, 2) - 2: the last two rows and columns take no part, and of the
rest only the interior is updated), which pins the restatement to the script.
GPU (marked): libfrgpu's residual bit for bit against the oracle, and Midpoint
steps as the script takes them."""
import numpy as np
import pytest

from test_parity_gpu import oracle_space2d

GAMMA = 5 / 3  # the script's Gas(..., 5/3, ...)
C_DISS = 40 * 0.002  # 40 dt with the script's dt = 0.002


def initial_state(xpg):
    """u0 of the script (lines 46-51): a density bump at (0, 3), at rest,
    prim = [rho, 0, 0, 1] (lambda = rho / (2 p) = 1, so p = rho / 2)."""
    rho = np.maximum(np.exp(-10 * (xpg[..., 0] ** 2 + (xpg[..., 1] - 3.0) ** 2)), 1e-2)
    u = np.zeros(rho.shape + (4,), order="F")
    u[..., 0] = rho
    u[..., 3] = 0.5 * rho / (GAMMA - 1)
    return u


def euler_flux(w):
    rho, mx, my, E = w
    U, V = mx / rho, my / rho
    p = (GAMMA - 1) * (E - 0.5 * rho * (U * U + V * V))
    return np.array([mx, mx * U + p, my * U, (E + p) * U]), np.array([my, mx * V, my * V + p, (E + p) * V])


def script_dudt(u, iJ, ll, lr, dhl, dhr, lpdm, c):
    """The active dudt! of dev/curve_euler.jl, transcribed loop for loop
    (0-based); J^-1 is iJ."""
    du = np.zeros_like(u)
    nx, ny, nsp = u.shape[0] - 2, u.shape[1] - 2, u.shape[2]
    f = np.zeros((nx, ny, nsp, nsp, 4, 2))
    for i in range(nx):
        for j in range(ny):
            for k in range(nsp):
                for l in range(nsp):
                    fg, gg = euler_flux(u[i, j, k, l, :])
                    for m in range(4):
                        f[i, j, k, l, m, :] = iJ[i, j, k, l] @ np.array([fg[m], gg[m]])
    u_face = np.zeros((nx, ny, 4, nsp, 4))
    f_face = np.zeros((nx, ny, 4, nsp, 4, 2))
    for i in range(nx):
        for j in range(ny):
            for l in range(nsp):
                for m in range(4):
                    u_face[i, j, 0, l, m] = np.dot(u[i, j, l, :, m], ll)
                    u_face[i, j, 1, l, m] = np.dot(u[i, j, :, l, m], lr)
                    u_face[i, j, 2, l, m] = np.dot(u[i, j, l, :, m], lr)
                    u_face[i, j, 3, l, m] = np.dot(u[i, j, :, l, m], ll)
                    for n in range(2):
                        f_face[i, j, 0, l, m, n] = np.dot(f[i, j, l, :, m, n], ll)
                        f_face[i, j, 1, l, m, n] = np.dot(f[i, j, :, l, m, n], lr)
                        f_face[i, j, 2, l, m, n] = np.dot(f[i, j, l, :, m, n], lr)
                        f_face[i, j, 3, l, m, n] = np.dot(f[i, j, :, l, m, n], ll)
    fx = np.zeros((nx + 1, ny, nsp, 4))
    for i in range(1, nx):
        for j in range(ny):
            for k in range(nsp):
                fx[i, j, k, :] = (0.5 * (f_face[i - 1, j, 1, k, :, 0] + f_face[i, j, 3, k, :, 0])
                                  - c * (u_face[i, j, 3, k, :] - u_face[i - 1, j, 1, k, :]))
    fy = np.zeros((nx, ny + 1, nsp, 4))
    for i in range(nx):
        for j in range(1, ny):
            for k in range(nsp):
                fy[i, j, k, :] = (0.5 * (f_face[i, j - 1, 2, k, :, 1] + f_face[i, j, 0, k, :, 1])
                                  - c * (u_face[i, j, 0, k, :] - u_face[i, j - 1, 2, k, :]))
    for i in range(1, nx - 1):
        for j in range(1, ny - 1):
            for k in range(nsp):
                for l in range(nsp):
                    for m in range(4):
                        rhs1 = np.dot(f[i, j, :, l, m, 0], lpdm[k, :])
                        rhs2 = np.dot(f[i, j, k, :, m, 1], lpdm[l, :])
                        du[i, j, k, l, m] = -(rhs1 + rhs2
                                              + (fx[i, j, l, m] - f_face[i, j, 3, l, m, 0]) * dhl[k]
                                              + (fx[i + 1, j, l, m] - f_face[i, j, 1, l, m, 0]) * dhr[k]
                                              + (fy[i, j, k, m] - f_face[i, j, 0, k, m, 1]) * dhl[l]
                                              + (fy[i, j + 1, k, m] - f_face[i, j, 2, k, m, 1]) * dhr[l])
    return du


def polar_case(frgpu, nr=12, nt=10, deg=2):
    ps = frgpu.FRPSpace2D(0, 1, nr, 0, 1, nt, deg)  # operators only; the geometry comes from V
    V = frgpu.polar_vertices(1.0, 6.0, nr, 0.0, np.pi, nt)
    iJ = frgpu.quad_metric(ps.xpl, V)
    u = initial_state(frgpu.quad_points(ps.xpl, V))
    return ps, V, iJ, u


def test_oracle_central_flux_is_the_script(frgpu, oracle):
    """On the leading (nr-2) x (nt-2) block, with all four sides Dirichlet, the
    oracle's central-flux residual equals the script's dudt! on the whole grid
    (where the last two rows and columns keep du = 0)."""
    ps, V, iJ, u = polar_case(frgpu)
    # a perturbed state, so that every term of the flux is exercised
    rng = np.random.default_rng(3)
    u = u * (1 + 0.05 * rng.standard_normal(u.shape[:4]))[..., None]
    u[..., 1] = 0.1 * u[..., 0] * rng.standard_normal(u.shape[:4])
    u[..., 2] = 0.1 * u[..., 0] * rng.standard_normal(u.shape[:4])
    u[..., 3] += 0.5 * (u[..., 1] ** 2 + u[..., 2] ** 2) / u[..., 0]
    ref = script_dudt(u, iJ, ps.ll, ps.lr, ps.dhl, ps.dhr, ps.dl, C_DISS)
    nr, nt = u.shape[:2]
    ub = np.asfortranarray(u[:nr - 2, :nt - 2])
    psb = frgpu.FRPSpace2D(0, 1, nr - 2, 0, 1, nt - 2, ps.deg)
    po = oracle_space2d(psb, 0, 1, nr - 2, 0, 1, nt - 2, ps.deg)
    P = oracle.Problem(oracle.EULER2D, po, gamma=GAMMA, flux=oracle.FLUX_CENTRAL, bc=oracle.BC_DIRICHLET,
                       flux_c=C_DISS)
    P.set_metric(np.asfortranarray(iJ[:nr - 2, :nt - 2]))
    du = P.rhs(ub)
    scale = np.abs(ref).max()
    assert scale > 1.0
    np.testing.assert_allclose(du, ref[:nr - 2, :nt - 2], rtol=0, atol=1e-12 * scale)
    assert np.all(ref[nr - 2:] == 0) and np.all(ref[:, nt - 2:] == 0)


def test_oracle_central_flux_periodic_keeps_uniform_state(frgpu, oracle):
    """A uniform state on periodic rectangles: every flux difference vanishes."""
    ps = frgpu.FRPSpace2D(0, 1, 6, 0, 1, 5, 3)
    po = oracle_space2d(ps, 0, 1, 6, 0, 1, 5, 3)
    u = np.zeros((6, 5, 4, 4, 4), order="F")
    u[..., 0], u[..., 1], u[..., 2], u[..., 3] = 1.2, 0.3, -0.2, 2.5
    P = oracle.Problem(oracle.EULER2D, po, gamma=1.4, flux=oracle.FLUX_CENTRAL, bc=oracle.BC_PERIODIC, flux_c=0.3)
    iJ = np.zeros((6, 5, 4, 4, 2, 2), order="F")
    iJ[..., 0, 0], iJ[..., 1, 1] = 2 / ps.dx, 2 / ps.dy
    P.set_metric(iJ)
    assert np.abs(P.rhs(u)).max() < 1e-12


# ---------------------------------------------------------------- GPU
def _gpu_problem(frgpu, u, ps, iJ, precision="fp64", bc="dirichlet", gamma=GAMMA, c=C_DISS):
    prob = frgpu.FREuler2DProblem(u, (0, 1), ps, gamma, flux="central", bc=bc, precision=precision)
    prob.set_metric(iJ)
    prob.set_flux_dissipation(c)
    return prob


def _oracle_problem(oracle, ps, iJ, bc=None, gamma=GAMMA, c=C_DISS):
    po = oracle_space2d(ps, 0, 1, ps.nx, 0, 1, ps.ny, ps.deg)
    P = oracle.Problem(oracle.EULER2D, po, gamma=gamma, flux=oracle.FLUX_CENTRAL,
                       bc=oracle.BC_DIRICHLET if bc is None else bc, flux_c=c)
    P.set_metric(iJ)
    return P


@pytest.mark.gpu
@pytest.mark.parametrize("deg", [1, 2, 3])
def test_central_flux_residual_bit_identical(frgpu, oracle, deg):
    """The script's residual on the polar grid, FP64, bit for bit."""
    ps, V, iJ, u = polar_case(frgpu, nr=40, nt=30, deg=deg)
    prob = _gpu_problem(frgpu, u, ps, iJ)
    np.testing.assert_array_equal(prob.rhs(u), _oracle_problem(oracle, ps, iJ).rhs(u))


@pytest.mark.gpu
def test_central_flux_periodic_sides(frgpu, oracle):
    """Periodic sides wrap the neighbours' traces (a sheared periodic metric)."""
    nx, ny, deg = 24, 18, 3
    ps = frgpu.FRPSpace2D(0, 1, nx, 0, 1, ny, deg)
    iJ = np.zeros((nx, ny, deg + 1, deg + 1, 2, 2), order="F")
    iJ[..., 0, 0], iJ[..., 1, 1], iJ[..., 0, 1] = 2 / ps.dx, 2 / ps.dy, 0.3 / ps.dy
    X, Y = ps.xpg[..., 0], ps.xpg[..., 1]
    u = np.zeros(X.shape + (4,), order="F")
    r = 1 + 0.2 * np.sin(2 * np.pi * X) * np.cos(2 * np.pi * Y)
    u[..., 0], u[..., 1], u[..., 2], u[..., 3] = r, 0.5 * r, -0.3 * r, 2.5 + 0.17 * r
    prob = _gpu_problem(frgpu, u, ps, iJ, bc="period", gamma=1.4, c=0.2)
    P = _oracle_problem(oracle, ps, iJ, bc=oracle.BC_PERIODIC, gamma=1.4, c=0.2)
    np.testing.assert_array_equal(prob.rhs(u), P.rhs(u))


@pytest.mark.gpu
def test_curve_euler_midpoint_steps(frgpu, oracle):
    """init(prob, Midpoint(); dt = 0.002) and 50 step!s as the script takes them:
    FP64 bit-identical to the oracle, FP32K close; the fused SSPRK3 step is
    refused for this flux (residual evaluations only)."""
    ps, V, iJ, u = polar_case(frgpu, nr=60, nt=50, deg=2)  # the script's grid
    nr, nt = u.shape[:2]
    ub = np.asfortranarray(u[:nr - 2, :nt - 2])
    psb = frgpu.FRPSpace2D(0, 1, nr - 2, 0, 1, nt - 2, 2)
    iJb = np.asfortranarray(iJ[:nr - 2, :nt - 2])
    mid = frgpu.Midpoint()
    itg = frgpu.init(_gpu_problem(frgpu, ub, psb, iJb), mid, dt=0.002)
    itg.step(50)
    P = _oracle_problem(oracle, psb, iJb)
    ref = P.erk(ub, 0.002, 50, mid.A, mid.b)
    np.testing.assert_array_equal(itg.u, ref)
    it32 = frgpu.init(_gpu_problem(frgpu, ub, psb, iJb, precision="fp32k"), mid, dt=0.002)
    it32.step(50)
    assert np.abs(it32.u - ref).max() < 1e-5 * np.abs(ref).max()
    with pytest.raises(frgpu.FRGPUError):
        frgpu.init(_gpu_problem(frgpu, ub, psb, iJb), dt=0.002).step(1)
