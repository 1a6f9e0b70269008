"""example/shock-vortex.jl's dudt! (lines 26-118) and its ghost handling.

The script's state carries a ghost layer (OffsetArray 0:nx+1, 0:ny+1); dudt!
computes fluxes and face traces on every element, ghosts included, and writes
du on the interior only, so the ghosts keep their values through a step; after
the step the script copies the copy-boundary ghosts from the adjacent interior
(lines 323-330) and never touches the fixed inflow ghost on the left.

CPU: SSPRK3 steps of a literal numpy transcription of that dudt! on the
ghost-extended array, with the script's boundary copies after each step,
against the oracle with ghosts refreshed once per step (FRO_FLUX_HLL, fixed left
side, copy elsewhere): equal to rounding.  The per-stage form (ghosts following
every stage input) differs at the boundaries.
GPU (marked): FRGPU_OPT_GHOSTS_PER_STEP bit-identical to the oracle, FP64, for
SSPRK3 and Midpoint (the script's integrator), and FP32K close."""
import numpy as np
import pytest

from test_parity_gpu import oracle_space2d

G = 1.4
LEFT = np.array([1.3, 0.4, 0.0, 3.2])  # fixed inflow state (conserved)


def euler_fluxes(w):
    rho, mx, my, E = w
    U, V = mx / rho, my / rho
    p = (G - 1) * (E - 0.5 * (mx * U + my * V))
    return np.array([mx, mx * U + p, my * U, (E + p) * U]), np.array([my, mx * V, my * V + p, (E + p) * V])


def hll_x(wL, wR):
    """HLL with Davis wave speeds in x (the restatement of KitBase.flux_hll!)."""
    def parts(w):
        rho, mx, my, E = w
        U, V = mx / rho, my / rho
        p = (G - 1) * (E - 0.5 * (mx * U + my * V))
        return euler_fluxes(w)[0], U, np.sqrt(G * p / rho)

    fL, uL, cL = parts(wL)
    fR, uR, cR = parts(wR)
    sl, sr = min(uL - cL, uR - cR), max(uL + cL, uR + cR)
    if sl >= 0:
        return fL
    if sr <= 0:
        return fR
    return (sr * fL - sl * fR + sl * sr * (wR - wL)) / (sr - sl)


def local_frame(w, c, s):
    return np.array([w[0], w[1] * c + w[2] * s, w[2] * c - w[1] * s, w[3]])


def global_frame(w, c, s):
    return np.array([w[0], w[1] * c - w[2] * s, w[1] * s + w[2] * c, w[3]])


def script_dudt(ug, iJx, iJy, ll, lr, dhl, dhr, lpdm):
    """The dudt! of example/shock-vortex.jl on the ghost-extended state
    ug[0:nx+2, 0:ny+2, np, np, 4]; iJ = diag(iJx, iJy) on the rectangles."""
    nx, ny, nsp = ug.shape[0] - 2, ug.shape[1] - 2, ug.shape[2]
    du = np.zeros_like(ug)
    f = np.zeros(ug.shape + (2,))
    for i in range(nx + 2):
        for j in range(ny + 2):
            for k in range(nsp):
                for l in range(nsp):
                    fg, gg = euler_fluxes(ug[i, j, k, l, :])
                    f[i, j, k, l, :, 0] = iJx * fg
                    f[i, j, k, l, :, 1] = iJy * gg
    u_face = np.zeros((nx + 2, ny + 2, 4, nsp, 4))
    f_face = np.zeros((nx + 2, ny + 2, 4, nsp, 4, 2))
    for i in range(nx + 2):
        for j in range(ny + 2):
            for l in range(nsp):
                for m in range(4):
                    u_face[i, j, 0, l, m] = np.dot(ug[i, j, l, :, m], ll)
                    u_face[i, j, 1, l, m] = np.dot(ug[i, j, :, l, m], lr)
                    u_face[i, j, 2, l, m] = np.dot(ug[i, j, l, :, m], lr)
                    u_face[i, j, 3, l, m] = np.dot(ug[i, j, :, l, m], ll)
                    for n in range(2):
                        f_face[i, j, 0, l, m, n] = np.dot(f[i, j, l, :, m, n], ll)
                        f_face[i, j, 1, l, m, n] = np.dot(f[i, j, :, l, m, n], lr)
                        f_face[i, j, 2, l, m, n] = np.dot(f[i, j, l, :, m, n], lr)
                        f_face[i, j, 3, l, m, n] = np.dot(f[i, j, :, l, m, n], ll)
    fx = np.zeros((nx + 2, ny + 2, nsp, 4))
    for k in range(nsp):
        for j in range(1, ny + 1):
            for i in range(1, nx + 2):
                fx[i, j, k, :] = hll_x(u_face[i - 1, j, 1, k, :], u_face[i, j, 3, k, :])
    fy = np.zeros((nx + 2, ny + 2, nsp, 4))
    for k in range(nsp):
        for j in range(1, ny + 2):
            for i in range(1, nx + 1):
                uL = local_frame(u_face[i, j - 1, 2, k, :], 0.0, 1.0)
                uR = local_frame(u_face[i, j, 0, k, :], 0.0, 1.0)
                fy[i, j, k, :] = global_frame(hll_x(uL, uR), 0.0, 1.0)
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            for k in range(nsp):
                for l in range(nsp):
                    for m in range(4):
                        rhs1 = np.dot(f[i, j, :, l, m, 0], lpdm[k, :])
                        rhs2 = np.dot(f[i, j, k, :, m, 1], lpdm[l, :])
                        du[i, j, k, l, m] = -(rhs1 + rhs2
                                              + (fx[i, j, l, m] * iJx - f_face[i, j, 3, l, m, 0]) * dhl[k]
                                              + (fx[i + 1, j, l, m] * iJx - f_face[i, j, 1, l, m, 0]) * dhr[k]
                                              + (fy[i, j, k, m] * iJy - f_face[i, j, 0, k, m, 1]) * dhl[l]
                                              + (fy[i, j + 1, k, m] * iJy - f_face[i, j, 2, k, m, 1]) * dhr[l])
    return du


def script_boundary(ug):
    """example/shock-vortex.jl:323-326 (the left ghost column keeps the inflow)."""
    ny, nx = ug.shape[1] - 2, ug.shape[0] - 2
    ug[:, 0] = ug[:, 1]
    ug[:, ny + 1] = ug[:, ny]
    ug[nx + 1, :] = ug[nx, :]


def with_ghosts(u):
    nx, ny = u.shape[:2]
    ug = np.zeros((nx + 2, ny + 2) + u.shape[2:])
    ug[1:-1, 1:-1] = u
    ug[0, :] = LEFT
    script_boundary(ug)
    return ug


def case(frgpu, nx=7, ny=5, deg=2, seed=1):
    ps = frgpu.FRPSpace2D(0, 2, nx, 0, 1, ny, deg)
    rng = np.random.default_rng(seed)
    X, Y = ps.xpg[..., 0], ps.xpg[..., 1]
    u = np.zeros(X.shape + (4,), order="F")
    rho = 1 + 0.2 * np.sin(3 * X + 1) * np.cos(2 * Y) + 0.02 * rng.standard_normal(X.shape)
    U = 0.3 + 0.1 * np.cos(X) + 0.02 * rng.standard_normal(X.shape)
    V = 0.1 * np.sin(4 * Y) + 0.02 * rng.standard_normal(X.shape)
    p = 1 + 0.1 * np.sin(X + Y)
    u[..., 0], u[..., 1], u[..., 2] = rho, rho * U, rho * V
    u[..., 3] = p / (G - 1) + 0.5 * rho * (U * U + V * V)
    return ps, u


def oracle_problem(oracle, ps, lag):
    po = oracle_space2d(ps, 0, 2, ps.nx, 0, 1, ps.ny, ps.deg)
    return oracle.Problem(oracle.EULER2D, po, gamma=G, flux=oracle.FLUX_HLL,
                          bcs=[oracle.BC_FIXED, oracle.BC_COPY, oracle.BC_COPY, oracle.BC_COPY],
                          fixed_states=[LEFT, LEFT, LEFT, LEFT], ghosts_per_step=lag)


@pytest.mark.parametrize("deg", [2, 3])
def test_oracle_steps_are_the_script(frgpu, oracle, deg):
    """Three SSPRK3 steps of the transcribed dudt! with the script's ghost
    handling equal the oracle's with ghosts refreshed once per step."""
    ps, u = case(frgpu, deg=deg)
    dt, nsteps = 2e-3, 3
    iJx, iJy = 2 / ps.dx, 2 / ps.dy
    args = (iJx, iJy, ps.ll, ps.lr, ps.dhl, ps.dhr, ps.dl)
    ug = with_ghosts(u)
    for _ in range(nsteps):
        u1 = ug + dt * script_dudt(ug, *args)
        u2 = 0.75 * ug + 0.25 * (u1 + dt * script_dudt(u1, *args))
        ug = ug / 3 + 2 / 3 * (u2 + dt * script_dudt(u2, *args))
        script_boundary(ug)
    ref = ug[1:-1, 1:-1]
    lagged = oracle_problem(oracle, ps, 1).ssprk3(u, dt, nsteps)
    scale = np.abs(ref).max()
    np.testing.assert_allclose(lagged, ref, rtol=0, atol=1e-12 * scale)
    per_stage = oracle_problem(oracle, ps, 0).ssprk3(u, dt, nsteps)
    assert np.abs(per_stage - ref).max() > 1e-9 * scale  # the ghosts' timing shows at the boundaries
    # the residual itself (no step start) is the same either way
    np.testing.assert_allclose(oracle_problem(oracle, ps, 1).rhs(u), script_dudt(with_ghosts(u), *args)[1:-1, 1:-1],
                               rtol=0, atol=1e-12 * np.abs(script_dudt(with_ghosts(u), *args)).max())


# ---------------------------------------------------------------- GPU
def gpu_problem(frgpu, u, ps, precision="fp64"):
    from frgpu import _lib as L

    prob = frgpu.FREuler2DProblem(u, (0, 1), ps, G, flux="hll", bc=("fix", "copy", "copy", "copy"),
                                  fixed_states=[LEFT, LEFT, LEFT, LEFT], precision=precision)
    prob.set_option(L.OPT_GHOSTS_PER_STEP, 1)
    return prob


@pytest.mark.gpu
@pytest.mark.parametrize("deg", [2, 3, 4])
def test_ghosts_per_step_bit_identical(frgpu, oracle, deg):
    ps, u = case(frgpu, nx=40, ny=23, deg=deg)
    dt = 1e-3
    itg = frgpu.init(gpu_problem(frgpu, u, ps), dt=dt)
    itg.step(6)
    ref = oracle_problem(oracle, ps, 1).ssprk3(u, dt, 6)
    np.testing.assert_array_equal(itg.u, ref)
    mid = frgpu.Midpoint()
    itm = frgpu.init(gpu_problem(frgpu, u, ps), mid, dt=dt)
    itm.step(6)
    refm = oracle_problem(oracle, ps, 1).erk(u, dt, 6, mid.A, mid.b)
    assert np.abs(itm.u - refm).max() <= 1e-12 * np.abs(refm).max()
    it32 = frgpu.init(gpu_problem(frgpu, u, ps, "fp32k"), dt=dt)
    it32.step(6)
    assert np.abs(it32.u - ref).max() < 2e-6 * np.abs(ref).max()


@pytest.mark.gpu
def test_ghosts_per_step_in_every_stepper(frgpu, oracle):
    """The generic explicit step (RK4) and a stabilised step keep the ghosts at
    the step's start as well: FP64 bit-identical to the oracle's fro_erk /
    fro_rock with ghosts refreshed once per step; per-stage ghosts differ."""
    ps, u = case(frgpu, nx=32, ny=18, deg=3)
    dt = 1e-3
    rk4 = frgpu.RK4()
    it = frgpu.init(gpu_problem(frgpu, u, ps), rk4, dt=dt)
    it.step(4)
    ref = oracle_problem(oracle, ps, 1).erk(u, dt, 4, rk4.A, rk4.b)
    np.testing.assert_array_equal(it.u, ref)
    assert np.abs(oracle_problem(oracle, ps, 0).erk(u, dt, 4, rk4.A, rk4.b) - ref).max() > 0
    al, be, mu, de, _ = frgpu.rkc2_coefficients(5)
    A = np.array([[0, 0], [0.5, 0]], dtype=float)
    b = np.array([0.0, 1.0])
    itr = frgpu.init(gpu_problem(frgpu, u, ps), dt=dt)
    itr.step_rock(al, be, mu, de, A, b, n=3)
    np.testing.assert_array_equal(itr.u, oracle_problem(oracle, ps, 1).rock(u, dt, 3, al, be, mu, de, A, b))
