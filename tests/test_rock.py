"""Stabilised explicit steps (the recurrence + finishing structure of
OrdinaryDiffEq's ROCK4, example/advection_kinetic.jl:133-146) on the CPU: the
built-in RKC2 coefficients, the oracle's stabilised step and its
spectral-radius estimate (the nonlinear power method the ROCK methods take
before every step)."""
import numpy as np
import pytest
from numpy.polynomial import polynomial as P

from test_parity_gpu import oracle_space1d

RK4_A = np.array([[0, 0, 0, 0], [0.5, 0, 0, 0], [0, 0.5, 0, 0], [0, 0, 1, 0]], dtype=float)
RK4_B = np.array([1 / 6, 1 / 3, 1 / 3, 1 / 6])


def stability_function(alpha, beta, mu, delta, z):
    """R(z) on an array of z, by running the recurrence (stable for any s)."""
    d2, d1 = np.zeros_like(z), np.zeros_like(z)
    for j in range(1, len(alpha) + 1):
        t = z * (mu[j - 1] * (1 + d1) + delta[j - 1])
        if j >= 3:
            t = t + beta[j - 1] * d2
        if j >= 2:
            t = t + alpha[j - 1] * d1
        d2, d1 = d1, t
    return 1 + d1


def stability_polynomial(alpha, beta, mu, delta):
    """R(z) of the increment-form recurrence on y' = lambda y (z = dt lambda)."""
    D = [np.zeros(1), np.zeros(1)]  # D_{-1}, D_0
    for j in range(1, len(alpha) + 1):
        t = P.polymul([0, 1], P.polyadd(mu[j - 1] * P.polyadd([1], D[-1]), [delta[j - 1]]))
        if j >= 3:
            t = P.polyadd(t, beta[j - 1] * D[-2])
        if j >= 2:
            t = P.polyadd(t, alpha[j - 1] * D[-1])
        D.append(t)
    return P.polyadd([1], D[-1])


@pytest.mark.parametrize("s", [2, 3, 5, 10, 40])
def test_rkc2_is_second_order_and_stable_to_its_bound(frgpu, s):
    """R_s(z) = 1 + z + z^2/2 + O(z^3), |R_s| <= 1 on [-beta(s), 0], and the
    bound is close to (2/3)(s^2 - 1)(1 - 2 eps/15) (damping eps = 2/13)."""
    al, be, mu, de, bound = frgpu.rkc2_coefficients(s)
    R = stability_polynomial(al, be, mu, de)
    assert len(R) == s + 1
    np.testing.assert_allclose(R[:3], [1.0, 1.0, 0.5], rtol=0, atol=1e-12)
    z = np.linspace(-bound, 0.0, 20001)
    assert np.abs(stability_function(al, be, mu, de, z)).max() <= 1.0 + 1e-9
    assert abs(bound / (2 / 3 * (s * s - 1) * (1 - 2 * (2 / 13) / 15)) - 1) < 0.02


def test_rkc2_and_rock_adapters(frgpu):
    """RKC2 takes the fewest stages whose bound covers dt * rho; ROCK maps the
    caller's (mu, kappa) tables to alpha = 1 + kappa, beta = -kappa."""
    alg = frgpu.RKC2()
    for z in (0.5, 3.0, 50.0, 1000.0):
        al, be, mu, de, A, b = alg.coefficients(z)
        s = len(al)
        assert frgpu.rkc2_coefficients(s)[4] >= z
        assert s == 2 or frgpu.rkc2_coefficients(s - 1)[4] < z or s > 10
        assert A is None and b is None
    mu = np.array([0.3, 0.2, 0.1])
    kappa = np.array([9.0, 0.5, 0.25])
    rock = frgpu.ROCK(lambda z: (mu, kappa, RK4_A, RK4_B))
    al, be, m2, de, A, b = rock.coefficients(1.0)
    np.testing.assert_array_equal(al, [0.0, 1.5, 1.25])
    np.testing.assert_array_equal(be, [0.0, -0.5, -0.25])
    np.testing.assert_array_equal(m2, mu)
    np.testing.assert_array_equal(de, 0.0)


@pytest.mark.parametrize("eps", [2 / 13, 0.0, 0.05])
def test_library_rkc2_coefficients_equal_the_restatement(frgpu, eps):
    """frgpu_rkc2_coefficients (host C++, used by frgpu_step_rkc2) gives the
    bits of the numpy restatement rkc2_coefficients: the same operations in the
    same order."""
    import ctypes as C

    from frgpu import _lib as L

    for s in (2, 3, 4, 7, 16, 100, 1000):
        out = [np.zeros(s) for _ in range(4)]
        bound = C.c_double()
        L.check(L.lib().frgpu_rkc2_coefficients(s, eps, *(x.ctypes.data_as(C.POINTER(C.c_double)) for x in out),
                                                C.byref(bound)))
        ref = frgpu.rkc2_coefficients(s, eps)
        for a, b in zip(out, ref[:4]):
            assert np.array_equal(a, b), s
        assert bound.value == ref[4], s
    assert L.lib().frgpu_rkc2_coefficients(1, eps, None, None, None, None, None) != 0


def _advection(frgpu, oracle, ne=16, deg=2):
    ps = frgpu.FRPSpace1D(0, 1, ne, deg)
    po = oracle_space1d(ps, 0, 1, ne, deg)
    Pr = oracle.Problem(oracle.ADVECTION, po, a=1.0)
    u = np.asfortranarray(np.sin(2 * np.pi * ps.xpg))
    return ps, Pr, u


def test_oracle_rock_reduces_to_rk4_and_converges(frgpu, oracle):
    """One recurrence stage with zero coefficients plus the RK4 tableau as the
    finishing procedure is RK4; RKC2 (5 stages) converges at second order."""
    ps, Pr, u = _advection(frgpu, oracle)
    r1 = Pr.rock(u, 1e-3, 10, [0.0], [0.0], [0.0], [0.0], RK4_A, RK4_B)
    r2 = Pr.erk(u, 1e-3, 10, RK4_A, RK4_B)
    assert np.abs(r1 - r2).max() < 1e-14
    ref = Pr.erk(u, 1e-4, 5000, RK4_A, RK4_B)
    al, be, mu, de, _ = frgpu.rkc2_coefficients(5)
    err = [np.abs(Pr.rock(u, dt, int(round(0.5 / dt)), al, be, mu, de) - ref).max() for dt in (4e-3, 2e-3, 1e-3)]
    for a, b in zip(err, err[1:]):
        assert 3.6 < a / b < 4.4


def test_oracle_spectral_radius_against_dense_eigenvalues(frgpu, oracle):
    """The power-method estimate of the FR advection operator's spectral radius
    lies within a few percent of the largest |eigenvalue| of the assembled
    Jacobian; a warm start from the returned direction settles in <= 3
    iterations."""
    ps, Pr, u = _advection(frgpu, oracle)
    n = u.size
    J = np.zeros((n, n))
    for i in range(n):
        e = np.zeros(n)
        e[i] = 1.0
        J[:, i] = Pr.rhs(e.reshape(u.shape, order="F")).ravel(order="F")
    lam = np.abs(np.linalg.eigvals(J)).max()
    rho, it, d = Pr.spectral_radius(u, 50)
    assert it > 0
    assert 0.95 < rho / 1.2 / lam < 1.01
    rho2, it2, _ = Pr.spectral_radius(u, 50, d)
    assert 0 < it2 <= 3
    assert abs(rho2 / rho - 1) < 0.02
