"""Error norms of src/tools.jl:43-53 and the accuracy helpers the bench uses
(quadrature-weighted L2, a 2x-refined solution evaluated at the coarse
solution points).  Host code only."""
import numpy as np
import pytest


def test_reference_norms_known_values():
    from frgpu import api

    u = np.array([1.0, 2.0, 3.0])
    ue = np.array([1.5, 2.0, 2.0])
    # tools.jl: L1 = sum(|u - ue| dx), L2 = sqrt(sum((|u - ue| dx)^2)), Linf = max(|u - ue| dx)
    assert api.L1_error(u, ue, 0.1) == pytest.approx(0.15, rel=1e-15)
    assert api.L2_error(u, ue, 0.1) == pytest.approx(np.sqrt(0.05 ** 2 + 0.1 ** 2), rel=1e-15)
    assert api.Linf_error(u, ue, 0.1) == pytest.approx(0.1, rel=1e-15)
    # the call of test/runtests.jl:6-10 (random vectors of 3, dx = 0.1): all
    # three are finite and ordered Linf <= L2 <= L1
    rng = np.random.default_rng(3)
    a, b = rng.random(3), rng.random(3)
    l1, l2, li = api.L1_error(a, b, 0.1), api.L2_error(a, b, 0.1), api.Linf_error(a, b, 0.1)
    assert 0 <= li <= l2 <= l1


def test_reference_norms_match_oracle(oracle):
    from frgpu import api

    rng = np.random.default_rng(11)
    u, ue = rng.standard_normal(1000), rng.standard_normal(1000)
    for dx in (0.1, 1.0 / 512):
        assert api.L1_error(u, ue, dx) == pytest.approx(oracle.l1_error(u, ue, dx), rel=1e-13)
        assert api.L2_error(u, ue, dx) == pytest.approx(oracle.l2_error(u, ue, dx), rel=1e-13)
        assert api.Linf_error(u, ue, dx) == pytest.approx(oracle.linf_error(u, ue, dx), rel=1e-15)


def _points(nx, ny, x1, y1, xpl):
    dx, dy = x1 / nx, y1 / ny
    xc = (np.arange(nx) + 0.5) * dx
    yc = (np.arange(ny) + 0.5) * dy
    X = xc[:, None, None, None] + 0.5 * dx * xpl[None, None, :, None]
    Y = yc[None, :, None, None] + 0.5 * dy * xpl[None, None, None, :]
    X, Y = np.broadcast_arrays(X, Y)
    return X, Y


@pytest.mark.parametrize("deg", [1, 3, 5])
def test_refined_at_coarse_points_is_exact_for_polynomials(deg):
    from frgpu import api

    xpl, w1 = np.polynomial.legendre.leggauss(deg + 1)
    nx, ny = 6, 4

    def field(X, Y):
        # degree deg in x and in y: the fine elements' interpolants are exact
        return np.stack([(1 + X) ** deg * (2 - Y) ** deg, X ** deg + Y, (X * Y) ** deg], axis=-1)

    Xf, Yf = _points(2 * nx, 2 * ny, 2.0, 1.0, xpl)
    Xc, Yc = _points(nx, ny, 2.0, 1.0, xpl)
    uf = np.asfortranarray(field(Xf, Yf))
    uc = api.refined_at_coarse_points(uf, xpl)
    np.testing.assert_allclose(uc, field(Xc, Yc), rtol=0, atol=1e-12 * np.abs(field(Xc, Yc)).max())


def test_quadrature_l2_error():
    from frgpu import api

    xpl, w1 = np.polynomial.legendre.leggauss(4)
    nx, ny = 8, 5
    X, Y = _points(nx, ny, 2.0, 1.0, xpl)
    e = np.ones(X.shape)
    # |1| over [0,2] x [0,1]: sqrt(area)
    assert api.quadrature_L2_error(e, 0 * e, 2.0 / nx, 1.0 / ny, w1) == pytest.approx(np.sqrt(2.0), rel=1e-14)
    # sin(pi x) over [0,2] x [0,1]: sqrt(1) (p = 3 Gauss is near exact on 8 elements)
    s = np.sin(np.pi * X)
    assert api.quadrature_L2_error(s, 0 * s, 2.0 / nx, 1.0 / ny, w1) == pytest.approx(1.0, rel=1e-6)
