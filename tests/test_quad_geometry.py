"""Geometry of general quadrilaterals in the host mirror: the per-point
Jacobian of FRPSpace2D (rs_jacobi, src/Geometry/geo_jacobi.jl:77-108;
src/struct.jl:135-143) and the face normals of dev/parallelogram.jl, as
frgpu_problem_set_metric takes them.  CPU only."""
import numpy as np
import pytest


def _vertices(nx, ny, mapping):
    """vertices[nx, ny, 4, 2] of the cells of the unit square under `mapping`,
    counterclockwise from the lower left."""
    X = np.linspace(0, 1, nx + 1)
    Y = np.linspace(0, 1, ny + 1)
    V = np.zeros((nx, ny, 4, 2))
    for a, (di, dj) in enumerate(((0, 0), (1, 0), (1, 1), (0, 1))):
        xx, yy = np.meshgrid(X[di:nx + di], Y[dj:ny + dj], indexing="ij")
        V[:, :, a, 0], V[:, :, a, 1] = mapping(xx, yy)
    return V


def test_rectangles_give_the_diagonal_metric(frgpu):
    nx, ny, deg = 5, 4, 3
    V = _vertices(nx, ny, lambda x, y: (2 * x, 3 * y))
    iJ = frgpu.quad_metric(frgpu.legendre_point(deg), V)
    assert iJ.shape == (nx, ny, deg + 1, deg + 1, 2, 2)
    np.testing.assert_allclose(iJ[..., 0, 0], 2 / (2 / nx), rtol=1e-14)
    np.testing.assert_allclose(iJ[..., 1, 1], 2 / (3 / ny), rtol=1e-14)
    assert np.max(np.abs(iJ[..., 0, 1])) < 1e-12 and np.max(np.abs(iJ[..., 1, 0])) < 1e-12
    n1, n2 = frgpu.quad_face_normals(V)
    assert n1.shape == (nx + 1, ny, 2) and n2.shape == (nx, ny + 1, 2)
    np.testing.assert_allclose(n1, np.broadcast_to([1.0, 0.0], n1.shape), atol=1e-15)
    np.testing.assert_allclose(n2, np.broadcast_to([0.0, 1.0], n2.shape), atol=1e-15)


def test_affine_mesh_metric_normals_and_free_stream(frgpu, oracle):
    """x = X + s Y, y = Y + t X: constant J = [[dx/2, s dy/2], [t dx/2, dy/2]],
    normals along (1, -s) and (-t, 1); with both, the oracle's residual keeps a
    uniform flow (dev/parallelogram.jl's formulation)."""
    s, t = 0.3, -0.2
    nx, ny, deg = 5, 4, 3
    V = _vertices(nx, ny, lambda x, y: (x + s * y, y + t * x))
    r = frgpu.legendre_point(deg)
    J = frgpu.rs_jacobi_quad(r, V)
    want = np.array([[0.5 / nx, s * 0.5 / ny], [t * 0.5 / nx, 0.5 / ny]])
    np.testing.assert_allclose(J, np.broadcast_to(want, J.shape), atol=1e-15)
    n1, n2 = frgpu.quad_face_normals(V)
    np.testing.assert_allclose(n1, np.broadcast_to(np.array([1.0, -s]) / np.hypot(1, s), n1.shape), atol=1e-15)
    np.testing.assert_allclose(n2, np.broadcast_to(np.array([-t, 1.0]) / np.hypot(1, t), n2.shape), atol=1e-15)
    O = oracle
    sp = O.Space2D(0, 1, nx, 0, 1, ny, deg)
    pr = O.Problem(O.EULER2D, sp, gamma=1.4, flux=O.FLUX_HLL)
    u = np.zeros((nx, ny, deg + 1, deg + 1, 4), order="F")
    u[..., 0], u[..., 1], u[..., 2], u[..., 3] = 1.2, 0.3, -0.2, 2.9
    pr.set_metric(frgpu.quad_metric(r, V), n1, n2)
    assert np.max(np.abs(pr.rhs(u))) < 1e-12


@pytest.mark.parametrize("deg", [1, 3])
def test_bilinear_jacobian_matches_finite_differences(frgpu, deg):
    """A non-affine quadrilateral: J varies from point to point and equals the
    derivative of the bilinear map X(r, s) = sum_a lambda_a V_a."""
    V = np.array([[[[0.0, 0.0], [1.0, 0.1], [1.3, 1.2], [-0.1, 0.9]]]])
    r = frgpu.legendre_point(deg)
    J = frgpu.rs_jacobi_quad(r, V)[0, 0]

    def X(rr, ss):
        lam = [(rr - 1) * (ss - 1) / 4, (rr + 1) * (1 - ss) / 4, (rr + 1) * (ss + 1) / 4, (1 - rr) * (ss + 1) / 4]
        return sum(lam[a] * V[0, 0, a] for a in range(4))

    h = 1e-6
    for k, rk in enumerate(r):
        for l, sl in enumerate(r):
            dr = (X(rk + h, sl) - X(rk - h, sl)) / (2 * h)
            ds = (X(rk, sl + h) - X(rk, sl - h)) / (2 * h)
            np.testing.assert_allclose(J[k, l], np.stack([dr, ds], axis=-1), atol=1e-9)
    assert np.ptp(J[..., 0, 0]) > 1e-3   # not constant


def test_face_jacobians_follow_the_reference_construction(frgpu, oracle):
    """FRPSpace2D's Ji (src/struct.jl:145-158): on a parallelogram mesh every
    face Jacobian is the constant J, and the oracle's residual with the
    face-Jacobian scaling of dev/cylinder2.jl:147-150 keeps a uniform flow; on a
    bilinear cell the four face matrices are rs_jacobi at (r_1, 0), (1, r_1),
    (r_np, 1) and (0, r_np), the points the reference's linear indexing of
    ri, si selects, the same for every point of a face."""
    s, t = 0.3, -0.2
    nx, ny, deg = 5, 4, 3
    V = _vertices(nx, ny, lambda x, y: (x + s * y, y + t * x))
    r = frgpu.legendre_point(deg)
    Ji = frgpu.quad_face_jacobians(r, V)
    assert Ji.shape == (nx, ny, 4, deg + 1, 2, 2)
    want = np.array([[0.5 / nx, s * 0.5 / ny], [t * 0.5 / nx, 0.5 / ny]])
    np.testing.assert_allclose(Ji, np.broadcast_to(want, Ji.shape), atol=1e-15)
    O = oracle
    sp = O.Space2D(0, 1, nx, 0, 1, ny, deg)
    pr = O.Problem(O.EULER2D, sp, gamma=1.4, flux=O.FLUX_HLL)
    u = np.zeros((nx, ny, deg + 1, deg + 1, 4), order="F")
    u[..., 0], u[..., 1], u[..., 2], u[..., 3] = 1.2, 0.3, -0.2, 2.9
    n1, n2 = frgpu.quad_face_normals(V)
    pr.set_metric(frgpu.quad_metric(r, V), n1, n2, Ji)
    assert np.max(np.abs(pr.rhs(u))) < 1e-12
    # a bilinear cell: the evaluation points of the reference
    B = np.array([[[[0.0, 0.0], [1.0, 0.1], [1.3, 1.2], [-0.1, 0.9]]]])
    Jb = frgpu.quad_face_jacobians(r, B)[0, 0]

    def J_at(rr, ss):
        v = B[0, 0]
        xr = (ss - 1) * v[0] / 4 + (1 - ss) * v[1] / 4 + (ss + 1) * v[2] / 4 - (ss + 1) * v[3] / 4
        xs = (rr - 1) * v[0] / 4 - (rr + 1) * v[1] / 4 + (rr + 1) * v[2] / 4 + (1 - rr) * v[3] / 4
        return np.stack([xr, xs], axis=-1)

    for f, (rr, ss) in enumerate([(r[0], 0.0), (1.0, r[0]), (r[-1], 1.0), (0.0, r[-1])]):
        for k in range(deg + 1):
            np.testing.assert_allclose(Jb[f, k], J_at(rr, ss), atol=1e-15)
