"""Unstructured triangles: TriFRPSpace (src/struct.jl:305-352) and the
linear-advection dudt! of dev/wave_triangle.jl:44-125.

CPU: the golden tri_quadrature points (made from the reference's own qpmin.py
by tests/golden/make_tri_quadrature.py) and the library's tri_quadrature
against them, libfrgpu's host operators against the
oracle's restatement, exactness of the operators, the mesh connectivity
against the reference's coordinate matching (neighbour_fpidx), and the
oracle's residual (uniform state kept, conservation, convergence order).
GPU (marked): the residual and explicit Runge-Kutta steps through the C ABI
against the oracle."""
import ctypes as C
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "tri_quadrature.npz")


@pytest.fixture(scope="module")
def quad():
    return np.load(GOLD)


def _xpl(quad, deg):
    return np.stack([quad[f"r{deg}"], quad[f"s{deg}"]], axis=1), quad[f"w{deg}"]


def _space(frgpu, quad, nx, ny, deg, periodic=True):
    pts, cid, key, ct = frgpu.tri_square_mesh(nx, ny, periodic=periodic)
    xpl, wp = _xpl(quad, deg)
    return frgpu.TriFRPSpace(pts, cid, deg, xpl, wp, key, ct)


def _oracle_problem(oracle, sp, a):
    return oracle.TriProblem(sp.deg, a, sp.dl, sp.lf, sp.phi, sp.J, sp.iJ, sp.nb_cell, sp.nb_face, sp.nb_point,
                             sp.cell_type)


def _wave(sp):
    X, Y = sp.xpg[..., 0], sp.xpg[..., 1]
    return np.asfortranarray(1.0 + 0.5 * np.sin(2 * np.pi * X) * np.cos(2 * np.pi * Y))


# ---------------------------------------------------------------- CPU
@pytest.mark.parametrize("deg", [1, 2, 3])
def test_library_tri_quadrature_is_the_golden_rule(frgpu, quad, deg):
    """frgpu.tri_quadrature(deg), the library's Williams-Shunn-Jameson table
    expanded by its own symmetry code and mapped by trilinear -> Cartesian ->
    xy_rs, reproduces the reference's qpmin.py points and weights bit for bit,
    in the same order; TriFRPSpace takes it by default."""
    xpl, w = _xpl(quad, deg)
    p, wl = frgpu.tri_quadrature(deg)
    np.testing.assert_array_equal(p, xpl)
    np.testing.assert_array_equal(wl, w)
    pts, cid, key, ct = frgpu.tri_square_mesh(3, 3, periodic=True)
    np.testing.assert_array_equal(frgpu.TriFRPSpace(pts, cid, deg, key=key, cell_type=ct).xpl, xpl)


def test_tri_quadrature_vertices_and_degrees(frgpu):
    """Other vertices: the points land inside that triangle with the same
    barycentric weights (transform=False keeps x, y); degrees the triangle
    kernel has no instance for are refused."""
    v = ((0.0, 0.0), (3.0, 0.0), (1.0, 2.0))
    p, w = frgpu.tri_quadrature(3, vertices=v, transform=False)
    A = np.array([[v[1][0] - v[0][0], v[2][0] - v[0][0]], [v[1][1] - v[0][1], v[2][1] - v[0][1]]])
    lam = np.linalg.solve(A, (p - np.asarray(v[0])).T).T
    assert np.all(lam > 0) and np.all(lam.sum(axis=1) < 1)
    assert abs(w.sum() - 1) < 1e-15
    # on the default equilateral triangle the trilinear map is the barycentric one
    pe, _ = frgpu.tri_quadrature(3, transform=False)
    r, s = frgpu.xy_rs(pe[:, 0], pe[:, 1])
    np.testing.assert_array_equal(np.stack([r, s], axis=1), frgpu.tri_quadrature(3)[0])
    for bad in (0, 4):
        with pytest.raises(ValueError):
            frgpu.tri_quadrature(bad)


@pytest.mark.parametrize("deg", [1, 2, 3])
def test_tri_quadrature_golden(quad, deg):
    """The Williams-Shunn-Jameson points of tri_quadrature(deg): (deg+1)(deg+2)/2
    points inside the reference right triangle, weights summing to 1, exact
    for the monomials r^i s^j, i + j <= deg + 1 (the rules' degree)."""
    xpl, w = _xpl(quad, deg)
    r, s = xpl[:, 0], xpl[:, 1]
    assert len(w) == (deg + 1) * (deg + 2) // 2
    assert np.all(r > -1) and np.all(s > -1) and np.all(r + s < 0)
    assert abs(w.sum() - 1) < 1e-14
    # exact integrals over the right triangle of area 2, by 1D Gauss-Jacobi in a
    # collapsed coordinate (numpy Gauss-Legendre of high order on the square map)
    x, wx = np.polynomial.legendre.leggauss(12)
    A, B = np.meshgrid(x, x, indexing="ij")
    WA = np.outer(wx, wx)
    R = (1 + A) * (1 - B) / 2 - 1
    S = B
    jac = (1 - B) / 2
    for i in range(deg + 2):
        for j in range(deg + 2 - i):
            exact = np.sum(WA * jac * R ** i * S ** j)
            assert abs(2 * np.dot(w, r ** i * s ** j) - exact) < 1e-13, (i, j)


@pytest.mark.parametrize("deg", [1, 2, 3])
def test_tri_operators_match_oracle(frgpu, oracle, quad, deg):
    """libfrgpu's host setup (frgpu_vandermonde_tri, frgpu_tri_operators: long
    double Jacobi recurrences) against the oracle's C restatement of
    transform_triangle.jl with numpy solves."""
    xpl, _ = _xpl(quad, deg)
    r, s = xpl[:, 0], xpl[:, 1]
    for a, b in zip(frgpu.vandermonde_tri(deg, r, s), oracle.vandermonde_tri(deg, r, s)):
        np.testing.assert_allclose(a, b, rtol=0, atol=5e-14)
    for a, b in zip(frgpu.tri_operators(deg, r, s), oracle.tri_operators(deg, r, s)):
        np.testing.assert_allclose(a, b, rtol=0, atol=5e-14)


@pytest.mark.parametrize("deg", [1, 2, 3])
def test_tri_operators_exact_on_polynomials(frgpu, quad, deg):
    """dl differentiates and lf interpolates every polynomial of degree deg
    exactly; the modal basis is orthonormal where the rule is exact."""
    xpl, w = _xpl(quad, deg)
    r, s = xpl[:, 0], xpl[:, 1]
    V, dl, lf, phi = frgpu.tri_operators(deg, r, s)
    pf, _ = frgpu.triface_quadrature(deg)
    for i in range(deg + 1):
        for j in range(deg + 1 - i):
            p = r ** i * s ** j
            dpr = i * r ** max(i - 1, 0) * s ** j
            dps = j * r ** i * s ** max(j - 1, 0)
            assert np.max(np.abs(dl[:, :, 0] @ p - dpr)) < 1e-12
            assert np.max(np.abs(dl[:, :, 1] @ p - dps)) < 1e-12
            for f in range(3):
                assert np.max(np.abs(lf[f] @ p - pf[f, :, 0] ** i * pf[f, :, 1] ** j)) < 1e-12
    if deg <= 2:
        assert np.max(np.abs(V.T @ np.diag(2 * w) @ V - np.eye(len(w)))) < 1e-13


@pytest.mark.parametrize("periodic", [True, False])
def test_tri_mesh_neighbours_match_coordinates(frgpu, quad, periodic):
    """The flux-point neighbours of the mesh builder (vertex keys, opposite
    traversal of a shared face) are the points neighbour_fpidx finds by
    coordinates (src/Geometry/geo_neighbor.jl:49-57), up to the period."""
    deg = 2
    sp = _space(frgpu, quad, 5, 4, deg, periodic)
    n = sp.nb_cell
    assert (np.all(n >= 0) if periodic else np.any(n < 0))
    for c in range(sp.ncell):
        for f in range(3):
            for k in range(deg + 1):
                m = n[c, f, k]
                if m < 0:
                    assert sp.cell_type[c] == 1
                    continue
                d = sp.xfg[c, f, k] - sp.xfg[m, sp.nb_face[c, f, k], sp.nb_point[c, f, k]]
                d -= np.round(d)  # periodic images of the unit square
                assert np.max(np.abs(d)) < 1e-14


@pytest.mark.parametrize("deg", [1, 2, 3])
def test_oracle_tri_free_stream_and_conservation(frgpu, oracle, quad, deg):
    """dudt! keeps a uniform state, and on a periodic mesh the residual's
    integral sum_c det J_c sum_j w_j du_j vanishes."""
    sp = _space(frgpu, quad, 6, 5, deg)
    P = _oracle_problem(oracle, sp, -1.0)
    assert np.max(np.abs(P.rhs(np.full((sp.ncell, sp.np), 1.3, order="F")))) < 1e-13
    du = P.rhs(_wave(sp))
    _, w = _xpl(quad, deg)
    assert abs(np.sum(np.linalg.det(sp.J)[:, None] * w[None, :] * du)) < 1e-12


@pytest.mark.parametrize("deg", [1, 2])
def test_oracle_tri_convergence(frgpu, oracle, quad, deg):
    """The residual of sin(2 pi x) cos(2 pi y) approaches -a (u_x + u_y) at
    order deg under refinement (a = -1 as dev/wave_triangle.jl:37)."""
    errs = []
    for nx in (8, 16, 32):
        sp = _space(frgpu, quad, nx, nx, deg)
        P = _oracle_problem(oracle, sp, -1.0)
        X, Y = sp.xpg[..., 0], sp.xpg[..., 1]
        u = np.sin(2 * np.pi * X) * np.cos(2 * np.pi * Y)
        ex = 2 * np.pi * (np.cos(2 * np.pi * X) * np.cos(2 * np.pi * Y) - np.sin(2 * np.pi * X) * np.sin(2 * np.pi * Y))
        errs.append(np.max(np.abs(P.rhs(np.asfortranarray(u)) - ex)))
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert np.all(rates > deg - 0.15), rates


def test_oracle_tri_erk_forms(frgpu, oracle, quad):
    """fro_tri_erk with Euler is fma(dt, L(u), u); with the SSPRK33 tableau it
    agrees with the Shu-Osher form of the same method to round-off."""
    sp = _space(frgpu, quad, 5, 5, 2)
    P = _oracle_problem(oracle, sp, -1.0)
    u = _wave(sp)
    dt = 1e-3
    e = P.erk(u, dt, 1, np.zeros((1, 1)), np.ones(1))
    assert np.max(np.abs(e - (u + dt * P.rhs(u)))) < 1e-15
    A = np.array([[0, 0, 0], [1, 0, 0], [0.25, 0.25, 0]])
    b = np.array([1 / 6, 1 / 6, 2 / 3])
    u1 = u + dt * P.rhs(u)
    u2 = 0.75 * u + 0.25 * (u1 + dt * P.rhs(u1))
    u3 = u / 3 + 2 / 3 * (u2 + dt * P.rhs(u2))
    assert np.max(np.abs(P.erk(u, dt, 1, A, b) - u3)) < 1e-14


def test_oracle_tri_boundary_cells_frozen(frgpu, oracle, quad):
    """Cells of type 1 (with a boundary face) keep du = 0; the others see no
    boundary face (dev/wave_triangle.jl:117-121)."""
    sp = _space(frgpu, quad, 6, 6, 2, periodic=False)
    du = _oracle_problem(oracle, sp, -1.0).rhs(_wave(sp))
    assert np.all(du[sp.cell_type == 1] == 0.0)
    assert np.any(du[sp.cell_type == 0] != 0.0)


def _write_gmsh(path, pts, cid, version):
    """A Gmsh ASCII file of the triangles (plus one line element, which the
    reader skips)."""
    with open(path, "w") as f:
        f.write(f"$MeshFormat\n{version} 0 8\n$EndMeshFormat\n")
        if version == "2.2":
            f.write(f"$Nodes\n{len(pts)}\n")
            for q, (x, y) in enumerate(pts.tolist()):
                f.write(f"{q + 1} {x!r} {y!r} 0\n")
            f.write(f"$EndNodes\n$Elements\n{len(cid) + 1}\n1 1 2 0 1 1 2\n")
            for q, c in enumerate(cid.tolist()):
                f.write(f"{q + 2} 2 2 0 1 {c[0] + 1} {c[1] + 1} {c[2] + 1}\n")
            f.write("$EndElements\n")
        else:
            f.write(f"$Nodes\n1 {len(pts)} 1 {len(pts)}\n2 1 0 {len(pts)}\n")
            f.write("".join(f"{q + 1}\n" for q in range(len(pts))))
            f.write("".join(f"{x!r} {y!r} 0\n" for x, y in pts.tolist()))
            f.write(f"$EndNodes\n$Elements\n2 {len(cid) + 1} 1 {len(cid) + 1}\n1 1 1 1\n1 1 2\n")
            f.write(f"2 1 2 {len(cid)}\n")
            f.write("".join(f"{q + 2} {c[0] + 1} {c[1] + 1} {c[2] + 1}\n" for q, c in enumerate(cid.tolist())))
            f.write("$EndElements\n")


def test_tri_square_mesh_counts(frgpu):
    """2 nx ny cells; on a periodic mesh every cell is interior, on a bounded
    one exactly the cells with a face on the rectangle's edge have type 1; a
    periodic mesh needs at least 3 squares per side."""
    pts, cid, key, ct = frgpu.tri_square_mesh(5, 4, periodic=True)
    assert cid.shape == (40, 3) and np.all(ct == 0)
    pts, cid, key, ct = frgpu.tri_square_mesh(5, 4, periodic=False)
    on_edge = np.zeros(len(cid), dtype=bool)
    for c, v in enumerate(cid):
        for a, b in ((v[0], v[1]), (v[1], v[2]), (v[2], v[0])):
            pa, pb = pts[a], pts[b]
            on_edge[c] |= bool(np.any((pa == pb) & ((pa == 0) | (pa == 1))))
    assert np.array_equal(ct == 1, on_edge)
    with pytest.raises(ValueError):
        frgpu.tri_square_mesh(2, 5, periodic=True)


@pytest.mark.parametrize("version", ["2.2", "4.1"])
def test_read_gmsh_round_trip(frgpu, tmp_path, version):
    pts, cid, _, ct = frgpu.tri_square_mesh(4, 3, periodic=False)
    path = str(tmp_path / "m.msh")
    _write_gmsh(path, pts, cid, version)
    p2, c2 = frgpu.read_gmsh(path)
    assert np.array_equal(p2, pts) and np.array_equal(c2, cid)
    assert np.array_equal(frgpu.boundary_cell_type(c2), ct)
    xpl, wp = np.stack([[-2 / 3, 1 / 3, -2 / 3], [1 / 3, -2 / 3, -2 / 3]], axis=1), np.full(3, 1 / 3)
    sp = frgpu.tri_space_from_gmsh(path, 1, xpl, wp)
    assert sp.ncell == len(cid) and np.array_equal(sp.cell_type, ct)


def _write_su2(path, pts, cid, edges):
    with open(path, "w") as f:
        f.write("% a triangulated rectangle\nNDIME= 2\n")
        f.write(f"NELEM= {len(cid)}\n")
        for c, v in enumerate(cid):
            f.write(f"5 {v[0]} {v[1]} {v[2]} {c}\n")
        f.write(f"NPOIN= {len(pts)}\n")
        for q, p in enumerate(pts):
            f.write(f"{float(p[0])!r} {float(p[1])!r} {q}\n")
        f.write("NMARK= 1\nMARKER_TAG= wall\n")
        f.write(f"MARKER_ELEMS= {len(edges)}\n")
        for a, b in edges:
            f.write(f"3 {a} {b}\n")


def test_read_su2_round_trip(frgpu, tmp_path):
    """SU2: triangles, points and the boundary marker's edges come back; the
    marker's edges are exactly the faces with no neighbour."""
    pts, cid, _, ct = frgpu.tri_square_mesh(4, 3, periodic=False)
    faces = {}
    for v in cid:
        for a, b in ((v[0], v[1]), (v[1], v[2]), (v[2], v[0])):
            faces[tuple(sorted((a, b)))] = faces.get(tuple(sorted((a, b))), 0) + 1
    edges = sorted(f for f, n in faces.items() if n == 1)
    path = str(tmp_path / "m.su2")
    _write_su2(path, pts, cid, edges)
    p2, c2, mk = frgpu.read_su2(path)
    assert np.array_equal(p2, pts) and np.array_equal(c2, cid)
    assert list(mk) == ["wall"] and np.array_equal(mk["wall"], np.array(edges))
    sp = frgpu.TriFRPSpace(p2, c2, 2, cell_type=frgpu.boundary_cell_type(c2))
    assert int((sp.nb_cell[:, :, 0] < 0).sum()) == len(edges)


# the reference checkout's meshes, when FR_REFERENCE names a checkout
REFERENCE_ASSETS = os.path.join(os.environ["FR_REFERENCE"], "assets") if os.environ.get("FR_REFERENCE") else None


def test_clockwise_cells_are_rejected(frgpu):
    """TriFRPSpace needs counterclockwise cells (det J > 0); a mesh with a
    clockwise cell is refused with the cell named."""
    pts, cid, key, ct = frgpu.tri_square_mesh(3, 3, periodic=False)
    bad = cid.copy()
    bad[4] = bad[4][[0, 2, 1]]
    xpl, wp = np.stack([[-2 / 3, 1 / 3, -2 / 3], [1 / 3, -2 / 3, -2 / 3]], axis=1), np.full(3, 1 / 3)
    frgpu.TriFRPSpace(pts, cid, 1, xpl, wp, key, ct)
    with pytest.raises(ValueError, match=r"clockwise.*\[4\]"):
        frgpu.TriFRPSpace(pts, bad, 1, xpl, wp, key, ct)


@pytest.mark.skipif(REFERENCE_ASSETS is None or not os.path.isdir(REFERENCE_ASSETS),
                    reason="set FR_REFERENCE to a reference checkout to read its meshes")
def test_reference_su2_mesh(frgpu):
    """assets/linesource.su2: 8442 positively oriented triangles on 4342 points;
    its marker holds the 240 faces that have no neighbour."""
    pts, cid, mk = frgpu.read_su2(os.path.join(REFERENCE_ASSETS, "linesource.su2"))
    assert cid.shape == (8442, 3) and pts.shape == (4342, 2)
    assert np.all(np.linalg.det(frgpu.rs_jacobi(cid, pts)) > 0)
    sp = frgpu.TriFRPSpace(pts, cid, 1, cell_type=frgpu.boundary_cell_type(cid))
    assert sum(len(e) for e in mk.values()) == int((sp.nb_cell[:, :, 0] < 0).sum()) == 240


@pytest.mark.skipif(REFERENCE_ASSETS is None or not os.path.isdir(REFERENCE_ASSETS),
                    reason="set FR_REFERENCE to a reference checkout to read its meshes")
@pytest.mark.parametrize("name,ncell", [("square.msh", 2120), ("linesource.msh", 2122)])
def test_reference_meshes(frgpu, oracle, quad, name, ncell):
    """The reference's triangle meshes: assets/square.msh (dev/wave_triangle.jl:6)
    and assets/linesource.msh (the TriFRPSpace of test/runtests.jl:22), Gmsh 4.1:
    every triangle positively oriented, the neighbour flux points equal to the
    coordinate matching of neighbour_fpidx, and the oracle's residual of a
    uniform state zero."""
    pts, cid = frgpu.read_gmsh(os.path.join(REFERENCE_ASSETS, name))
    assert cid.shape == (ncell, 3) and np.all(np.linalg.det(frgpu.rs_jacobi(cid, pts)) > 0)
    xpl, wp = _xpl(quad, 2)
    sp = frgpu.TriFRPSpace(pts, cid, 2, xpl, wp, cell_type=frgpu.boundary_cell_type(cid))
    m = sp.nb_cell >= 0
    c, f, k = np.nonzero(m)
    d = sp.xfg[c, f, k] - sp.xfg[sp.nb_cell[m], sp.nb_face[m], sp.nb_point[m]]
    assert np.max(np.abs(d)) < 1e-14
    P = _oracle_problem(oracle, sp, -1.0)
    assert np.max(np.abs(P.rhs(np.full((sp.ncell, sp.np), 0.7, order="F")))) < 1e-11


def test_tri_create_rejects_bad_arguments(frgpu):
    """Argument checks of frgpu_tri_create run before any device work."""
    from frgpu import _lib

    L = _lib.lib()
    h = C.c_void_p()
    z = np.zeros(64)
    zi = np.zeros(64, dtype=np.int32)
    d, i = _lib.dptr(z), zi.ctypes.data_as(_lib._I)
    assert L.frgpu_tri_create(4, 5, 0, 1.0, d, d, d, d, d, i, i, i, i, C.byref(h)) == _lib.ERR_ARG
    assert "degree" in _lib.last_error()
    assert L.frgpu_tri_create(4, 1, 0, 1.0, d, None, d, d, d, i, i, i, i, C.byref(h)) == _lib.ERR_ARG
    assert L.frgpu_tri_create(0, 1, 0, 1.0, d, d, d, d, d, i, i, i, i, C.byref(h)) == _lib.ERR_ARG
    assert L.frgpu_tri_step_erk(None, 1, d, d, 0.1, 1) == _lib.ERR_ARG
    assert L.frgpu_tri_operators(0, d, d, None, None, None, None) == _lib.ERR_ARG
    assert L.frgpu_tri_operators(2, None, d, None, None, None, None) == _lib.ERR_ARG
    assert L.frgpu_vandermonde_tri(2, d, d, 0, d, None, None) == _lib.ERR_ARG
    with pytest.raises(ValueError):
        frgpu.tri_operators(2, np.zeros(5), np.zeros(5))   # degree 2 takes 6 points
    # coincident solution points: a singular Vandermonde matrix is refused
    with pytest.raises(frgpu.FRGPUError):
        frgpu.tri_operators(1, np.full(3, -0.5), np.full(3, -0.5))


# ---------------------------------------------------------------- GPU
def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.gpu
@pytest.mark.parametrize("deg", [1, 2, 3])
@pytest.mark.parametrize("periodic", [True, False])
def test_tri_rhs_matches_oracle(frgpu, oracle, quad, deg, periodic):
    """frgpu_tri_rhs in FP64 gives the oracle's bits (same evaluation order,
    no contracted multiply-adds).  FP32K: the interface wave speed
    (fL - fR) / (uL - uR + 1e-6) of dev/wave_triangle.jl:95 cancels to a few
    FP32 digits where the jump is small, so the residual of a smooth state
    holds 1e-3 relative (measured 9.5e-4 at p=3, 2e-5 at p <= 2)."""
    sp = _space(frgpu, quad, 12, 9, deg, periodic)
    u = _wave(sp)
    ref = _oracle_problem(oracle, sp, -1.0).rhs(u)
    prob = frgpu.TriAdvectionProblem(u, sp, -1.0)
    assert np.array_equal(prob.rhs(u), ref)
    p32 = frgpu.TriAdvectionProblem(u, sp, -1.0, precision="fp32k")
    assert _rel(p32.rhs(u), ref) < (2e-3 if deg == 3 else 1e-4)


@pytest.mark.gpu
@pytest.mark.parametrize("alg", ["SSPRK33", "Euler", "RK4"])
def test_tri_steps_match_oracle(frgpu, oracle, quad, alg):
    """Fixed explicit steps on the device state (CUDA-graph replay) against the
    oracle's fro_tri_erk: FP64 bit-identical, FP32K (compensated update,
    residual limited by the FP32 wave-speed estimate) within 1e-4."""
    deg = 3
    sp = _space(frgpu, quad, 10, 10, deg)
    u = _wave(sp)
    dt = 2e-3
    if alg == "SSPRK33":
        A, b, m = np.array([[0, 0, 0], [1, 0, 0], [0.25, 0.25, 0]]), np.array([1 / 6, 1 / 6, 2 / 3]), None
    else:
        m = frgpu.Euler() if alg == "Euler" else frgpu.RK4()
        A, b = m.A, m.b
    ref = _oracle_problem(oracle, sp, -1.0).erk(u, dt, 5, A, b)
    prob = frgpu.TriAdvectionProblem(u, sp, -1.0)
    prob.step(3, dt, m)
    prob.step(2, dt, m)
    assert np.array_equal(prob.u, ref)
    assert prob.launches() > 0
    p32 = frgpu.TriAdvectionProblem(u, sp, -1.0, precision="fp32k")
    p32.step(5, dt, m)
    assert _rel(p32.u, ref) < 1e-4


@pytest.mark.gpu
def test_tri_state_round_trip_and_errors(frgpu, quad):
    """set/get of the state is exact in FP64 and within the high + low pair in
    FP32K; a non-finite state and a bad dt are refused."""
    sp = _space(frgpu, quad, 6, 6, 2)
    u = _wave(sp)
    prob = frgpu.TriAdvectionProblem(u, sp, -1.0)
    assert np.array_equal(prob.u, u)
    p32 = frgpu.TriAdvectionProblem(u, sp, -1.0, precision="fp32k")
    assert np.max(np.abs(p32.u - u)) < 1e-13
    bad = u.copy()
    bad[0, 0] = np.nan
    with pytest.raises(frgpu.FRGPUError):
        prob.u = bad
    with pytest.raises(frgpu.FRGPUError):
        prob.step(1, -1.0)
