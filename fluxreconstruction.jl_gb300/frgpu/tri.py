"""Unstructured triangles on the GPU.

``TriFRPSpace`` mirrors the reference's TriFRPSpace (src/struct.jl:305-352)
for a mesh given as vertex coordinates and cell vertex ids; its operators come
from libfrgpu's host setup math (``frgpu_tri_operators``).  The solution
points are tri_quadrature(deg) (src/Quadrature/quadrature.jl:14-71; the
Williams-Shunn-Jameson rules), unless the caller passes its own.  ``TriAdvectionProblem`` is the linear-advection dudt! of
dev/wave_triangle.jl:44-125 with its explicit time steps, all on the GPU
through the ``frgpu_tri_*`` entry points.  Meshes come from Gmsh ASCII
files (``read_gmsh``, the reference's assets/*.msh), SU2 files (``read_su2``) or from
``tri_square_mesh`` (a triangulated rectangle, two right triangles per square,
periodic or not).
"""
from __future__ import annotations

import ctypes as C
from fractions import Fraction

import numpy as np

from . import _lib as L
from ._lib import check, dptr


def _ip(a):
    return a.ctypes.data_as(L._I)


# Williams-Shunn-Jameson rules (D. M. Williams, L. Shunn, A. Jameson, "Symmetric
# quadrature rules for simplexes based on sphere close packed lattice
# arrangements", J. Comput. Appl. Math. 266 (2014) 18-38) in barycentric orbits:
# tri_quadrature(deg) takes the rule with deg + 1 points per edge (the
# reference's src/Quadrature/williams_shunn_jameson_{2,3,4} schemes).  Each orbit
# is (kind, weights, parameters...) with one weight and parameter per orbit of
# that kind.  Degree 1 is the interior three-point rule (a = 1/6) and degree 2
# the unique symmetric six-point rule of degree 4; degree 3 is the published
# member of the one-parameter family of symmetric ten-point rules of degree 5,
# as printed (the points define the discretisation, so they have to be the same).
_WSJ_ORBITS = {
    1: (("d3_aa", (Fraction(1, 3),), (Fraction(1, 6),)),),
    2: (("d3_aa", (0.1099517436553219, 0.2233815896780114), (0.09157621350977073, 0.4459484909159649)),),
    3: (("centroid", (0.2015429868248577,)),
        ("d3_aa", (0.04195551878545865,), (0.05556405873493273,)),
        ("d3_ab", (0.1120984094697944,), (0.2955337173474313,), (0.6342107415763597,))),
}


def _wsj_points(deg: int):
    """Barycentric points [n, 3] and weights [n] (summing to 1) of the rule for
    degree deg, orbit by orbit; inside an orbit kind, point-major across its
    orbits (the reference's expansion order, which fixes the point order)."""
    if deg not in _WSJ_ORBITS:
        raise ValueError(f"tri_quadrature is built for degrees {sorted(_WSJ_ORBITS)}, not {deg}")
    pts, wts = [], []
    for kind, w, *par in _WSJ_ORBITS[deg]:
        # object arrays: exact for the Fraction entries, IEEE double for the rest
        w = np.asarray(w, dtype=object)
        par = [np.asarray(q, dtype=object) for q in par]
        if kind == "centroid":
            orb = [np.full((len(w), 3), Fraction(1, 3), dtype=object)]
        elif kind == "d3_aa":
            a = par[0]
            b = 1 - 2 * a
            orb = [np.stack(t, axis=1) for t in ((a, a, b), (a, b, a), (b, a, a))]
        else:  # d3_ab
            a, b = par
            c = 1 - a - b
            orb = [np.stack(t, axis=1) for t in ((a, b, c), (c, a, b), (b, c, a), (b, a, c), (c, b, a), (a, c, b))]
        for o in orb:
            pts.append(o)
            wts.append(w)
    return np.concatenate(pts).astype(np.float64), np.concatenate(wts).astype(np.float64)


def xy_rs(x, y):
    """xy_rs (src/Geometry/geo_transform.jl:65-73): the equilateral triangle with
    vertices (-1, -1/sqrt 3), (1, -1/sqrt 3), (0, 2/sqrt 3) -> the reference right
    triangle (r, s)."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    L1 = (np.sqrt(3.0) * y + 1.0) / 3.0
    L2 = (-3.0 * x - np.sqrt(3.0) * y + 2.0) / 6.0
    L3 = (3.0 * x - np.sqrt(3.0) * y + 2.0) / 6.0
    return -L2 + L3 - L1, -L2 - L3 + L1


def tri_quadrature(deg: int, vertices=None, transform: bool = True):
    """tri_quadrature(deg; vertices, transform) (src/Quadrature/quadrature.jl:14-71):
    the (deg+1)(deg+2)/2 Williams-Shunn-Jameson solution points of a triangle and
    their weights (summing to 1).  The barycentric points are placed in the
    triangle with the given vertices (default: the equilateral triangle
    (-1, -1/sqrt 3), (1, -1/sqrt 3), (0, 2/sqrt 3)) through the trilinear ->
    Cartesian map (a x p1 + b y p2 + c z p3) / (a x + b y + c z), a, b, c the
    lengths of the sides opposite p1, p2, p3; with transform the result is mapped
    to the reference right triangle by xy_rs.  Returns points [n, 2], weights [n].
    Degrees 1-3, those the triangle residual kernel is built for."""
    if vertices is None:
        vertices = ((-1.0, -1 / np.sqrt(3.0)), (1.0, -1 / np.sqrt(3.0)), (0.0, 2 / np.sqrt(3.0)))
    p1, p2, p3 = (np.asarray(v, dtype=np.float64) for v in vertices)
    a = np.linalg.norm(p2 - p3)
    b = np.linalg.norm(p3 - p1)
    c = np.linalg.norm(p2 - p1)
    bary, w = _wsj_points(deg)
    x, y, z = bary[:, 0:1], bary[:, 1:2], bary[:, 2:3]
    pts = (a * x * p1 + b * y * p2 + c * z * p3) / (a * x + b * y + c * z)
    if transform:
        r, s = xy_rs(pts[:, 0], pts[:, 1])
        pts = np.stack([r, s], axis=1)
    return pts, w


def triface_quadrature(deg: int):
    """triface_quadrature(N) (src/Quadrature/quadrature.jl:86-106): flux points
    pf[3, N+1, 2] on faces 1 -> 2, 2 -> 3, 3 -> 1 of the reference right
    triangle and weights wf[3, N+1] (Gauss-Legendre times the face length)."""
    x, w = np.polynomial.legendre.leggauss(deg + 1)
    pf = np.zeros((3, deg + 1, 2))
    pf[0, :, 0], pf[0, :, 1] = x, -1.0
    pf[1, :, 0], pf[1, :, 1] = x[::-1], x
    pf[2, :, 0], pf[2, :, 1] = -1.0, x[::-1]
    wf = np.stack([w, w * np.sqrt(2.0), w])
    return pf, wf


def rs_xy(r, s, v1, v2, v3):
    """rs_xy (src/Geometry/geo_transform.jl:16-24): reference (r, s) -> (x, y)."""
    r = np.asarray(r, dtype=np.float64)[..., None]
    s = np.asarray(s, dtype=np.float64)[..., None]
    return -(r + s) / 2 * v1 + (r + 1) / 2 * v2 + (s + 1) / 2 * v3


def rs_jacobi(cellid, points):
    """rs_jacobi(cells, points) (src/Geometry/geo_jacobi.jl:32-43): per cell
    J = [xr xs; yr ys] with (xr, yr) = (v2 - v1) / 2, (xs, ys) = (v3 - v1) / 2;
    returned as an array [ncell, 2, 2]."""
    v1, v2, v3 = (points[cellid[:, m]] for m in range(3))
    J = np.zeros((len(cellid), 2, 2))
    J[:, :, 0] = (v2 - v1) / 2
    J[:, :, 1] = (v3 - v1) / 2
    return J


def vandermonde_tri(deg: int, r, s):
    """vandermonde_matrix(Tri, N, r, s) and its r, s derivatives
    (src/Transform/transform.jl:36-50, :106-127)."""
    r = np.ascontiguousarray(r, dtype=np.float64)
    s = np.ascontiguousarray(s, dtype=np.float64)
    npm = (deg + 1) * (deg + 2) // 2
    V, Vr, Vs = (np.zeros((len(r), npm), order="F") for _ in range(3))
    check(L.lib().frgpu_vandermonde_tri(deg, dptr(r), dptr(s), len(r), dptr(V), dptr(Vr), dptr(Vs)))
    return V, Vr, Vs


def tri_operators(deg: int, r, s):
    """V, dl[np, np, 2], lf[3, deg+1, np] and phi[3, deg+1, np] of TriFRPSpace
    at the solution points (r, s)."""
    r = np.ascontiguousarray(r, dtype=np.float64)
    s = np.ascontiguousarray(s, dtype=np.float64)
    npm = (deg + 1) * (deg + 2) // 2
    if len(r) != npm or len(s) != npm:
        raise ValueError(f"degree {deg} takes {npm} solution points")
    V = np.zeros((npm, npm), order="F")
    dl = np.zeros((npm, npm, 2), order="F")
    lf = np.zeros((3, deg + 1, npm), order="F")
    phi = np.zeros((3, deg + 1, npm), order="F")
    check(L.lib().frgpu_tri_operators(deg, dptr(r), dptr(s), dptr(V), dptr(dl), dptr(lf), dptr(phi)))
    return V, dl, lf, phi


def tri_square_mesh(nx: int, ny: int, x0=0.0, x1=1.0, y0=0.0, y1=1.0, periodic=True):
    """Triangulated rectangle: nx x ny squares, each split along its rising
    diagonal into (p00, p10, p11) and (p00, p11, p01), counterclockwise; cells
    numbered square by square, row by row.  Returns points [npts, 2], cellid
    [ncell, 3] (0-based), the vertex key that identifies periodic images (the
    vertex id itself when not periodic) and cell_type [ncell] (0 interior,
    1 a cell with a boundary face, as KitBase's UnstructPSpace marks them)."""
    if nx < 1 or ny < 1 or (periodic and (nx < 3 or ny < 3)):
        raise ValueError("need nx, ny >= 1 (>= 3 when periodic, so that every face has two distinct cells)")
    xs = np.linspace(x0, x1, nx + 1)
    ys = np.linspace(y0, y1, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    points = np.stack([X.ravel(order="F"), Y.ravel(order="F")], axis=1)
    I, J = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="ij")
    vid = lambda i, j: i + (nx + 1) * j  # noqa: E731
    key = ((I % nx) + nx * (J % ny) if periodic else vid(I, J)).ravel(order="F")
    si, sj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    si, sj = si.ravel(order="F"), sj.ravel(order="F")
    cellid = np.zeros((2 * nx * ny, 3), dtype=np.int64)
    cellid[0::2] = np.stack([vid(si, sj), vid(si + 1, sj), vid(si + 1, sj + 1)], axis=1)
    cellid[1::2] = np.stack([vid(si, sj), vid(si + 1, sj + 1), vid(si, sj + 1)], axis=1)
    nbc, _, _ = _face_neighbours(cellid, key)
    cell_type = np.where(np.any(nbc < 0, axis=1), 1, 0).astype(np.int32)
    return points, cellid, key, cell_type


def read_gmsh(path: str):
    """Triangles of a Gmsh ASCII mesh (format 2.2 or 4.1), the meshes the
    reference's examples read through KitBase's UnstructPSpace
    (assets/*.msh): vertex coordinates [npts, 2] (z dropped) and the 0-based
    vertex ids [ncell, 3] of every 3-node triangle (element type 2), in the
    file's order."""
    with open(path) as f:
        lines = [ln.strip() for ln in f]
    sec = {}
    i = 0
    while i < len(lines):
        if lines[i].startswith("$") and not lines[i].startswith("$End"):
            name = lines[i][1:]
            j = lines.index("$End" + name, i)
            sec[name] = lines[i + 1:j]
            i = j
        i += 1
    if "MeshFormat" not in sec or "Nodes" not in sec or "Elements" not in sec:
        raise ValueError(f"{path}: not a Gmsh mesh with nodes and elements")
    version, binary = sec["MeshFormat"][0].split()[:2]
    if binary != "0":
        raise ValueError(f"{path}: binary Gmsh files are not read")
    tags, xy, tris = [], [], []
    nodes, elems = sec["Nodes"], sec["Elements"]
    if version.startswith("4"):
        nblocks = int(nodes[0].split()[0])
        k = 1
        for _ in range(nblocks):
            _, _, param, n = (int(v) for v in nodes[k].split())
            tags += [int(nodes[k + 1 + m]) for m in range(n)]
            xy += [[float(v) for v in nodes[k + 1 + n + m].split()[:2]] for m in range(n)]
            k += 1 + 2 * n
        nblocks = int(elems[0].split()[0])
        k = 1
        for _ in range(nblocks):
            _, _, etype, n = (int(v) for v in elems[k].split())
            if etype == 2:
                tris += [[int(v) for v in elems[k + 1 + m].split()[1:4]] for m in range(n)]
            k += 1 + n
    elif version.startswith("2"):
        n = int(nodes[0])
        for m in range(n):
            v = nodes[1 + m].split()
            tags.append(int(v[0]))
            xy.append([float(v[1]), float(v[2])])
        n = int(elems[0])
        for m in range(n):
            v = [int(t) for t in elems[1 + m].split()]
            if v[1] == 2:
                tris.append(v[3 + v[2]:6 + v[2]])
    else:
        raise ValueError(f"{path}: Gmsh format {version} is not read")
    index = {t: q for q, t in enumerate(tags)}
    cellid = np.array([[index[t] for t in c] for c in tris], dtype=np.int64).reshape(-1, 3)
    return np.array(xy, dtype=np.float64).reshape(-1, 2), cellid


def read_su2(path: str):
    """Triangles of an SU2 ASCII mesh (the reference's assets/linesource.su2):
    vertex coordinates [npts, 2], the 0-based vertex ids [ncell, 3] of every
    triangle (element type 5) in the file's order, and the boundary markers as
    {tag: edges [n, 2]} (line elements, type 3).  Other element types are
    skipped."""
    with open(path) as f:
        toks = [ln.split("%")[0].strip() for ln in f]
    lines = [t for t in toks if t]
    xy, tris, markers = None, [], {}
    i = 0

    def value(line):
        return line.split("=", 1)[1].split()

    while i < len(lines):
        key = lines[i].split("=", 1)[0].strip().upper() if "=" in lines[i] else ""
        if key == "NDIME":
            if int(value(lines[i])[0]) != 2:
                raise ValueError(f"{path}: only 2D SU2 meshes are read")
            i += 1
        elif key == "NELEM":
            n = int(value(lines[i])[0])
            for ln in lines[i + 1:i + 1 + n]:
                v = [int(t) for t in ln.split()]
                if v[0] == 5:
                    tris.append(v[1:4])
            i += 1 + n
        elif key == "NPOIN":
            n = int(value(lines[i])[0])
            xy = [[float(t) for t in ln.split()[:2]] for ln in lines[i + 1:i + 1 + n]]
            i += 1 + n
        elif key == "MARKER_TAG":
            tag = value(lines[i])[0] if value(lines[i]) else ""
            n = int(value(lines[i + 1])[0])
            edges = [[int(t) for t in ln.split()[1:3]] for ln in lines[i + 2:i + 2 + n]
                     if int(ln.split()[0]) == 3]
            markers[tag] = np.array(edges, dtype=np.int64).reshape(-1, 2)
            i += 2 + n
        else:
            i += 1
    if xy is None or not tris:
        raise ValueError(f"{path}: no points or no triangles")
    return (np.array(xy, dtype=np.float64).reshape(-1, 2), np.array(tris, dtype=np.int64).reshape(-1, 3),
            markers)


def boundary_cell_type(cellid, key=None):
    """Cell types as the triangle script uses them: 1 for a cell with a face on
    the boundary (no neighbour), 0 otherwise."""
    key = np.arange(int(np.max(cellid)) + 1) if key is None else np.asarray(key)
    nbc, _, _ = _face_neighbours(np.asarray(cellid), key)
    return np.where(np.any(nbc < 0, axis=1), 1, 0).astype(np.int32)


def _face_neighbours(cellid, key):
    """Per cell and face (1 -> 2, 2 -> 3, 3 -> 1) the neighbour cell (-1 on a
    boundary), its face, and whether it runs along the face in the same
    direction; faces matched by their vertex keys."""
    nc = len(cellid)
    kv = key[cellid]
    a = np.stack([kv[:, 0], kv[:, 1], kv[:, 2]], axis=1)
    b = np.stack([kv[:, 1], kv[:, 2], kv[:, 0]], axis=1)
    lo, hi = np.minimum(a, b).ravel(), np.maximum(a, b).ravel()
    order = np.lexsort((hi, lo))
    nbc = -np.ones(3 * nc, dtype=np.int64)
    nbf = -np.ones(3 * nc, dtype=np.int64)
    same = np.zeros(3 * nc, dtype=bool)
    lo_s, hi_s = lo[order], hi[order]
    pair = np.nonzero((lo_s[:-1] == lo_s[1:]) & (hi_s[:-1] == hi_s[1:]))[0]
    if len(pair) and np.any(np.diff(pair) == 1):
        raise ValueError("a face is shared by more than two cells")
    fa, fb = order[pair], order[pair + 1]
    nbc[fa], nbf[fa] = fb // 3, fb % 3
    nbc[fb], nbf[fb] = fa // 3, fa % 3
    af, bf = a.ravel(), b.ravel()
    same[fa] = af[fa] == af[fb]
    same[fb] = af[fb] == af[fa]
    return nbc.reshape(nc, 3), nbf.reshape(nc, 3), same.reshape(nc, 3)


class TriFRPSpace:
    """TriFRPSpace(file, deg) of src/struct.jl:305-352 for a mesh in memory:
    points [npts, 2], cellid [ncell, 3] (0-based, counterclockwise), the
    solution points xpl[np, 2] and weights wp[np] (default: tri_quadrature(deg)), and
    optionally a vertex key identifying periodic images and the cell types.
    Fields as the reference names them: J, iJ, xpl, wp, xpg, xfl, xfg, wf, V,
    dl (the reference's ∂l), lf, phi (ϕ), and fpn as the three arrays
    nb_cell, nb_face, nb_point [ncell, 3, deg+1] (0-based neighbour_fpidx,
    src/Geometry/geo_neighbor.jl:8-60; nb_cell = -1 on a boundary face)."""

    def __init__(self, points, cellid, deg: int, xpl=None, wp=None, key=None, cell_type=None):
        self.points = np.asarray(points, dtype=np.float64)
        self.cellid = np.asarray(cellid, dtype=np.int64)
        self.deg = deg
        self.np = (deg + 1) * (deg + 2) // 2
        if xpl is None:
            xpl, wq = tri_quadrature(deg)
            wp = wq if wp is None else wp
        self.xpl = np.asarray(xpl, dtype=np.float64)
        self.wp = np.asarray(wp, dtype=np.float64)
        if self.xpl.shape != (self.np, 2):
            raise ValueError(f"degree {deg} takes {self.np} solution points")
        ncell = len(self.cellid)
        self.ncell = ncell
        key = np.arange(len(self.points)) if key is None else np.asarray(key)
        self.cell_type = (np.zeros(ncell, dtype=np.int32) if cell_type is None
                          else np.asarray(cell_type, dtype=np.int32))
        self.J = rs_jacobi(self.cellid, self.points)
        det = np.linalg.det(self.J)
        bad = np.flatnonzero(~(det > 0))
        if bad.size:
            raise ValueError(f"{bad.size} cell(s) are clockwise or degenerate (det J <= 0), for example cells "
                             f"{bad[:8].tolist()}: TriFRPSpace needs counterclockwise vertex order")
        self.iJ = np.linalg.inv(self.J)
        self.V, self.dl, self.lf, self.phi = tri_operators(deg, self.xpl[:, 0], self.xpl[:, 1])
        self.xfl, self.wf = triface_quadrature(deg)
        v = [self.points[self.cellid[:, m]][:, None, :] for m in range(3)]
        self.xpg = rs_xy(self.xpl[:, 0], self.xpl[:, 1], *v)
        self.xfg = np.stack([rs_xy(self.xfl[f, :, 0], self.xfl[f, :, 1], *v) for f in range(3)], axis=1)
        nbc, nbf, same = _face_neighbours(self.cellid, key)
        m = deg + 1
        k = np.arange(m)
        self.nb_cell = np.repeat(nbc[:, :, None], m, axis=2)
        self.nb_face = np.where(self.nb_cell >= 0, np.repeat(nbf[:, :, None], m, axis=2), -1)
        # a neighbour running the other way along the face meets point k at m-1-k
        self.nb_point = np.where(same[:, :, None], k[None, None, :], (m - 1 - k)[None, None, :])
        self.nb_point = np.where(self.nb_cell >= 0, self.nb_point, -1)


def tri_space_from_gmsh(path: str, deg: int, xpl=None, wp=None) -> TriFRPSpace:
    """TriFRPSpace(file, deg) (src/struct.jl:305-352) for a Gmsh ASCII file:
    its triangles, the solution points xpl and weights wp (default:
    tri_quadrature(deg)), and the cells with a boundary face marked type 1."""
    points, cellid = read_gmsh(path)
    return TriFRPSpace(points, cellid, deg, xpl, wp, cell_type=boundary_cell_type(cellid))


class TriAdvectionProblem:
    """The ODEProblem(dudt!, u, tspan, p) of dev/wave_triangle.jl:44-135
    (u_t + a u_x + a u_y = 0 on a TriFRPSpace) held on the GPU; ``u[ncell, np]``.
    ``precision`` is "fp64" (bit-identical to the oracle) or "fp32k" (FP32
    residual, compensated update)."""

    def __init__(self, u, space: TriFRPSpace, a: float, precision: str = "fp64"):
        self.space = space
        prec = {"fp64": L.FP64, "fp32k": L.FP32K}[precision]
        sp = space
        arrs = [np.asfortranarray(x, dtype=np.float64) for x in (sp.dl, sp.lf, sp.phi, sp.J, sp.iJ)]
        ints = [np.asfortranarray(x, dtype=np.int32) for x in (sp.nb_cell, sp.nb_face, sp.nb_point, sp.cell_type)]
        h = C.c_void_p()
        check(L.lib().frgpu_tri_create(sp.ncell, sp.deg, prec, float(a), *(dptr(x) for x in arrs),
                                       *(_ip(x) for x in ints), C.byref(h)))
        self._h = h
        self.shape = (sp.ncell, sp.np)
        self.u = u

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            L.lib().frgpu_tri_destroy(h)
            self._h = None

    @property
    def u(self) -> np.ndarray:
        out = np.zeros(self.shape, order="F")
        check(L.lib().frgpu_tri_get_state(self._h, dptr(out)))
        return out

    @u.setter
    def u(self, u) -> None:
        a = np.asfortranarray(u, dtype=np.float64)
        if a.shape != self.shape:
            raise ValueError(f"u must have shape {self.shape}")
        check(L.lib().frgpu_tri_set_state(self._h, dptr(a)))

    def rhs(self, u) -> np.ndarray:
        """dudt!(du, u, p, t) (dev/wave_triangle.jl:44-125) on the GPU."""
        a = np.asfortranarray(u, dtype=np.float64)
        if a.shape != self.shape:
            raise ValueError(f"u must have shape {self.shape}")
        du = np.zeros(self.shape, order="F")
        check(L.lib().frgpu_tri_rhs(self._h, dptr(du), dptr(a)))
        return du

    def step(self, n: int, dt: float, alg=None) -> None:
        """n fixed steps of ``alg`` (an ExplicitRK tableau, e.g. Euler(); None:
        SSPRK33) on the device state."""
        if alg is None:
            A = np.array([[0, 0, 0], [1, 0, 0], [0.25, 0.25, 0]], dtype=np.float64)
            b = np.array([1 / 6, 1 / 6, 2 / 3])
        else:
            A, b = alg.A, alg.b
        A = np.ascontiguousarray(A, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        check(L.lib().frgpu_tri_step_erk(self._h, len(b), dptr(A), dptr(b), float(dt), int(n)))

    def rhs_device(self) -> None:
        """The residual of the device state into device scratch (timing)."""
        check(L.lib().frgpu_tri_rhs_device(self._h))

    def stream(self) -> int:
        s = C.c_void_p()
        check(L.lib().frgpu_tri_stream(self._h, C.byref(s)))
        return s.value or 0

    def launches(self) -> int:
        n = C.c_longlong()
        check(L.lib().frgpu_tri_launches(self._h, C.byref(n)))
        return n.value


def Euler():
    """OrdinaryDiffEq Euler() with a fixed step, as dev/wave_triangle.jl:133 uses it."""
    from .api import ExplicitRK

    return ExplicitRK([[0.0]], [1.0], "Euler")
