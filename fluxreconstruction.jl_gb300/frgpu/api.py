"""Python mirror of FluxReconstruction.jl's interface for the residual and
time-stepping hot path, backed by libfrgpu.so (CUDA, sm_103a).

Names follow the reference (Julia's ``!`` becomes a trailing ``_``):

* ``FRPSpace1D`` / ``FRPSpace2D``           -- src/struct.jl:40-88, :229-245
* ``interp_face_`` / ``poly_derivative_``    -- src/interpolate.jl:1-10, src/derivative.jl:1-10
* ``FRAdvectionProblem`` / ``FREulerProblem`` -- src/Equation/eq_advection.jl:1-26, eq_euler.jl:1-27
* ``FREuler2DProblem`` / ``FRBGKProblem`` / ``FRBurgersProblem`` -- the ``dudt!`` / ``mol!``
  closures of example/shock-vortex.jl:26-118 and example/bgk_wave.jl:69-129
* ``init`` / ``step_`` / ``solve`` with ``SSPRK33``  -- OrdinaryDiffEq's integrator API as used
  by the examples (``init(prob, alg; adaptive=false, dt)``, ``step!(itg)``, ``itg.u``)
* ``shock_detector`` -- src/dissipation.jl:13-23; ``L1_error``/``L2_error``/``Linf_error`` --
  src/tools.jl:43-53; ``modal_filter_`` -- the :l2 filter called at example/shock-vortex.jl:316.

Arrays use the reference's index order and Julia's column-major memory order
(numpy ``order='F'``): ``u[i, k]`` (1D scalar), ``u[i, k, m]`` (1D Euler),
``u[i, j, k, l, m]`` (2D Euler), ``u[i, v, k]`` (BGK).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L
from ._lib import check, dptr

_CORR = {"radau": L.RADAU, "sd": L.SD, "huynh": L.HUYNH}
_BC = {"period": L.BC_PERIODIC, "periodic": L.BC_PERIODIC, "copy": L.BC_COPY, "extra": L.BC_COPY,
       "fix": L.BC_FIXED, "fixed": L.BC_FIXED, "dirichlet": L.BC_DIRICHLET}
_FLUX = {"roe": L.FLUX_ROE, "lf": L.FLUX_LF, "lax": L.FLUX_LF, "hll": L.FLUX_HLL, "upwind": L.FLUX_UPWIND,
         "central": L.FLUX_CENTRAL}
_PREC = {"fp64": L.FP64, "fp32k": L.FP32K, "fp32": L.FP32K}
_IND = {"none": L.IND_NONE, "plain": L.IND_PLAIN, "mlp": L.IND_MLP}


def _f64(a) -> np.ndarray:
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


# ---------------------------------------------------------------- setup math
def legendre_point(deg: int) -> np.ndarray:
    """Gauss-Legendre nodes of degree deg (src/Polynomial/poly_legendre.jl:6)."""
    r = np.zeros(deg + 1)
    check(L.lib().frgpu_legendre_point(deg, dptr(r), None))
    return r


def gauss_weights(deg: int) -> np.ndarray:
    r, w = np.zeros(deg + 1), np.zeros(deg + 1)
    check(L.lib().frgpu_legendre_point(deg, dptr(r), dptr(w)))
    return w


def lagrange_point(sp, x) -> np.ndarray:
    """lagrange_point (src/Polynomial/poly_lagrange.jl:6-31), scalar or vector x."""
    sp = _f64(sp).ravel()
    if np.ndim(x) == 0:
        out = np.zeros_like(sp)
        check(L.lib().frgpu_lagrange_point(dptr(sp), len(sp), float(x), dptr(out)))
        return out
    return np.stack([lagrange_point(sp, xi) for xi in np.asarray(x, dtype=np.float64)])


def dlagrange(sp) -> np.ndarray:
    """∂lagrange(sp) (src/Polynomial/poly_lagrange.jl:38-59): lpdm[m, k] = l_k'(r_m)."""
    sp = _f64(sp).ravel()
    n = len(sp)
    out = np.zeros((n, n), order="F")
    check(L.lib().frgpu_dlagrange(dptr(sp), n, dptr(out)))
    return out


def standard_lagrange(x):
    """standard_lagrange (src/Polynomial/poly_lagrange.jl:99-105) -> (ll, lr, lpdm)."""
    return lagrange_point(x, -1.0), lagrange_point(x, 1.0), dlagrange(x)


def _dcorr(kind: int, deg: int, x):
    x = _f64(np.atleast_1d(x)).ravel()
    dgl, dgr = np.zeros_like(x), np.zeros_like(x)
    check(L.lib().frgpu_dcorrection(kind, deg, dptr(x), len(x), dptr(dgl), dptr(dgr)))
    return dgl, dgr


def dradau(deg: int, x):
    """∂radau (src/Polynomial/poly_legendre.jl:29-37)."""
    return _dcorr(L.RADAU, deg, x)


def dsd(deg: int, x):
    """∂sd (src/Polynomial/poly_legendre.jl:44-54)."""
    return _dcorr(L.SD, deg, x)


def dhuynh(deg: int, x):
    """∂huynh (src/Polynomial/poly_legendre.jl:61-71)."""
    return _dcorr(L.HUYNH, deg, x)


def vandermonde_matrix(deg: int, r, s=None) -> np.ndarray:
    """vandermonde_matrix(N, r) (transform.jl:18-26) or (Quad, N, r, s) (:55-68)."""
    r = _f64(r).ravel()
    if s is None:
        V = np.zeros((len(r), deg + 1), order="F")
        check(L.lib().frgpu_vandermonde(deg, dptr(r), len(r), dptr(V)))
        return V
    s = _f64(s).ravel()
    V = np.zeros((len(r), (deg + 1) ** 2), order="F")
    check(L.lib().frgpu_vandermonde_quad(deg, dptr(r), dptr(s), len(r), dptr(V)))
    return V


# ---------------------------------------------------------------- spaces
class _Space:
    _h = None

    def _get(self, name: str, shape) -> np.ndarray:
        n = int(np.prod(shape))
        out = np.zeros(n)
        check(L.lib().frgpu_space_get(self._h, name.encode(), dptr(out), n))
        return out.reshape(shape, order="F")

    def __del__(self):
        if self._h is not None and L._lib is not None:
            L._lib.frgpu_space_destroy(self._h)
            self._h = None


class FRPSpace1D(_Space):
    """FRPSpace1D(x0, x1, nx, deg, ng=0, correction=:radau) (src/struct.jl:40-85).

    Fields as in the reference: deg, J, np, xpl, xpg, wp, dl, ll, lr, dhl, dhr,
    V, iV, plus the forwarded mesh fields x0, x1, nx, dx, x.  Ghost layers (ng)
    are not stored: the problem's boundary kind supplies the neighbours."""

    def __init__(self, x0, x1, nx, deg, ng=0, correction="radau"):
        h = C.c_void_p()
        check(L.lib().frgpu_space_create_1d(float(x0), float(x1), int(nx), int(deg), _CORR[correction],
                                            C.byref(h)))
        self._h = h
        self.x0, self.x1, self.nx, self.deg, self.np, self.ng = float(x0), float(x1), int(nx), int(deg), deg + 1, ng
        n = self.np
        self.dx = np.full(nx, (x1 - x0) / nx)
        self.x = x0 + (np.arange(nx) + 0.5) * self.dx
        self.J = self._get("J", (nx,))
        self.xpl = self._get("xpl", (n,))
        self.wp = self._get("wp", (n,))
        self.xpg = self._get("xpg", (nx, n))
        self.ll = self._get("ll", (n,))
        self.lr = self._get("lr", (n,))
        self.dl = self._get("dl", (n, n))
        self.dhl = self._get("dhl", (n,))
        self.dhr = self._get("dhr", (n,))
        self.V = self._get("V", (n, n))
        self.iV = self._get("iV", (n, n))


class FRPSpace2D(_Space):
    """FRPSpace2D(x0, x1, nx, y0, y1, ny, deg, ngx=0, ngy=0) (src/struct.jl:229-242)
    on uniform rectangles.  As in the reference, ``np`` is (deg+1)^2, ``wp`` is
    the tensor weight matrix, ``dhl``/``dhr`` are the Radau derivatives
    (src/struct.jl:193) and ``V``/``iV`` the tensor Vandermonde matrices.
    ``iJ`` is the (constant) inverse Jacobian diag(2/dx, 2/dy)."""

    def __init__(self, x0, x1, nx, y0, y1, ny, deg, ngx=0, ngy=0):
        h = C.c_void_p()
        check(L.lib().frgpu_space_create_2d(float(x0), float(x1), int(nx), float(y0), float(y1), int(ny),
                                            int(deg), C.byref(h)))
        self._h = h
        self.x0, self.x1, self.y0, self.y1 = float(x0), float(x1), float(y0), float(y1)
        self.nx, self.ny, self.deg = int(nx), int(ny), int(deg)
        n = deg + 1
        self.np = n * n
        self.dx = (x1 - x0) / nx
        self.dy = (y1 - y0) / ny
        self.iJ = np.array([[1.0 / (0.5 * self.dx), 0.0], [0.0, 1.0 / (0.5 * self.dy)]])
        self.J = np.array([[0.5 * self.dx, 0.0], [0.0, 0.5 * self.dy]])
        self.xpl = self._get("xpl", (n,))
        self.wp = self._get("wp", (n, n))
        self.xpg = self._get("xpg", (nx, ny, n, n, 2))
        self.ll = self._get("ll", (n,))
        self.lr = self._get("lr", (n,))
        self.dl = self._get("dl", (n, n))
        self.dhl = self._get("dhl", (n,))
        self.dhr = self._get("dhr", (n,))
        self.V = self._get("V", (n * n, n * n))
        self.iV = self._get("iV", (n * n, n * n))
        xc = x0 + (np.arange(nx) + 0.5) * self.dx
        yc = y0 + (np.arange(ny) + 0.5) * self.dy
        self.x, self.y = np.meshgrid(xc, yc, indexing="ij")


# ---------------------------------------------------------------- stateless operators
def rs_jacobi_quad(r, vertices) -> np.ndarray:
    """Jacobians of bilinear quadrilaterals at the tensor points (r_k, r_l):
    rs_jacobi(r, vertices) of src/Geometry/geo_jacobi.jl:77-108 as FRPSpace2D
    calls it (src/struct.jl:135): vertices[nx, ny, 4, 2] counterclockwise from
    the lower left; returns J[nx, ny, np, np, 2, 2] = [x_r x_s; y_r y_s] of
    X = sum_a lambda_a(r, s) V_a."""
    r = np.asarray(r, dtype=np.float64)
    V = np.asarray(vertices, dtype=np.float64)
    R, S = np.meshgrid(r, r, indexing="ij")          # point (k, l) at (r_k, r_l)
    R, S = R[None, None, :, :, None], S[None, None, :, :, None]
    v = [V[:, :, a, None, None, :] for a in range(4)]
    Xr = (S - 1) * v[0] / 4 + (1 - S) * v[1] / 4 + (S + 1) * v[2] / 4 - (S + 1) * v[3] / 4
    Xs = (R - 1) * v[0] / 4 - (R + 1) * v[1] / 4 + (R + 1) * v[2] / 4 + (1 - R) * v[3] / 4
    return np.stack([Xr, Xs], axis=-1)


def quad_points(r, vertices) -> np.ndarray:
    """xpg[nx, ny, np, np, 2] of FRPSpace2D(base, deg) for a mesh of bilinear
    quadrilaterals (src/struct.jl:161-175): the solution points (r_k, r_l) mapped
    by X = sum_a lambda_a(r, s) V_a, vertices[nx, ny, 4, 2] counterclockwise
    from the lower left."""
    r = np.asarray(r, dtype=np.float64)
    V = np.asarray(vertices, dtype=np.float64)
    R, S = np.meshgrid(r, r, indexing="ij")
    R, S = R[None, None, :, :, None], S[None, None, :, :, None]
    v = [V[:, :, a, None, None, :] for a in range(4)]
    return ((R - 1) * (S - 1) / 4 * v[0] + (R + 1) * (1 - S) / 4 * v[1] + (R + 1) * (S + 1) / 4 * v[2]
            + (1 - R) * (S + 1) / 4 * v[3])


def polar_vertices(r0, r1, nr, t0, t1, nt) -> np.ndarray:
    """Cell corners vertices[nr, nt, 4, 2] of the polar grid r0 <= r <= r1,
    t0 <= theta <= t1 with nr x nt cells (KitBase.CSpace2D, the grid of
    dev/curve_euler.jl and the cylinder scripts), counterclockwise from
    (r_i, theta_j)."""
    r = np.linspace(r0, r1, nr + 1)
    t = np.linspace(t0, t1, nt + 1)
    V = np.zeros((nr, nt, 4, 2))
    for a, (di, dj) in enumerate([(0, 0), (1, 0), (1, 1), (0, 1)]):
        R = r[di:di + nr][:, None]
        T = t[dj:dj + nt][None, :]
        V[:, :, a, 0] = R * np.cos(T)
        V[:, :, a, 1] = R * np.sin(T)
    return V


def quad_metric(r, vertices) -> np.ndarray:
    """iJ[nx, ny, np, np, 2, 2] = inv(J) at the solution points, the field
    FRPSpace2D.iJ (src/struct.jl:135-143) that ODEProblem.set_metric takes."""
    return np.asfortranarray(np.linalg.inv(rs_jacobi_quad(r, vertices)))


def quad_face_jacobians(r, vertices) -> np.ndarray:
    """FRPSpace2D's face Jacobians Ji[i, j][f, k] (src/struct.jl:145-158) as an
    array Ji[nx, ny, 4, np, 2, 2], built as the reference builds them: the face
    coordinates ri[f, :], si[f, :] (face 1: (r, 0); 2: (1, r); 3: (reversed r, 1);
    4: (0, reversed r)) go through rs_jacobi(ri, si, vertices), whose matrix method
    (src/Geometry/geo_jacobi.jl) indexes ri[i], si[i] linearly over the face
    index i only, so every point k of face f gets the Jacobian at (ri[f, 1],
    si[f, 1]): (r_1, 0), (1, r_1), (r_np, 1), (0, r_np).  On a parallelogram J
    is the same everywhere, so these equal the Jacobian on the faces."""
    r = np.asarray(r, dtype=np.float64)
    V = np.asarray(vertices, dtype=np.float64)
    nx, ny = V.shape[:2]
    n = len(r)
    pts = [(r[0], 0.0), (1.0, r[0]), (r[-1], 1.0), (0.0, r[-1])]
    v = [V[:, :, a, :] for a in range(4)]
    Ji = np.zeros((nx, ny, 4, n, 2, 2), order="F")
    for f, (R, S) in enumerate(pts):
        Xr = (S - 1) * v[0] / 4 + (1 - S) * v[1] / 4 + (S + 1) * v[2] / 4 - (S + 1) * v[3] / 4
        Xs = (R - 1) * v[0] / 4 - (R + 1) * v[1] / 4 + (R + 1) * v[2] / 4 + (1 - R) * v[3] / 4
        Ji[:, :, f, :, :, 0] = Xr[:, :, None, :]
        Ji[:, :, f, :, :, 1] = Xs[:, :, None, :]
    return Ji


def quad_face_normals(vertices):
    """Unit normals of the straight faces of a structured quadrilateral mesh
    (vertices[nx, ny, 4, 2]), in the orientation dev/parallelogram.jl uses:
    n1[i, j] on x face i (between elements i-1 and i) pointing to increasing
    i, n2[i, j] on y face j pointing to increasing j; shapes (nx+1, ny, 2) and
    (nx, ny+1, 2)."""
    V = np.asarray(vertices, dtype=np.float64)
    nx, ny = V.shape[:2]
    left = V[:, :, 3] - V[:, :, 0]                     # edge 1 -> 4 of each element
    right = V[-1:, :, 2] - V[-1:, :, 1]                # edge 2 -> 3 of the last column
    tx = np.concatenate([left, right], axis=0)
    n1 = np.stack([tx[..., 1], -tx[..., 0]], axis=-1)
    bottom = V[:, :, 1] - V[:, :, 0]                   # edge 1 -> 2
    top = V[:, -1:, 2] - V[:, -1:, 3]                  # edge 4 -> 3 of the last row
    ty = np.concatenate([bottom, top], axis=1)
    n2 = np.stack([-ty[..., 1], ty[..., 0]], axis=-1)
    n1 /= np.linalg.norm(n1, axis=-1, keepdims=True)
    n2 /= np.linalg.norm(n2, axis=-1, keepdims=True)
    return np.asfortranarray(n1), np.asfortranarray(n2)


def interp_face_(fdelta: np.ndarray, f: np.ndarray, ll, lr) -> None:
    """interp_face!(fδ, f, ll, lr) (src/interpolate.jl:1-10): fδ[.., 0] = f·ll,
    fδ[.., 1] = f·lr, row by row for a matrix f, evaluated on the GPU."""
    f2 = _f64(np.atleast_2d(f))
    n, npts = f2.shape
    out = np.zeros((n, 2), order="F")
    check(L.lib().frgpu_interp_face(dptr(f2), n, npts, dptr(_f64(ll)), dptr(_f64(lr)), dptr(out)))
    if np.ndim(f) == 1:
        fdelta[0], fdelta[1] = out[0, 0], out[0, 1]
    else:
        fdelta[...] = out


def poly_derivative_(df: np.ndarray, f: np.ndarray, pdm) -> None:
    """poly_derivative!(df, f, pdm) (src/derivative.jl:1-10): df[m] = f·pdm[m, :]
    (row by row for a matrix f), evaluated on the GPU."""
    f2 = _f64(np.atleast_2d(f))
    n, npts = f2.shape
    if np.shape(pdm) != (npts, npts):
        raise ValueError("poly_derivative_: pdm must be np x np with np = len(f)")
    out = np.zeros((n, npts), order="F")
    check(L.lib().frgpu_poly_derivative(dptr(f2), n, npts, dptr(_f64(pdm)), dptr(out)))
    if np.ndim(f) == 1:
        df[...] = out[0]
    else:
        df[...] = out


def shock_detector(Se: float, deg: int, S0: float | None = None, kappa: float = 4.0) -> bool:
    """shock_detector(Se, deg, S0 = -3 log10(deg), κ = 4) (src/dissipation.jl:13-23)."""
    if S0 is None:
        S0 = -3.0 * math.log10(deg)
    if Se < S0 - kappa:
        sigma = 1.0
    elif S0 - kappa <= Se < S0 + kappa:
        sigma = 0.5 * (1.0 - math.sin(0.5 * math.pi * (Se - S0) / kappa))
    else:
        sigma = 0.0
    return sigma < 0.99


def modal_filter_(uh: np.ndarray, lam: float, filter: str = "l2") -> None:
    """KitBase modal_filter!(û, λ; filter=:l2) on a flat modal vector, as called at
    example/shock-vortex.jl:316: û[q] /= 1 + λ q²(q+1)² (q = 0-based mode)."""
    if filter != "l2":
        raise NotImplementedError("only the :l2 filter is on the accelerated path")
    q = np.arange(len(uh), dtype=np.float64)
    uh /= 1.0 + lam * (q + 1) ** 2 * q ** 2


def L1_error(u, ue, dx):
    """src/tools.jl:43-45"""
    return float(np.sum(np.abs(np.asarray(u) - np.asarray(ue)) * dx))


def L2_error(u, ue, dx):
    """src/tools.jl:47-49 (Δx inside the square)"""
    return float(np.sqrt(np.sum((np.abs(np.asarray(u) - np.asarray(ue)) * dx) ** 2)))


def Linf_error(u, ue, dx):
    """src/tools.jl:51-53"""
    return float(np.max(np.abs(np.asarray(u) - np.asarray(ue)) * dx))


def quadrature_L2_error(u, ue, dx, dy, w1):
    """L2 norm of u - ue over a uniform 2D mesh by the solution points' Gauss
    quadrature: sqrt(sum_e sum_kl w_k w_l (dx dy / 4) |u - ue|^2), for arrays
    u[i, j, k, l] (one variable) of the reference layout; w1 are the 1D
    Gauss-Legendre weights on [-1, 1]."""
    e = np.asarray(u, dtype=np.float64) - np.asarray(ue, dtype=np.float64)
    W = np.outer(w1, w1) * (dx * dy / 4.0)
    return float(np.sqrt(np.einsum("ijkl,kl->", e * e, W)))


def _lagrange_rows(nodes, x):
    """rows[a, b] = l_b(x_a): the Lagrange basis of `nodes` at the points x."""
    nodes = np.asarray(nodes, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    rows = np.ones((len(x), len(nodes)))
    for b in range(len(nodes)):
        for m in range(len(nodes)):
            if m != b:
                rows[:, b] *= (x - nodes[m]) / (nodes[b] - nodes[m])
    return rows


def refined_at_coarse_points(u_fine, xpl):
    """Values at the solution points of a uniform 2D mesh of a solution computed
    on the mesh refined twice in each direction (fine element 2i + a, 2j + b
    inside coarse element i, j).  u_fine[I, J, k, l, m] in the reference layout;
    xpl are the solution points on [-1, 1] of both meshes.  Coarse point r lies in
    the fine element a = (r > 0) at the fine coordinate 2r + 1 - 2a, where the
    fine element's Lagrange interpolant is evaluated.  Returns u[i, j, k, l, m]."""
    xpl = np.asarray(xpl, dtype=np.float64)
    nxf, nyf, npk, npl, nv = u_fine.shape
    if nxf % 2 or nyf % 2:
        raise ValueError("the fine mesh must have an even number of elements in each direction")
    side = (xpl > 0).astype(int)
    L = _lagrange_rows(xpl, 2 * xpl + 1 - 2 * side)
    uf = np.asarray(u_fine, dtype=np.float64).reshape(2, nxf // 2, 2, nyf // 2, npk, npl, nv, order="F")
    out = np.zeros((nxf // 2, nyf // 2, npk, npl, nv), order="F")
    for k in range(npk):
        for l in range(npl):
            out[:, :, k, l, :] = np.einsum("K,L,IJKLm->IJm", L[k], L[l], uf[side[k], :, side[l]])
    return out


def fma_peak(kind: str = "fp64") -> float:
    """Measured fused multiply-add throughput of the current GPU in FLOP/s (an FMA
    counts 2): "fp64", "fp32" or "fp32x2" (packed pairs)."""
    out = C.c_double()
    check(L.lib().frgpu_fma_peak({"fp64": 0, "fp32": 1, "fp32x2": 2}[kind], C.byref(out)))
    return out.value


# ---------------------------------------------------------------- problems
class ODEProblem:
    """The object FRAdvectionProblem / FREulerProblem return (an ODEProblem of
    rhs!(du, u, p, t) over u0 and tspan); ``p`` is the device-resident problem."""

    def __init__(self, space, desc: L.ProblemDesc, u0, tspan, shape, keep=()):
        self.space = space
        self.shape = tuple(shape)
        self._keep = keep
        h = C.c_void_p()
        check(L.lib().frgpu_problem_create(space._h, C.byref(desc), C.byref(h)))
        self._h = h
        self.desc = desc
        self.u0 = _f64(u0)
        if self.u0.shape != self.shape:
            raise ValueError(f"u0 has shape {self.u0.shape}, expected {self.shape}")
        self.tspan = (float(tspan[0]), float(tspan[1]))
        self.p = self

    @property
    def ndof(self) -> int:
        return int(L.lib().frgpu_problem_ndof(self._h))

    def f(self, du: np.ndarray, u: np.ndarray, p=None, t: float = 0.0) -> None:
        """rhs!(du, u, p, t): residual of host array u into host array du."""
        uf = _f64(u)
        if uf.shape != self.shape:
            raise ValueError(f"u has shape {uf.shape}, expected {self.shape}")
        if isinstance(du, np.ndarray) and du.dtype == np.float64 and du.flags.f_contiguous and \
                du.shape == self.shape and du.flags.writeable:
            check(L.lib().frgpu_rhs(self._h, dptr(du), dptr(uf), float(t)))  # straight into the caller's array
            return
        out = np.zeros(self.shape, order="F")
        check(L.lib().frgpu_rhs(self._h, dptr(out), dptr(uf), float(t)))
        du[...] = out

    def rhs(self, u: np.ndarray, t: float = 0.0) -> np.ndarray:
        du = np.zeros(self.shape, order="F")
        self.f(du, u, self, t)
        return du

    def set_metric(self, iJ, n1=None, n2=None, Ji=None) -> None:
        """Per-point inverse Jacobian (FRPSpace2D's iJ[i, j][k, l],
        src/struct.jl:135-158) as an array [nx, ny, np, np, 2, 2], and optionally
        the unit normals of the x faces n1[nx+1, ny, 2] and the y faces
        n2[nx, ny+1, 2] (straight-sided quadrilaterals, dev/parallelogram.jl:115-160);
        with the normals, optionally the face Jacobians Ji[nx, ny, 4, np, 2, 2]
        (FRPSpace2D's Ji, src/struct.jl:145-158; quad_face_jacobians) for the
        face-Jacobian interface-flux scaling of dev/cylinder2.jl:147-150;
        None returns to the uniform rectangles."""
        if iJ is None:
            check(L.lib().frgpu_problem_set_metric(self._h, None, None, None))
            return
        a = np.asfortranarray(np.asarray(iJ, dtype=np.float64))
        if a.shape != tuple(self.shape[:4]) + (2, 2):
            raise ValueError("iJ must have shape (nx, ny, np, np, 2, 2)")
        if n1 is None:
            check(L.lib().frgpu_problem_set_metric(self._h, dptr(a), None, None))
            return
        nx, ny = self.shape[0], self.shape[1]
        b1 = np.asfortranarray(np.asarray(n1, dtype=np.float64))
        b2 = np.asfortranarray(np.asarray(n2, dtype=np.float64))
        if b1.shape != (nx + 1, ny, 2) or b2.shape != (nx, ny + 1, 2):
            raise ValueError("face normals must have shapes (nx+1, ny, 2) and (nx, ny+1, 2)")
        check(L.lib().frgpu_problem_set_metric(self._h, dptr(a), dptr(b1), dptr(b2)))
        if Ji is not None:
            c = np.asfortranarray(np.asarray(Ji, dtype=np.float64))
            if c.shape != (nx, ny, 4, self.shape[2], 2, 2):
                raise ValueError("Ji must have shape (nx, ny, 4, np, 2, 2)")
            self._keep_ji = c
            check(L.lib().frgpu_problem_set_face_jacobians(self._h, dptr(c), dptr(b1), dptr(b2)))

    def set_flux_dissipation(self, c: float) -> None:
        """Dissipation coefficient of flux="central" (dev/curve_euler.jl's 40 dt)."""
        check(L.lib().frgpu_problem_set_flux_dissipation(self._h, float(c)))

    def set_option(self, option: int, value: int) -> None:
        """Kernel choice for measurements (frgpu_problem_set_option), e.g.
        ``set_option(L.OPT_BGK_TENSOR, 0)`` for the CUDA-core BGK transport, 2 for
        the tcgen05 form of the tensor-core product (1, the default, is mma.sync)."""
        check(L.lib().frgpu_problem_set_option(self._h, int(option), int(value)))

    def __del__(self):
        if getattr(self, "_h", None) is not None and L._lib is not None:
            L._lib.frgpu_problem_destroy(self._h)
            self._h = None


def _desc(equation, flux=L.FLUX_ROE, precision="fp64", bcs=(L.BC_PERIODIC,) * 4, a=1.0, gamma=1.4, tau=1.0,
          fixed_states=None, eps_interior=1e-8, eps_periodic=1e-6):
    d = L.ProblemDesc()
    d.equation, d.flux, d.precision = equation, flux, _PREC[precision]
    for s in range(4):
        d.bc[s] = bcs[s]
    if fixed_states is not None:
        for s in range(4):
            if fixed_states[s] is not None:
                for m in range(len(fixed_states[s])):
                    d.fixed_state[s][m] = float(fixed_states[s][m])
    d.a, d.gamma, d.tau = float(a), float(gamma), float(tau)
    d.eps_interior, d.eps_periodic = eps_interior, eps_periodic
    return d


def FRAdvectionProblem(u, tspan, ps: FRPSpace1D, a, bc="period", precision="fp64") -> ODEProblem:
    """FRAdvectionProblem(u, tspan, ps, a, bc) (src/Equation/eq_advection.jl:1-26)."""
    d = _desc(L.ADVECTION, precision=precision, bcs=(_BC[str(bc)],) * 4, a=a)
    return ODEProblem(ps, d, u, tspan, (ps.nx, ps.np))


def FRBurgersProblem(u, tspan, ps: FRPSpace1D, bc="period", precision="fp64") -> ODEProblem:
    """Inviscid Burgers u_t + (u²/2)_x = 0 with the scalar machinery of
    eq_advection.jl (Roe flux, same epsilons)."""
    d = _desc(L.BURGERS, precision=precision, bcs=(_BC[str(bc)],) * 4)
    return ODEProblem(ps, d, u, tspan, (ps.nx, ps.np))


def FREulerProblem(u, tspan, ps: FRPSpace1D, gamma, bc="dirichlet", precision="fp64") -> ODEProblem:
    """FREulerProblem(u, tspan, ps, γ, bc) (src/Equation/eq_euler.jl:1-27), HLL flux."""
    d = _desc(L.EULER1D, flux=L.FLUX_HLL, precision=precision, bcs=(_BC[str(bc)],) * 4, gamma=gamma)
    return ODEProblem(ps, d, u, tspan, (ps.nx, ps.np, 3))


def FREuler2DProblem(u, tspan, ps: FRPSpace2D, gamma, flux="hll", bc="period", fixed_states=None,
                     precision="fp64") -> ODEProblem:
    """The 2D Euler ``dudt!`` closure of example/shock-vortex.jl:26-118 as an
    ODEProblem.  ``bc`` is one kind for all sides or (left, right, bottom, top);
    ``fixed_states`` gives the conserved ghost state of each fixed side.
    flux="central" is the dudt! of dev/curve_euler.jl (with set_metric and
    set_flux_dissipation; sides "period" or "dirichlet", the latter keeping the
    elements along it at du = 0)."""
    bcs = (bc,) * 4 if isinstance(bc, str) else tuple(bc)
    d = _desc(L.EULER2D, flux=_FLUX[flux], precision=precision, bcs=tuple(_BC[b] for b in bcs), gamma=gamma,
              fixed_states=fixed_states)
    n = ps.deg + 1
    return ODEProblem(ps, d, u, tspan, (ps.nx, ps.ny, n, n, 4))


def FRBGKProblem(u, tspan, ps: FRPSpace1D, velo, weights, tau, precision="fp64", closure="conserve_prim",
                 a=1.0) -> ODEProblem:
    """The 1D1V BGK ``mol!`` closure of example/bgk_wave.jl:69-129 (kinetic
    upwind flux, Maxwellian relaxation with time tau, periodic).  With
    closure="density" the Maxwellian is that of example/advection_kinetic.jl:
    73-128, prim = [rho, a, 1] from the density alone (the problem that script
    steps with ROCK4)."""
    if closure not in ("conserve_prim", "density"):
        raise ValueError("closure is 'conserve_prim' or 'density'")
    velo = np.ascontiguousarray(velo, dtype=np.float64)
    weights = np.ascontiguousarray(weights, dtype=np.float64)
    d = _desc(L.BGK1D, flux=L.FLUX_UPWIND, precision=precision, tau=tau, a=a)
    d.nvel = len(velo)
    d.velo, d.weights = dptr(velo), dptr(weights)
    prob = ODEProblem(ps, d, u, tspan, (ps.nx, len(velo), ps.np), keep=(velo, weights))
    if closure == "density":
        prob.set_option(L.OPT_BGK_CLOSURE, 1)
    return prob


class SSPRK33:
    """Marker for the three-stage SSP Runge-Kutta method (OrdinaryDiffEq SSPRK33);
    it runs fused into the residual kernels."""


class ExplicitRK:
    """A fixed-step explicit Runge-Kutta method given by its Butcher tableau
    (A strictly lower triangular, weights b); stepped by frgpu_step_erk."""

    def __init__(self, A, b, name: str = "ExplicitRK"):
        self.A = np.ascontiguousarray(np.asarray(A, dtype=np.float64))
        self.b = np.ascontiguousarray(np.asarray(b, dtype=np.float64))
        self.name = name
        s = len(self.b)
        if self.A.shape != (s, s) or np.any(np.triu(self.A) != 0.0):
            raise ValueError("need an explicit s x s tableau (A strictly lower triangular)")

    def __repr__(self):
        return f"{self.name}()"


def Midpoint() -> ExplicitRK:
    """OrdinaryDiffEq Midpoint (explicit midpoint rule), as example/shock-vortex.jl:294 uses it."""
    return ExplicitRK([[0, 0], [0.5, 0]], [0, 1], "Midpoint")


def Heun() -> ExplicitRK:
    return ExplicitRK([[0, 0], [1, 0]], [0.5, 0.5], "Heun")


def Ralston() -> ExplicitRK:
    return ExplicitRK([[0, 0], [2 / 3, 0]], [0.25, 0.75], "Ralston")


def SSPRK22() -> ExplicitRK:
    return ExplicitRK([[0, 0], [1, 0]], [0.5, 0.5], "SSPRK22")


def RK4() -> ExplicitRK:
    return ExplicitRK([[0, 0, 0, 0], [0.5, 0, 0, 0], [0, 0.5, 0, 0], [0, 0, 1, 0]],
                      [1 / 6, 1 / 3, 1 / 3, 1 / 6], "RK4")


def Tsit5() -> ExplicitRK:
    """Tsitouras 5(4) pair (Ch. Tsitouras, Comput. Math. Appl. 62 (2011) 770-775),
    fifth-order weights, fixed dt (adaptive=false): the last row of A is b (FSAL)."""
    a = np.zeros((7, 7))
    a[1, 0] = 0.161
    a[2, :2] = [-0.008480655492356989, 0.335480655492357]
    a[3, :3] = [2.897153057105493, -6.359448489975075, 4.3622954328695815]
    a[4, :4] = [5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525]
    a[5, :5] = [5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383]
    a[6, :6] = [0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081,
                2.324710524099774]
    return ExplicitRK(a, np.append(a[6, :6], 0.0), "Tsit5")


class Stabilized:
    """A stabilised explicit method: a three-term recurrence of m stages and an
    explicit finishing tableau, stepped by frgpu_step_rock (the structure of
    OrdinaryDiffEq's ROCK2/ROCK4, example/advection_kinetic.jl:133-146, and of
    the Runge-Kutta-Chebyshev methods).  ``coefficients(z)`` maps z = dt * rho,
    rho the spectral-radius estimate taken before every step (as the ROCK
    methods do), to (alpha, beta, mu, delta, A, b) of the increment form
    D_j = alpha_j D_{j-1} + beta_j D_{j-2} + dt (mu_j f(u + D_{j-1}) + delta_j f(u))."""

    def __init__(self, coefficients, name: str = "Stabilized", maxiter: int = 50):
        self.coefficients = coefficients
        self.name = name
        self.maxiter = int(maxiter)

    def __repr__(self):
        return f"{self.name}()"


def rkc2_coefficients(s: int, eps: float = 2 / 13):
    """Second-order Runge-Kutta-Chebyshev method of s >= 2 stages with damping
    eps (B. P. Sommeijer, L. F. Shampine, J. G. Verwer, J. Comput. Appl. Math. 88
    (1997) 315-326): with w0 = 1 + eps/s^2, w1 = T_s'(w0)/T_s''(w0), b_j =
    T_j''(w0)/T_j'(w0)^2 (b_0 = b_1 = b_2), a_j = 1 - b_j T_j(w0):
    Y_1 = u + mu~_1 dt f(u), mu~_1 = b_1 w1, and for j >= 2
    Y_j = (1 - mu_j - nu_j) u + mu_j Y_{j-1} + nu_j Y_{j-2} + mu~_j dt f(Y_{j-1})
          + gamma~_j dt f(u),
    mu_j = 2 b_j w0 / b_{j-1}, nu_j = -b_j / b_{j-2}, mu~_j = 2 b_j w1 / b_{j-1},
    gamma~_j = -a_{j-1} mu~_j.  Returns (alpha, beta, mu, delta) of the increment
    form and the real stability bound (w0 + 1) T_s''(w0) / T_s'(w0)."""
    if s < 2:
        raise ValueError("RKC2 needs s >= 2 stages")
    w0 = 1.0 + eps / (s * s)
    T = np.zeros(s + 1)
    dT = np.zeros(s + 1)
    d2T = np.zeros(s + 1)
    T[0], T[1], dT[1] = 1.0, w0, 1.0
    for j in range(2, s + 1):
        T[j] = 2 * w0 * T[j - 1] - T[j - 2]
        dT[j] = 2 * T[j - 1] + 2 * w0 * dT[j - 1] - dT[j - 2]
        d2T[j] = 4 * dT[j - 1] + 2 * w0 * d2T[j - 1] - d2T[j - 2]
    w1 = dT[s] / d2T[s]
    b = np.zeros(s + 1)
    b[2:] = d2T[2:] / dT[2:] ** 2
    b[0] = b[1] = b[2]
    a = 1.0 - b * T
    alpha, beta, mu, delta = (np.zeros(s) for _ in range(4))
    mu[0] = b[1] * w1
    for j in range(2, s + 1):
        alpha[j - 1] = 2 * b[j] * w0 / b[j - 1]
        beta[j - 1] = -b[j] / b[j - 2]
        mu[j - 1] = 2 * b[j] * w1 / b[j - 1]
        delta[j - 1] = -a[j - 1] * mu[j - 1]
    return alpha, beta, mu, delta, (w0 + 1) * d2T[s] / dT[s]


def RKC2(eps: float = 2 / 13, smax: int = 4096, maxiter: int = 50) -> Stabilized:
    """RKC2 with the fewest stages s >= 2 (s = 2, then max(s + 1, floor(1.1 s)),
    at most smax) whose stability bound covers dt * rho (rho from the power
    method, which includes the 1.2 safety factor).  Integrator.step runs it with
    frgpu_step_rkc2, which makes the same choices in one call per n steps."""
    cache = {}

    def coefficients(z):
        s = 2
        while True:
            if s not in cache:
                cache[s] = rkc2_coefficients(s, eps)
            if cache[s][4] >= z or s >= smax:
                break
            s = min(smax, max(s + 1, int(s * 1.1)))
        if cache[s][4] < z:
            raise ValueError(f"dt * rho = {z:.4g} needs more than {smax} RKC2 stages")
        al, be, mu, de, _ = cache[s]
        return al, be, mu, de, None, None

    alg = Stabilized(coefficients, "RKC2", maxiter)
    alg.rkc2 = (float(eps), int(smax))
    return alg


def ROCK(select, name: str = "ROCK", maxiter: int = 50) -> Stabilized:
    """A ROCK2/ROCK4-type method from the caller's tables: ``select(z)`` returns
    (mu[m], kappa[m], A, b) for z = dt * rho: the recurrence Y_1 = u + dt mu_1 f(u),
    Y_j = dt mu_j f(Y_{j-1}) + (1 + kappa_j) Y_{j-1} - kappa_j Y_{j-2} (kappa_1
    unused) and the finishing procedure (A, b) of the chosen degree.  For ROCK4
    these are OrdinaryDiffEq's tables (the recurrence coefficients recf of the
    degree chosen for z and its finishing procedure fpa, fpb), which stay with
    the caller."""

    def coefficients(z):
        mu, kappa, A, b = select(z)
        mu = np.asarray(mu, dtype=np.float64)
        kappa = np.asarray(kappa, dtype=np.float64)
        alpha, beta = 1.0 + kappa, -kappa
        alpha[0] = beta[0] = 0.0
        return alpha, beta, mu, np.zeros_like(mu), A, b

    return Stabilized(coefficients, name, maxiter)


class Integrator:
    """Device-resident integrator: ``itg.u`` reads the state back, ``step_(itg)``
    advances one step of ``dt`` on the GPU (OrdinaryDiffEq's init/step! API)."""

    def __init__(self, prob: ODEProblem, dt: float, alg=None):
        self.prob = prob
        self.dt = float(dt)
        self.t = prob.tspan[0]
        self.alg = alg if isinstance(alg, (ExplicitRK, Stabilized)) else None
        self.stages = []  # stabilised methods: recurrence stages taken per step
        check(L.lib().frgpu_state_upload(prob._h, dptr(prob.u0)))

    @property
    def u(self) -> np.ndarray:
        out = np.zeros(self.prob.shape, order="F")
        check(L.lib().frgpu_state_download(self.prob._h, dptr(out)))
        return out

    def read_u(self, out: np.ndarray) -> np.ndarray:
        """Download the state into a caller-owned FP64 array of the host layout
        (for example page-locked memory, which the copy engine reads and
        writes directly)."""
        if out.shape != self.prob.shape or out.dtype != np.float64 or not out.flags.f_contiguous:
            raise ValueError("read_u needs an F-contiguous float64 array of the state's shape")
        check(L.lib().frgpu_state_download(self.prob._h, dptr(out)))
        return out

    @u.setter
    def u(self, value) -> None:
        v = _f64(value)
        if v.shape != self.prob.shape:
            raise ValueError("state shape mismatch")
        check(L.lib().frgpu_state_upload(self.prob._h, dptr(v)))

    def step(self, n: int = 1, dt: float | None = None) -> None:
        dt = self.dt if dt is None else float(dt)
        if self.alg is None:
            check(L.lib().frgpu_step_ssprk3(self.prob._h, dt, int(n)))
        elif isinstance(self.alg, Stabilized) and getattr(self.alg, "rkc2", None) is not None:
            eps, smax = self.alg.rkc2
            st = np.zeros(max(int(n), 1), dtype=np.int32)
            check(L.lib().frgpu_step_rkc2(self.prob._h, dt, int(n), eps, smax, self.alg.maxiter,
                                          st.ctypes.data_as(L._I)))
            self.stages.extend(int(x) for x in st[:int(n)])
        elif isinstance(self.alg, Stabilized):
            for _ in range(int(n)):
                rho, _ = self.spectral_radius(self.alg.maxiter)
                self.step_rock(*self.alg.coefficients(dt * rho), dt=dt)
                self.t -= dt
        else:
            a = self.alg
            check(L.lib().frgpu_step_erk(self.prob._h, len(a.b), dptr(a.A), dptr(a.b), dt, int(n)))
        self.t += n * dt

    def spectral_radius(self, maxiter: int = 50):
        """(rho, iterations) of frgpu_spectral_radius at the current state: the
        nonlinear power-method estimate of the residual Jacobian's spectral
        radius, times 1.2; iterations < 0 when it did not settle."""
        rho = C.c_double(0.0)
        it = C.c_int(0)
        check(L.lib().frgpu_spectral_radius(self.prob._h, int(maxiter), C.byref(rho), C.byref(it)))
        return rho.value, it.value

    def step_rock(self, alpha, beta, mu, delta, A=None, b=None, n: int = 1, dt: float | None = None) -> None:
        """n stabilised steps with fixed coefficients (frgpu_step_rock)."""
        dt = self.dt if dt is None else float(dt)
        co = [np.ascontiguousarray(x, dtype=np.float64) for x in (alpha, beta, mu, delta)]
        m = len(co[0])
        if any(len(x) != m for x in co):
            raise ValueError("alpha, beta, mu, delta need the same length")
        if b is None:
            sf, Ap, bp = 0, None, None
        else:
            A = np.ascontiguousarray(A, dtype=np.float64)
            b = np.ascontiguousarray(b, dtype=np.float64)
            sf = len(b)
            if A.shape != (sf, sf):
                raise ValueError("the finishing tableau needs A of shape (len(b), len(b))")
            Ap, bp = dptr(A), dptr(b)
        check(L.lib().frgpu_step_rock(self.prob._h, m, *(dptr(x) for x in co), sf, Ap, bp, dt, int(n)))
        self.stages.append(m)
        self.t += n * dt

    def step_async(self, n: int = 1, dt: float | None = None) -> None:
        """Queue n SSPRK3 steps and return without waiting; ``synchronize()``
        (or the next synchronous call) reports their device status."""
        if self.alg is not None:
            raise NotImplementedError("step_async queues the fused SSPRK3 step")
        dt = self.dt if dt is None else float(dt)
        check(L.lib().frgpu_step_ssprk3_async(self.prob._h, dt, int(n)))
        self.t += n * dt

    def set_filter(self, indicator="plain", lam=5e-4, S0=None, kappa=9.0) -> None:
        """Post-step troubled-cell indicator + :l2 modal filter (shock-vortex.jl:308-321)."""
        deg = self.prob.space.deg
        if S0 is None:
            S0 = -3.0 * math.log10(deg)
        check(L.lib().frgpu_set_filter(self.prob._h, _IND[indicator], float(lam), float(S0), float(kappa)))

    def modal_filter(self, indicator="plain", lam=5e-4, S0=None, kappa=9.0) -> int:
        deg = self.prob.space.deg
        if S0 is None:
            S0 = -3.0 * math.log10(deg)
        n = C.c_int(0)
        check(L.lib().frgpu_modal_filter(self.prob._h, _IND[indicator], float(lam), float(S0), float(kappa),
                                         C.byref(n)))
        return n.value

    def positive_limiter(self, weights=None, t0: float = 1.0) -> int:
        """positive_limiter (src/dissipation.jl:38-216) on every element, once
        now; returns the number of elements it scaled.  weights: element
        quadrature weights (Euler forms: summing to 1), default the space's
        Gauss weights so normalised."""
        n = C.c_int(0)
        w = None if weights is None else _f64(np.asarray(weights).ravel(order="F"))
        check(L.lib().frgpu_positive_limiter(self.prob._h, None if w is None else dptr(w), float(t0), C.byref(n)))
        return n.value

    def set_limiter(self, on: bool = True, weights=None, t0: float = 1.0) -> None:
        """Run the limiter before every step (example/shock-vortex.jl:297-303)."""
        w = None if weights is None else _f64(np.asarray(weights).ravel(order="F"))
        check(L.lib().frgpu_set_limiter(self.prob._h, int(bool(on)), None if w is None else dptr(w), float(t0)))

    def troubled(self) -> np.ndarray:
        sp = self.prob.space
        ne = sp.nx * getattr(sp, "ny", 1)
        flags = np.zeros(ne, dtype=np.int32)
        check(L.lib().frgpu_troubled_flags(self.prob._h, flags.ctypes.data_as(L._I), ne))
        return flags

    def cfl_dt(self, cfl: float) -> float:
        dt = C.c_double()
        check(L.lib().frgpu_cfl_dt(self.prob._h, float(cfl), C.byref(dt)))
        return dt.value

    def reduce(self):
        """FP64 conserved sums (per variable) and the maximum wave speed."""
        sums = np.zeros(4)
        ms = C.c_double()
        check(L.lib().frgpu_reduce(self.prob._h, dptr(sums), C.byref(ms)))
        return sums, ms.value

    def step_reduce(self, n: int = 1, dt: float | None = None):
        """n SSPRK3 steps, then the FP64 conserved sums and the maximum wave
        speed, with one synchronisation (frgpu_step_ssprk3_reduce)."""
        if self.alg is not None:
            raise NotImplementedError("step_reduce runs the fused SSPRK3 step")
        dt = self.dt if dt is None else float(dt)
        sums = np.zeros(4)
        ms = C.c_double()
        check(L.lib().frgpu_step_ssprk3_reduce(self.prob._h, dt, int(n), dptr(sums), C.byref(ms)))
        self.t += n * dt
        return sums, ms.value

    def stream(self) -> int:
        s = C.c_void_p()
        check(L.lib().frgpu_problem_stream(self.prob._h, C.byref(s)))
        return s.value or 0

    def launches(self) -> int:
        return int(L.lib().frgpu_problem_launches(self.prob._h))

    def synchronize(self) -> None:
        check(L.lib().frgpu_synchronize(self.prob._h))


def init(prob: ODEProblem, alg=None, *, dt: float, adaptive: bool = False, **kwargs) -> Integrator:
    """init(prob, alg; adaptive=false, dt) (OrdinaryDiffEq): SSPRK33 (default,
    fused into the residual kernels), an explicit tableau (Midpoint(), RK4(),
    Tsit5(), ... or ExplicitRK(A, b)) or a stabilised method (RKC2(), or ROCK(...)
    with the caller's ROCK4 tables)."""
    if alg is not None and not isinstance(alg, (SSPRK33, ExplicitRK, Stabilized)) and alg is not SSPRK33:
        raise NotImplementedError("the device integrator implements SSPRK33, explicit Runge-Kutta tableaux and "
                                  "stabilised (ROCK / RKC) methods")
    if adaptive:
        raise NotImplementedError("fixed time steps only (adaptive=false)")
    return Integrator(prob, dt, alg)


def step_(itg: Integrator, n: int = 1) -> None:
    """step!(itg)"""
    itg.step(n)


def solve(prob: ODEProblem, alg=None, *, dt: float, adaptive: bool = False, **kwargs) -> np.ndarray:
    """solve(prob, SSPRK33(); adaptive=false, dt): full steps of dt to tspan[1],
    the last one shortened to land on it.  Returns the final state."""
    itg = init(prob, alg, dt=dt, adaptive=adaptive)
    span = prob.tspan[1] - prob.tspan[0]
    n = int(math.floor(span / dt + 1e-9))
    if n:
        itg.step(n)
    rest = span - n * dt
    if rest > 1e-12 * max(1.0, abs(span)):
        itg.step(1, rest)
    return itg.u
