"""ctypes front end of the CPU FP64 oracle (fr_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU legs of ``bench.py``.  The product library never imports it.

The oracle restates FluxReconstruction.jl's residuals (src/Equation/*.jl,
example/shock-vortex.jl:26-118, example/bgk_wave.jl:69-129) and setup math
(src/Polynomial/*.jl, src/Transform/transform.jl) in C; this module builds and
loads it and offers numpy-level helpers that mirror the reference's calls.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "fr_oracle.c")

ADVECTION, BURGERS, EULER1D, EULER2D, BGK1D = 0, 1, 2, 3, 4
FLUX_ROE, FLUX_LF, FLUX_HLL, FLUX_UPWIND, FLUX_CENTRAL = 0, 1, 2, 3, 4
BC_PERIODIC, BC_COPY, BC_FIXED, BC_DIRICHLET = 0, 1, 2, 3


def build(force: bool = False) -> str:
    """Compile fr_oracle.c into liboracle.so (gcc, OpenMP, no FMA contraction)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(SRC):
        cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               "-o", LIB_PATH, SRC, "-lm"]
        subprocess.check_call(cmd)
    return LIB_PATH


_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)


class Cfg(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("flux", C.c_int),
        ("nx", C.c_int), ("ny", C.c_int), ("np", C.c_int), ("nvel", C.c_int),
        ("a", C.c_double), ("gamma", C.c_double), ("tau", C.c_double),
        ("bc", C.c_int * 4),
        ("fixed_state", (C.c_double * 4) * 4),
        ("eps_interior", C.c_double), ("eps_periodic", C.c_double),
        ("J", _D),
        ("iJx", C.c_double), ("iJy", C.c_double),
        ("ll", _D), ("lr", _D), ("lpdm", _D), ("dgl", _D), ("dgr", _D),
        ("velo", _D), ("weights", _D),
        ("iJ", _D), ("n1", _D), ("n2", _D), ("Ji", _D),
        ("bgk_closure", C.c_int),
        ("flux_c", C.c_double),
        ("ghosts_per_step", C.c_int),
        ("ghost_src", _D),
    ]


_lib = None


class TriCfg(C.Structure):
    _fields_ = [("ncell", C.c_int), ("deg", C.c_int), ("np", C.c_int), ("nfp", C.c_int), ("a", C.c_double),
                ("dl", _D), ("lf", _D), ("phi", _D), ("J", _D), ("iJ", _D),
                ("nbc", _I), ("nbf", _I), ("nbk", _I), ("ctype", _I)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        sig = {
            "fro_gauss_legendre": (None, [C.c_int, _D, _D]),
            "fro_legendre_p": (C.c_double, [C.c_int, C.c_double]),
            "fro_dlegendre": (C.c_double, [C.c_int, C.c_double]),
            "fro_dcorrection": (None, [C.c_int, C.c_int, _D, C.c_int, _D, _D]),
            "fro_lagrange_point": (None, [_D, C.c_int, C.c_double, _D]),
            "fro_dlagrange": (None, [_D, C.c_int, _D]),
            "fro_jacobi_p": (C.c_double, [C.c_double, C.c_double, C.c_double, C.c_int]),
            "fro_djacobi_p": (C.c_double, [C.c_double, C.c_double, C.c_double, C.c_int]),
            "fro_vandermonde_1d": (None, [C.c_int, _D, C.c_int, _D]),
            "fro_dvandermonde_1d": (None, [C.c_int, _D, C.c_int, _D]),
            "fro_vandermonde_quad": (None, [C.c_int, _D, _D, C.c_int, _D]),
            "fro_inverse": (C.c_int, [C.c_int, _D, _D]),
            "fro_shock_detector": (C.c_int, [C.c_double, C.c_int, C.c_double, C.c_double]),
            "fro_ndof": (C.c_long, [C.POINTER(Cfg)]),
            "fro_rhs": (None, [C.POINTER(Cfg), _D, _D]),
            "fro_ssprk3": (None, [C.POINTER(Cfg), _D, C.c_double, C.c_int, _D]),
            "fro_erk": (None, [C.POINTER(Cfg), _D, C.c_double, C.c_int, C.c_int, _D, _D, _D]),
            "fro_rock": (None, [C.POINTER(Cfg), _D, C.c_double, C.c_int, C.c_int, _D, _D, _D, _D, C.c_int, _D, _D,
                                _D]),
            "fro_spectral_radius": (C.c_int, [C.POINTER(Cfg), _D, C.c_int, _D, C.POINTER(C.c_int), _D, _D]),
            "fro_ssprk3_filtered": (None, [C.POINTER(Cfg), _D, C.c_double, C.c_int, _D, _D, _D, C.c_double,
                                           C.c_double, C.c_double]),
            "fro_filter2d": (C.c_int, [C.POINTER(Cfg), _D, _D, _D, C.c_double, C.c_double,
                                       C.c_double, _I]),
            "fro_filter1d": (C.c_int, [C.POINTER(Cfg), _D, C.c_int, _D, _D, C.c_double, _I]),
            "fro_modal_features2d": (None, [C.POINTER(Cfg), _D, _D, _D]),
            "fro_modal_features1d": (None, [C.POINTER(Cfg), _D, _D, _D]),
            "fro_positive_limiter2d": (C.c_int, [C.POINTER(Cfg), _D, _D, C.c_double]),
            "fro_positive_limiter1d": (C.c_int, [C.POINTER(Cfg), _D, _D, C.c_double]),
            "fro_positive_limiter_scalar": (C.c_int, [C.POINTER(Cfg), _D, _D, C.c_double]),
            "fro_conserved_sums2d": (None, [C.POINTER(Cfg), _D, _D, _D]),
            "fro_max_speed2d": (C.c_double, [C.POINTER(Cfg), _D]),
            "fro_L1_error": (C.c_double, [_D, _D, C.c_long, C.c_double]),
            "fro_L2_error": (C.c_double, [_D, _D, C.c_long, C.c_double]),
            "fro_Linf_error": (C.c_double, [_D, _D, C.c_long, C.c_double]),
            "fro_prim_conserve2d": (None, [_D, C.c_double, _D]),
            "fro_conserve_prim2d": (None, [_D, C.c_double, _D]),
            "fro_prim_conserve1d": (None, [_D, C.c_double, _D]),
            "fro_flux_hll2d": (None, [_D, _D, C.c_double, C.c_int, _D]),
            "fro_flux_lf2d": (None, [_D, _D, C.c_double, C.c_int, _D]),
            "fro_flux_hll1d": (None, [_D, _D, C.c_double, _D]),
            "fro_ib_rh": (None, [C.c_double, C.c_double, _D, _D]),
            "fro_mlp_forward": (None, [_D, _D, C.c_int, C.c_int, C.c_int, _D]),
            "fro_mlp_loss_grad": (C.c_double, [_D, _D, _D, C.c_int, C.c_int, C.c_int, _D]),
            "fro_vandermonde_tri": (None, [C.c_int, _D, _D, C.c_int, _D]),
            "fro_dvandermonde_tri": (None, [C.c_int, _D, _D, C.c_int, _D, _D]),
            "fro_tri_rhs": (None, [C.POINTER(TriCfg), _D, _D]),
            "fro_tri_erk": (None, [C.POINTER(TriCfg), _D, C.c_double, C.c_int, C.c_int, _D, _D, _D]),
            "fro_set_threads": (None, [C.c_int]),
            "fro_get_threads": (C.c_int, []),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and (a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"])
    return a.ctypes.data_as(_D)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel(order="F"))


# ---------------------------------------------------------------- setup math
def gauss_legendre(n: int):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().fro_gauss_legendre(n, _p(x), _p(w))
    return x, w


def legendre_point(deg: int) -> np.ndarray:
    return gauss_legendre(deg + 1)[0]


def dcorrection(kind: str, deg: int, x) -> tuple[np.ndarray, np.ndarray]:
    k = {"radau": 0, "sd": 1, "huynh": 2}[kind]
    x = _f64(x)
    dgl = np.zeros_like(x)
    dgr = np.zeros_like(x)
    lib().fro_dcorrection(k, deg, _p(x), len(x), _p(dgl), _p(dgr))
    return dgl, dgr


def lagrange_point(sp, x: float) -> np.ndarray:
    sp = _f64(sp)
    out = np.zeros_like(sp)
    lib().fro_lagrange_point(_p(sp), len(sp), float(x), _p(out))
    return out


def dlagrange(sp) -> np.ndarray:
    sp = _f64(sp)
    n = len(sp)
    flat = np.zeros(n * n)
    lib().fro_dlagrange(_p(sp), n, _p(flat))
    return flat.reshape((n, n), order="F")


def vandermonde_1d(N: int, r) -> np.ndarray:
    r = _f64(r)
    flat = np.zeros(len(r) * (N + 1))
    lib().fro_vandermonde_1d(N, _p(r), len(r), _p(flat))
    return flat.reshape((len(r), N + 1), order="F")


def dvandermonde_1d(N: int, r) -> np.ndarray:
    r = _f64(r)
    flat = np.zeros(len(r) * (N + 1))
    lib().fro_dvandermonde_1d(N, _p(r), len(r), _p(flat))
    return flat.reshape((len(r), N + 1), order="F")


def vandermonde_quad(N: int, r, s) -> np.ndarray:
    r = _f64(r)
    s = _f64(s)
    n = len(r)
    flat = np.zeros(n * (N + 1) ** 2)
    lib().fro_vandermonde_quad(N, _p(r), _p(s), n, _p(flat))
    return flat.reshape((n, (N + 1) ** 2), order="F")


def inverse(A) -> np.ndarray:
    A = np.asarray(A, dtype=np.float64)
    n = A.shape[0]
    a = _f64(A)
    out = np.zeros(n * n)
    rc = lib().fro_inverse(n, _p(a), _p(out))
    assert rc == 0
    return out.reshape((n, n), order="F")


def shock_detector(Se: float, deg: int, S0: float | None = None, kappa: float = 4.0) -> bool:
    if S0 is None:
        S0 = -3.0 * np.log10(deg)
    return bool(lib().fro_shock_detector(float(Se), deg, float(S0), float(kappa)))


# --------------------------------------------------------------- spaces
class Space1D:
    """Restatement of FRPSpace1D (src/struct.jl:40-85) for the oracle."""

    def __init__(self, x0, x1, nx, deg, correction="radau"):
        self.nx, self.deg, self.np = nx, deg, deg + 1
        dx = (x1 - x0) / nx
        self.dx = np.full(nx, dx)
        self.x = x0 + (np.arange(nx) + 0.5) * dx
        self.J = self.dx / 2
        self.xpl, self.wp = gauss_legendre(deg + 1)
        xi = np.append(self.x - 0.5 * self.dx, self.x[-1] + 0.5 * self.dx[-1])
        # global_sp (src/Geometry/geo_points.jl:8-15) with r_x (geo_transform.jl:7)
        self.xpg = np.array([[((1.0 - r) / 2.0) * xi[i] + ((1.0 + r) / 2.0) * xi[i + 1] for r in self.xpl]
                             for i in range(nx)])
        self.ll = lagrange_point(self.xpl, -1.0)
        self.lr = lagrange_point(self.xpl, 1.0)
        self.dl = dlagrange(self.xpl)
        self.V = vandermonde_1d(deg, self.xpl)
        self.iV = inverse(self.V)
        self.dhl, self.dhr = dcorrection(correction, deg, self.xpl)


class Space2D:
    """Restatement of FRPSpace2D (src/struct.jl:130-242) on uniform
    rectangles: iJ = diag(2/dx, 2/dy), dhl/dhr = dradau (:193)."""

    def __init__(self, x0, x1, nx, y0, y1, ny, deg):
        self.nx, self.ny, self.deg, self.np = nx, ny, deg, deg + 1
        self.dx = (x1 - x0) / nx
        self.dy = (y1 - y0) / ny
        self.iJx = 1.0 / (0.5 * self.dx)
        self.iJy = 1.0 / (0.5 * self.dy)
        self.xpl, w = gauss_legendre(deg + 1)
        self.wp = np.outer(w, w)
        self.ll = lagrange_point(self.xpl, -1.0)
        self.lr = lagrange_point(self.xpl, 1.0)
        self.dl = dlagrange(self.xpl)
        self.dhl, self.dhr = dcorrection("radau", deg, self.xpl)
        n = self.np
        r2 = np.repeat(self.xpl[:, None], n, axis=1)   # r2d[:, j] = r
        s2 = np.repeat(self.xpl[None, :], n, axis=0)   # s2d[i, :] = r
        self.V = vandermonde_quad(deg, r2.ravel(order="F"), s2.ravel(order="F"))
        self.iV = inverse(self.V)
        xc = x0 + (np.arange(nx) + 0.5) * self.dx
        yc = y0 + (np.arange(ny) + 0.5) * self.dy
        # xpg[i, j, k, l, 1:2] (src/struct.jl:161-175) for rectangles
        X = xc[:, None, None, None] + 0.5 * self.dx * self.xpl[None, None, :, None]
        Y = yc[None, :, None, None] + 0.5 * self.dy * self.xpl[None, None, None, :]
        self.xpg = np.stack(np.broadcast_arrays(X, Y), axis=-1)


# --------------------------------------------------------------- residuals
class Problem:
    """Holds an oracle configuration; arrays use the reference's Julia layout
    (numpy arrays with order='F' and the reference's index order)."""

    def __init__(self, kind, space, *, flux=FLUX_ROE, a=1.0, gamma=1.4, tau=1e-2, bc=BC_PERIODIC,
                 bcs=None, fixed_states=None, velo=None, weights=None, eps_interior=1e-8,
                 eps_periodic=1e-6, bgk_closure=0, flux_c=0.0, ghosts_per_step=0):
        c = Cfg()
        c.kind, c.flux = kind, flux
        c.bgk_closure = bgk_closure
        c.flux_c = flux_c
        c.ghosts_per_step = ghosts_per_step
        c.nx = space.nx
        c.ny = getattr(space, "ny", 1)
        c.np = space.np
        c.a, c.gamma, c.tau = a, gamma, tau
        sides = bcs if bcs is not None else [bc] * 4
        for s in range(4):
            c.bc[s] = sides[s]
        if fixed_states is not None:
            for s in range(4):
                for m in range(4):
                    c.fixed_state[s][m] = fixed_states[s][m]
        c.eps_interior, c.eps_periodic = eps_interior, eps_periodic
        self._keep = []

        def arr(x):
            a_ = _f64(x)
            self._keep.append(a_)
            return _p(a_)

        if hasattr(space, "J"):
            c.J = arr(space.J)
        if hasattr(space, "iJx"):
            c.iJx, c.iJy = space.iJx, space.iJy
        c.ll, c.lr = arr(space.ll), arr(space.lr)
        c.lpdm = arr(space.dl)
        c.dgl, c.dgr = arr(space.dhl), arr(space.dhr)
        if velo is not None:
            c.nvel = len(velo)
            c.velo, c.weights = arr(velo), arr(weights)
        self.cfg = c
        self.space = space
        self.kind = kind

    def set_metric(self, iJ, n1=None, n2=None, Ji=None) -> None:
        """2D: per-point inverse Jacobian iJ[nx, ny, np, np, 2, 2] (None: diag(iJx,
        iJy)), and optionally the unit normals of the x faces n1[nx+1, ny, 2] and
        the y faces n2[nx, ny+1, 2] (None: the Cartesian axes), and with them the
        face Jacobians Ji[nx, ny, 4, np, 2, 2] of the cylinder scripts' scaling."""
        self.cfg.iJ = self.cfg.n1 = self.cfg.n2 = self.cfg.Ji = None
        if iJ is None:
            return

        def keep(x):
            a = np.asfortranarray(np.asarray(x, dtype=np.float64))
            self._keep.append(a)
            return a.ctypes.data_as(_D)

        self.cfg.iJ = keep(iJ)
        if n1 is not None:
            self.cfg.n1, self.cfg.n2 = keep(n1), keep(n2)
            if Ji is not None:
                self.cfg.Ji = keep(Ji)

    def shape(self):
        c = self.cfg
        if self.kind in (ADVECTION, BURGERS):
            return (c.nx, c.np)
        if self.kind == EULER1D:
            return (c.nx, c.np, 3)
        if self.kind == EULER2D:
            return (c.nx, c.ny, c.np, c.np, 4)
        return (c.nx, c.nvel, c.np)

    def rhs(self, u: np.ndarray) -> np.ndarray:
        uf = np.asfortranarray(u, dtype=np.float64)
        du = np.zeros(self.shape(), order="F")
        lib().fro_rhs(C.byref(self.cfg), du.ctypes.data_as(_D), uf.ctypes.data_as(_D))
        return du

    def ssprk3(self, u: np.ndarray, dt: float, nsteps: int) -> np.ndarray:
        uf = np.array(u, dtype=np.float64, order="F", copy=True)
        work = np.zeros(2 * uf.size)
        lib().fro_ssprk3(C.byref(self.cfg), uf.ctypes.data_as(_D), float(dt), int(nsteps), _p(work))
        return uf

    def ssprk3_filtered(self, u: np.ndarray, dt: float, nsteps: int, lam: float, S0: float,
                        kappa: float) -> np.ndarray:
        """nsteps of (SSPRK3 step, plain indicator + :l2 filter), the loop of
        example/shock-vortex.jl:294-321 with SSPRK3; 2D Euler."""
        uf = np.array(u, dtype=np.float64, order="F", copy=True)
        work = np.zeros(2 * uf.size)
        V = _f64(self.space.V)
        iV = _f64(self.space.iV)
        lib().fro_ssprk3_filtered(C.byref(self.cfg), uf.ctypes.data_as(_D), float(dt), int(nsteps), _p(work),
                                  _p(V), _p(iV), float(lam), float(S0), float(kappa))
        return uf

    def erk(self, u: np.ndarray, dt: float, nsteps: int, A, b) -> np.ndarray:
        """Fixed-step explicit Runge-Kutta with the Butcher tableau (A, b)."""
        uf = np.array(u, dtype=np.float64, order="F", copy=True)
        A = np.ascontiguousarray(A, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        s = len(b)
        work = np.zeros((s + 1) * uf.size)
        lib().fro_erk(C.byref(self.cfg), uf.ctypes.data_as(_D), float(dt), int(nsteps), s, _p(A), _p(b), _p(work))
        return uf

    def rock(self, u: np.ndarray, dt: float, nsteps: int, alpha, beta, mu, delta, A=None, b=None) -> np.ndarray:
        """Stabilised step: the m-stage recurrence (alpha, beta, mu, delta) in
        increment form and the finishing tableau (A, b) (fro_rock)."""
        uf = np.array(u, dtype=np.float64, order="F", copy=True)
        co = [np.ascontiguousarray(x, dtype=np.float64) for x in (alpha, beta, mu, delta)]
        m = len(co[0])
        A = np.zeros((0, 0)) if A is None else np.ascontiguousarray(A, dtype=np.float64)
        b = np.zeros(0) if b is None else np.ascontiguousarray(b, dtype=np.float64)
        sf = len(b)
        work = np.zeros((7 + sf) * uf.size)
        lib().fro_rock(C.byref(self.cfg), uf.ctypes.data_as(_D), float(dt), int(nsteps), m, *(_p(x) for x in co), sf,
                       _p(A) if sf else None, _p(b) if sf else None, _p(work))
        return uf

    def spectral_radius(self, u: np.ndarray, maxiter: int = 50, direction=None):
        """Nonlinear power-method estimate (fro_spectral_radius): returns
        (rho, iterations, direction); pass direction back to start from it."""
        uf = np.array(u, dtype=np.float64, order="F", copy=True)
        have = C.c_int(0 if direction is None else 1)
        d = np.zeros(uf.size) if direction is None else np.array(direction, dtype=np.float64, copy=True)
        rho = C.c_double(0.0)
        work = np.zeros(3 * uf.size)
        it = lib().fro_spectral_radius(C.byref(self.cfg), uf.ctypes.data_as(_D), int(maxiter), _p(d), C.byref(have),
                                       C.byref(rho), _p(work))
        return rho.value, it, d

    def filter2d(self, u: np.ndarray, lam: float, S0: float, kappa: float):
        uf = np.array(u, dtype=np.float64, order="F", copy=True)
        flags = np.zeros(self.cfg.nx * self.cfg.ny, dtype=np.int32)
        V = _f64(self.space.V)
        iV = _f64(self.space.iV)
        n = lib().fro_filter2d(C.byref(self.cfg), uf.ctypes.data_as(_D), _p(V), _p(iV), lam, S0,
                               kappa, flags.ctypes.data_as(_I))
        return uf, flags.reshape((self.cfg.nx, self.cfg.ny), order="F"), n

    def filter1d(self, u: np.ndarray, nvar: int, lam: float):
        """example/euler_highlevel.jl:37-52 indicator + :l2 filter (1D)."""
        uf = np.array(u, dtype=np.float64, order="F", copy=True)
        flags = np.zeros(self.cfg.nx, dtype=np.int32)
        V = _f64(self.space.V)
        iV = _f64(self.space.iV)
        n = lib().fro_filter1d(C.byref(self.cfg), uf.ctypes.data_as(_D), int(nvar), _p(V), _p(iV), float(lam),
                               flags.ctypes.data_as(_I))
        return uf, flags, n

    def features2d(self, u: np.ndarray) -> np.ndarray:
        uf = np.asfortranarray(u, dtype=np.float64)
        nn = self.cfg.nx * self.cfg.ny
        N = self.cfg.np ** 2
        feat = np.zeros(nn * 2 * N)
        iV = _f64(self.space.iV)
        lib().fro_modal_features2d(C.byref(self.cfg), uf.ctypes.data_as(_D), _p(iV), _p(feat))
        return feat.reshape(nn, 2 * N)

    def features1d(self, u: np.ndarray) -> np.ndarray:
        """Features of the 1D learned indicator (32 per element) of a scalar state u[ne, np]."""
        uf = np.asfortranarray(u, dtype=np.float64)
        feat = np.zeros(self.cfg.nx * 32)
        iV = _f64(self.space.iV)
        lib().fro_modal_features1d(C.byref(self.cfg), uf.ctypes.data_as(_D), _p(iV), _p(feat))
        return feat.reshape(self.cfg.nx, 32)

    def positive_limiter(self, u: np.ndarray, w=None, t0: float = 1.0):
        """positive_limiter (src/dissipation.jl:38-216) on every element.  w:
        element quadrature weights summing to 1 (default: the Gauss weights,
        2D: wp / 4 as example/shock-vortex.jl:301 passes them).  Returns the
        limited state and the count (negative: elements whose density
        parameter left (0, 1])."""
        uf = np.array(u, dtype=np.float64, order="F", copy=True)
        kind = self.cfg.kind
        if w is None:
            w = np.asarray(self.space.wp).ravel(order="F")
            w = w / 4.0 if kind == EULER2D else w / 2.0
        w = _f64(np.asarray(w).ravel(order="F"))
        fn = {EULER2D: "fro_positive_limiter2d", EULER1D: "fro_positive_limiter1d"}.get(kind,
                                                                                        "fro_positive_limiter_scalar")
        n = getattr(lib(), fn)(C.byref(self.cfg), uf.ctypes.data_as(_D), _p(w), float(t0))
        return uf, n

    def conserved_sums2d(self, u: np.ndarray) -> np.ndarray:
        uf = np.asfortranarray(u, dtype=np.float64)
        out = np.zeros(4)
        wp = _f64(self.space.wp)
        lib().fro_conserved_sums2d(C.byref(self.cfg), uf.ctypes.data_as(_D), _p(wp), _p(out))
        return out

    def max_speed2d(self, u: np.ndarray) -> float:
        uf = np.asfortranarray(u, dtype=np.float64)
        return lib().fro_max_speed2d(C.byref(self.cfg), uf.ctypes.data_as(_D))


def set_threads(n: int) -> None:
    lib().fro_set_threads(int(n))


def get_threads() -> int:
    return lib().fro_get_threads()


def l1_error(u, ue, dx):
    a, b = _f64(u), _f64(ue)
    return lib().fro_L1_error(_p(a), _p(b), a.size, dx)


def l2_error(u, ue, dx):
    a, b = _f64(u), _f64(ue)
    return lib().fro_L2_error(_p(a), _p(b), a.size, dx)


def linf_error(u, ue, dx):
    a, b = _f64(u), _f64(ue)
    return lib().fro_Linf_error(_p(a), _p(b), a.size, dx)


def prim_conserve2d(prim, gamma):
    p = _f64(prim)
    w = np.zeros(4)
    lib().fro_prim_conserve2d(_p(p), gamma, _p(w))
    return w


def flux_hll2d(wL, wR, gamma, d):
    a, b = _f64(wL), _f64(wR)
    f = np.zeros(4)
    lib().fro_flux_hll2d(_p(a), _p(b), gamma, d, _p(f))
    return f


def flux_lf2d(wL, wR, gamma, d):
    a, b = _f64(wL), _f64(wR)
    f = np.zeros(4)
    lib().fro_flux_lf2d(_p(a), _p(b), gamma, d, _p(f))
    return f


def mlp_forward(params, x, nin=32, nh=64):
    P = _f64(params)
    X = np.ascontiguousarray(x, dtype=np.float64)
    n = X.shape[0]
    y = np.zeros(n)
    lib().fro_mlp_forward(_p(P), X.ctypes.data_as(_D), n, nin, nh, _p(y))
    return y


def mlp_loss_grad(params, x, labels, nin=32, nh=64):
    P = _f64(params)
    X = np.ascontiguousarray(x, dtype=np.float64)
    t = _f64(labels)
    g = np.zeros_like(P)
    loss = lib().fro_mlp_loss_grad(_p(P), X.ctypes.data_as(_D), _p(t), X.shape[0], nin, nh, _p(g))
    return loss, g


# ---------------------------------------------------------------- triangles
def vandermonde_tri(N: int, r, s):
    """vandermonde_matrix(Tri, N, r, s) (src/Transform/transform.jl:36-50) and
    its r, s derivatives (:106-127), restated in fr_oracle.c."""
    r, s = _f64(r), _f64(s)
    npm = (N + 1) * (N + 2) // 2
    V, Vr, Vs = (np.zeros((len(r), npm), order="F") for _ in range(3))
    lib().fro_vandermonde_tri(N, _p(r), _p(s), len(r), _p(V))
    lib().fro_dvandermonde_tri(N, _p(r), _p(s), len(r), _p(Vr), _p(Vs))
    return V, Vr, Vs


def triface_points(N: int):
    """triface_quadrature(N) (src/Quadrature/quadrature.jl:86-106)."""
    p0, w0 = gauss_legendre(N + 1)
    pf = np.zeros((3, N + 1, 2))
    pf[0, :, 0], pf[0, :, 1] = p0, -1.0
    pf[1, :, 0], pf[1, :, 1] = p0[::-1], p0
    pf[2, :, 0], pf[2, :, 1] = -1.0, p0[::-1]
    wf = np.stack([w0, w0 * np.sqrt(2.0), w0])
    return pf, wf


def tri_operators(N: int, r, s):
    """TriFRPSpace's V, dl = dlagrange(V, Vr, Vs) (V' \\ Vr[i, :] per point),
    lf (V' \\ psi_f) and phi = correction_field(N, V)
    (src/struct.jl:305-352, src/Polynomial/poly_triangle.jl:1-28), with numpy
    solves on the oracle's Vandermonde matrices."""
    V, Vr, Vs = vandermonde_tri(N, r, s)
    npm = V.shape[0]
    dl = np.zeros((npm, npm, 2), order="F")
    dl[:, :, 0] = np.linalg.solve(V.T, Vr.T).T
    dl[:, :, 1] = np.linalg.solve(V.T, Vs.T).T
    pf, wf = triface_points(N)
    lf = np.zeros((3, N + 1, npm), order="F")
    phi = np.zeros((3, N + 1, npm), order="F")
    for f in range(3):
        psi, _, _ = vandermonde_tri(N, pf[f, :, 0], pf[f, :, 1])
        lf[f] = np.linalg.solve(V.T, psi.T).T
        sigma = wf[f][:, None] * psi
        phi[f] = sigma @ V.T
    return V, dl, lf, phi


class TriProblem:
    """The linear-advection dudt! of dev/wave_triangle.jl:44-125 on given
    TriFRPSpace operators and mesh connectivity (fro_tri_rhs); u[ncell, np]."""

    def __init__(self, deg, a, dl, lf, phi, J, iJ, nb_cell, nb_face, nb_point, cell_type):
        self._keep = [np.asfortranarray(x, dtype=np.float64) for x in (dl, lf, phi, J, iJ)]
        self._keep += [np.asfortranarray(x, dtype=np.int32) for x in (nb_cell, nb_face, nb_point, cell_type)]
        d = self._keep
        ncell = d[3].shape[0]
        self.shape = (ncell, (deg + 1) * (deg + 2) // 2)
        self.cfg = TriCfg(ncell, deg, self.shape[1], deg + 1, float(a),
                          *(x.ctypes.data_as(_D) for x in d[:5]), *(x.ctypes.data_as(_I) for x in d[5:]))

    def rhs(self, u) -> np.ndarray:
        uf = np.asfortranarray(u, dtype=np.float64)
        du = np.zeros(self.shape, order="F")
        lib().fro_tri_rhs(C.byref(self.cfg), _p(du), _p(uf))
        return du

    def erk(self, u, dt: float, nsteps: int, A, b) -> np.ndarray:
        uf = np.array(u, dtype=np.float64, order="F", copy=True)
        A = np.ascontiguousarray(A, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        s = len(b)
        work = np.zeros((s + 1) * uf.size)
        lib().fro_tri_erk(C.byref(self.cfg), _p(uf), float(dt), int(nsteps), s, _p(A), _p(b), _p(work))
        return uf
