"""Batched ensembles of 1D Burgers instances (uneven element counts and
degrees) advanced together by one persistent kernel launch per run."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L
from ._lib import check, dptr, fptr

_PREC = {"fp64": L.FP64, "fp32": L.FP32K}


def config4_sizes(n: int = 4096, seed: int = 0):
    """Element counts (log-uniform in [32, 2048]) and degrees (uniform 1..5)
    of the config-4 ensemble, drawn per instance id from Philox-4x32-10."""
    ne = np.zeros(n, dtype=np.int32)
    deg = np.zeros(n, dtype=np.int32)
    check(L.lib().frgpu_ensemble_config4_sizes(n, seed, ne.ctypes.data_as(L._I), deg.ctypes.data_as(L._I)))
    return ne, deg


class Ensemble:
    def __init__(self, ne, deg, x0=0.0, x1=2 * math.pi, precision="fp32"):
        self.ne = np.ascontiguousarray(ne, dtype=np.int32)
        self.deg = np.ascontiguousarray(deg, dtype=np.int32)
        self.n = len(self.ne)
        self.x0, self.x1 = float(x0), float(x1)
        h = C.c_void_p()
        check(L.lib().frgpu_ensemble_create(self.n, self.ne.ctypes.data_as(L._I), self.deg.ctypes.data_as(L._I),
                                            self.x0, self.x1, _PREC[precision], C.byref(h)))
        self._h = h

    @classmethod
    def config4(cls, n=4096, seed=0, precision="fp32", sigma=0.3):
        ne, deg = config4_sizes(n, seed)
        e = cls(ne, deg, 0.0, 2 * math.pi, precision)
        e.init_fourier(sigma, seed)
        return e

    def __del__(self):
        if getattr(self, "_h", None) is not None and L._lib is not None:
            L._lib.frgpu_ensemble_destroy(self._h)
            self._h = None

    @property
    def ndof(self) -> int:
        return int(L.lib().frgpu_ensemble_ndof(self._h))

    def set_state(self, i, u):
        u = np.asfortranarray(u, dtype=np.float64)
        assert u.shape == (self.ne[i], self.deg[i] + 1)
        check(L.lib().frgpu_ensemble_set_state(self._h, int(i), dptr(u)))

    def get_state(self, i) -> np.ndarray:
        out = np.zeros((int(self.ne[i]), int(self.deg[i]) + 1), order="F")
        check(L.lib().frgpu_ensemble_get_state(self._h, int(i), dptr(out)))
        return out

    def init_fourier(self, sigma=0.3, seed=0):
        check(L.lib().frgpu_ensemble_init_fourier(self._h, float(sigma), int(seed)))

    @property
    def tiles(self):
        t = np.zeros(5, dtype=np.int32)
        check(L.lib().frgpu_ensemble_get_tiles(self._h, t.ctypes.data_as(L._I)))
        return t

    @tiles.setter
    def tiles(self, thr):
        t = np.ascontiguousarray(thr, dtype=np.int32)
        check(L.lib().frgpu_ensemble_set_tiles(self._h, t.ctypes.data_as(L._I)))

    def run(self, t_end, cfl=0.4, filter=True) -> int:
        """Advance every running instance by t_end; returns the number of
        instances stopped so far because their state turned non-finite."""
        check(L.lib().frgpu_ensemble_run(self._h, float(t_end), float(cfl), int(bool(filter))))
        return self.failed().astype(bool).sum()

    def failed(self) -> np.ndarray:
        """Per instance: 0, or the step after which it stopped (non-finite state)."""
        f = np.zeros(self.n, dtype=np.int32)
        rc = L.lib().frgpu_ensemble_failed(self._h, f.ctypes.data_as(L._I))
        if rc < 0:
            check(rc)
        return f

    def tune(self, t_probe=0.01, cfl=0.4, filter=True):
        t = np.zeros(5, dtype=np.int32)
        check(L.lib().frgpu_ensemble_tune(self._h, float(t_probe), float(cfl), int(bool(filter)),
                                          t.ctypes.data_as(L._I)))
        return t

    def stats(self):
        tot = C.c_double()
        mx = C.c_int()
        ms = C.c_float()
        dt = np.zeros(self.n)
        steps = np.zeros(self.n, dtype=np.int32)
        check(L.lib().frgpu_ensemble_stats(self._h, C.byref(tot), C.byref(mx), C.byref(ms), dptr(dt),
                                           steps.ctypes.data_as(L._I)))
        return {"dof_stage_updates": tot.value, "max_steps": mx.value, "ms": ms.value, "dt": dt, "steps": steps}

    def launches(self) -> int:
        return int(L.lib().frgpu_ensemble_launches(self._h))

    def set_mlp(self, net, threshold=0.5, band=0.0):
        """Learned indicator in the post-step filter (None: plain modal-decay test)."""
        check(L.lib().frgpu_ensemble_set_mlp(self._h, net._h if net is not None else None, float(threshold),
                                             float(band)))
        self._net = net  # the library borrows the network

    def indicator_stats(self):
        """Last run's learned-indicator counts over all steps and instances."""
        s = (C.c_longlong * 4)()
        check(L.lib().frgpu_ensemble_indicator_stats(self._h, s))
        return {"troubled": s[0], "misfires": s[1], "fallbacks": s[2], "judged": s[3]}

    @property
    def nelem(self) -> int:
        return int(L.lib().frgpu_ensemble_nelem(self._h))

    def features(self):
        """(features [nelem, 32] float32, plain labels [nelem] int32) of the current state."""
        n = self.nelem
        feat = np.zeros((n, 32), dtype=np.float32)
        lab = np.zeros(n, dtype=np.int32)
        check(L.lib().frgpu_ensemble_features(self._h, fptr(feat), lab.ctypes.data_as(L._I), n))
        return feat, lab
