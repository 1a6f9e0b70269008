"""Learned troubled-cell indicator: network object, the shock-vortex workload
that supplies its labels, and the training driver.

The indicator replaces the modal-decay test of the post-step filter loop of
example/shock-vortex.jl:308-321 (shock_detector, src/dissipation.jl:13-23).
Labels come from the plain test itself, evaluated on states of plain-indicator
runs of the shock-vortex problem over 64 seeded vortex strengths; training
and evaluation run on the GPU through libfrgpu's BF16-in / FP32-accumulate
tensor-core kernels.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L
from . import api
from ._lib import check, fptr

NIN = 32


class MLPIndicator:
    """32 -> 64 -> 64 -> 1 perceptron (GELU, GELU, sigmoid) on the device."""

    def __init__(self, seed: int = 0):
        h = C.c_void_p()
        check(L.lib().frgpu_mlp_create(int(seed), C.byref(h)))
        self._h = h
        self.nparams = int(L.lib().frgpu_mlp_nparams())

    def __del__(self):
        if getattr(self, "_h", None) is not None and L._lib is not None:
            L._lib.frgpu_mlp_destroy(self._h)
            self._h = None

    @property
    def params(self) -> np.ndarray:
        out = np.zeros(self.nparams, dtype=np.float32)
        check(L.lib().frgpu_mlp_get_params(self._h, fptr(out)))
        return out

    @params.setter
    def params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparams
        check(L.lib().frgpu_mlp_set_params(self._h, fptr(p)))

    def forward(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, NIN)
        y = np.zeros(x.shape[0], dtype=np.float32)
        check(L.lib().frgpu_mlp_forward(self._h, fptr(x), x.shape[0], fptr(y)))
        return y

    def loss_grad(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, NIN)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        g = np.zeros(self.nparams, dtype=np.float32)
        check(L.lib().frgpu_mlp_loss_grad(self._h, fptr(x), fptr(t), x.shape[0], fptr(loss), fptr(g)))
        return float(loss[0]), g

    def train(self, x, t, epochs=10, batch=4096, lr=3e-3, seed=0) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, NIN)
        t = np.ascontiguousarray(t, dtype=np.float32)
        losses = np.zeros(max(epochs, 1), dtype=np.float32)
        check(L.lib().frgpu_mlp_train(self._h, fptr(x), fptr(t), x.shape[0], int(epochs), int(batch), float(lr),
                                      int(seed), fptr(losses)))
        return losses[:epochs]

    def save(self, path: str) -> None:
        np.save(path, self.params)

    @classmethod
    def load(cls, path: str) -> "MLPIndicator":
        m = cls(0)
        m.params = np.load(path)
        return m


# ---------------------------------------------------------------- shock-vortex workload
GAMMA = 1.4
MACH_SHOCK = 1.1
VORTEX_RC = 0.075
VORTEX_ALPHA = 0.204
VORTEX_CENTRE = (0.25, 0.5)
SHOCK_X = 0.5
# peak of tau exp(alpha (1 - tau^2)): the vortex's maximum tangential speed is
# TAU_PEAK * eps for strength eps
TAU_PEAK = (1 / math.sqrt(2 * VORTEX_ALPHA)) * math.exp(VORTEX_ALPHA - 0.5)


def vortex_strength(mach_v: float) -> float:
    """Strength eps whose peak tangential speed is mach_v times the upstream sound speed."""
    return mach_v * math.sqrt(GAMMA) / TAU_PEAK


def shock_vortex_state(xpg, mach_v: float = 0.25, gamma: float = GAMMA):
    """Config 3 initial state on [0,2] x [0,1]: a stationary Mach 1.1 normal shock
    at x = 0.5 (upstream rho = 1, p = 1, u = 1.1 c) and an isentropic vortex of
    radius 0.075 centred at (0.25, 0.5) (the form of example/shock-vortex.jl:170-190,
    with these parameters) in the upstream flow.  Returns (u, upstream conserved state)."""
    X, Y = xpg[..., 0], xpg[..., 1]
    c1 = math.sqrt(gamma)
    u1 = MACH_SHOCK * c1
    M2 = MACH_SHOCK ** 2
    rr = (gamma + 1) * M2 / ((gamma - 1) * M2 + 2)
    pr = 1 + 2 * gamma / (gamma + 1) * (M2 - 1)
    eps = vortex_strength(mach_v)
    x0, y0 = VORTEX_CENTRE
    r = np.hypot(X - x0, Y - y0)
    tau = r / VORTEX_RC
    a = VORTEX_ALPHA
    e1 = np.exp(a * (1 - tau ** 2))
    rs = np.maximum(r, 1e-300)
    du = eps * tau * e1 * (Y - y0) / rs
    dv = -eps * tau * e1 * (X - x0) / rs
    dT = -(gamma - 1) * eps ** 2 / (4 * a * gamma) * np.exp(2 * a * (1 - tau ** 2))
    inside = r <= 8 * VORTEX_RC
    T = 1 + np.where(inside, dT, 0.0)
    rho = T ** (1 / (gamma - 1))
    p = rho * T
    U = u1 + np.where(inside, du, 0.0)
    V = np.where(inside, dv, 0.0)
    post = X > SHOCK_X
    rho = np.where(post, rr, rho)
    p = np.where(post, pr, p)
    U = np.where(post, u1 / rr, U)
    V = np.where(post, 0.0, V)
    w = np.zeros(X.shape + (4,), order="F")
    w[..., 0] = rho
    w[..., 1] = rho * U
    w[..., 2] = rho * V
    w[..., 3] = p / (gamma - 1) + 0.5 * rho * (U * U + V * V)
    upstream = [1.0, u1, 0.0, 1 / (gamma - 1) + 0.5 * u1 * u1]
    return w, upstream


def shock_vortex_problem(ps, mach_v=0.25, precision="fp32k", flux="hll"):
    """The shock-vortex ODE problem: fixed upstream inflow on the left, copy
    (extrapolation) ghosts elsewhere, as in example/shock-vortex.jl:323-330."""
    u, upstream = shock_vortex_state(ps.xpg, mach_v)
    return api.FREuler2DProblem(u, (0.0, 1.0), ps, GAMMA, flux=flux, bc=("fix", "copy", "copy", "copy"),
                                fixed_states=[upstream, None, None, None], precision=precision)


FILTER_LAMBDA = 5e-4  # example/shock-vortex.jl:316
FILTER_KAPPA = 9.0    # example/shock-vortex.jl:311


def filter_S0(deg: int = 3) -> float:
    return -3.0 * math.log10(deg)


def label_run(ps, mach_v, nsteps, every, cfl=0.1, keep_neg=0.02, seed=0):
    """Plain-indicator run of the shock-vortex problem; every `every` steps the
    indicator inputs of all elements and the plain test's verdicts are
    recorded (all troubled elements plus a `keep_neg` fraction of the rest)."""
    rng = np.random.default_rng(seed)
    prob = shock_vortex_problem(ps, mach_v)
    itg = api.init(prob, dt=1.0)
    itg.dt = itg.cfl_dt(cfl)
    S0 = filter_S0(ps.deg)
    ne = ps.nx * ps.ny
    xs, ts = [], []
    done = 0
    while done < nsteps:
        n = min(every, nsteps - done)
        itg.set_filter("plain", FILTER_LAMBDA, S0, FILTER_KAPPA)
        if n > 1:
            itg.step(n - 1)
        itg.set_filter("none")
        itg.step(1)
        done += n
        feat = np.zeros(ne * NIN, dtype=np.float32)
        check(L.lib().frgpu_modal_features(prob._h, fptr(feat), feat.size))
        feat = feat.reshape(ne, NIN)
        itg.modal_filter("plain", FILTER_LAMBDA, S0, FILTER_KAPPA)
        flags = itg.troubled().astype(bool)
        keep = flags | (rng.random(ne) < keep_neg)
        xs.append(feat[keep])
        ts.append(flags[keep].astype(np.float32))
    return np.concatenate(xs), np.concatenate(ts)


def seeded_mach(seed: int) -> float:
    """Vortex Mach number of training seed `seed`: uniform on [0.1, 0.4] around 0.25."""
    return float(np.random.default_rng(10_000 + seed).uniform(0.1, 0.4))


def build_dataset(ps, seeds, nsteps=600, every=60, keep_neg=0.02):
    xs, ts = [], []
    for s in seeds:
        x, t = label_run(ps, seeded_mach(s), nsteps, every, keep_neg=keep_neg, seed=s)
        xs.append(x)
        ts.append(t)
    return np.concatenate(xs), np.concatenate(ts)


def balance(x, t, seed=0, ratio=3.0):
    """All positives and `ratio` times as many negatives, shuffled."""
    rng = np.random.default_rng(seed)
    pos = np.flatnonzero(t > 0.5)
    neg = np.flatnonzero(t <= 0.5)
    k = min(len(neg), int(ratio * max(len(pos), 1)))
    sel = np.concatenate([pos, rng.choice(neg, k, replace=False)])
    rng.shuffle(sel)
    return x[sel], t[sel]
