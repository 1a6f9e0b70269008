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


def shock_vortex_problem(ps, mach_v=0.25, precision="fp32k", flux="hll", ghosts_per_step=True):
    """The shock-vortex ODE problem: fixed upstream inflow on the left, copy
    (extrapolation) ghosts elsewhere, refreshed once per step as
    example/shock-vortex.jl:323-330 does after each step (ghosts_per_step=False:
    they follow every stage's input)."""
    u, upstream = shock_vortex_state(ps.xpg, mach_v)
    prob = api.FREuler2DProblem(u, (0.0, 1.0), ps, GAMMA, flux=flux, bc=("fix", "copy", "copy", "copy"),
                                fixed_states=[upstream, None, None, None], precision=precision)
    if ghosts_per_step:
        prob.set_option(L.OPT_GHOSTS_PER_STEP, 1)
    return prob


FILTER_LAMBDA = 5e-4  # example/shock-vortex.jl:316
FILTER_KAPPA = 9.0    # example/shock-vortex.jl:311
# Decision threshold of the shipped shock-vortex network (troubled when its
# output exceeds it).  The network is trained on class-balanced plain labels,
# which biases it toward "troubled": at 0.5 it filters 6-20 % more elements
# than the plain test on the shock-vortex workload; at 0.97 it filters fewer
# (1.6-25 % over 600 steps at two vortex strengths with the script's
# once-per-step ghosts, 0.7-2.3 % with per-stage ghosts) at the plain test's L2
# error or below (tests/test_learned_gain_gpu.py).
DECISION_THRESHOLD = 0.97


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
        try:
            itg.set_filter("plain", FILTER_LAMBDA, S0, FILTER_KAPPA)
            if n > 1:
                itg.step(n - 1)
            itg.set_filter("none")
            itg.step(1)
        except L.FRGPUError:
            break  # the filtered scheme lost positivity: keep the snapshots taken so far
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


# ---------------------------------------------------------------- full-scale training
import os as _os

WEIGHTS = _os.path.join(_os.path.dirname(_os.path.abspath(__file__)), "data", "shock_vortex_mlp.npy")
RECORD = _os.path.join(_os.path.dirname(_os.path.abspath(__file__)), "data", "shock_vortex_mlp.json")
CONFIG3 = dict(x0=0.0, x1=2.0, nx=400, y0=0.0, y1=1.0, ny=200, deg=3)


def config3_space():
    c = CONFIG3
    return api.FRPSpace2D(c["x0"], c["x1"], c["nx"], c["y0"], c["y1"], c["ny"], c["deg"])


def load_trained() -> "MLPIndicator":
    """The network trained by `train_config3` (shipped with the package)."""
    return MLPIndicator.load(WEIGHTS)


def evaluate(m, ps, mach_v, nsteps, indicator, cfl=0.1, threshold=0.5, band=0.0):
    """Run the shock-vortex problem with one indicator ('none', 'plain', 'mlp')
    and report the final state, the network's misfires (judged by the plain
    test) and the troubled-element count of the last step."""
    prob = shock_vortex_problem(ps, mach_v)
    itg = api.init(prob, dt=1.0)
    itg.dt = itg.cfl_dt(cfl)
    if indicator == "mlp":
        check(L.lib().frgpu_problem_set_mlp(prob._h, m._h, float(threshold), float(band)))
    stats = np.zeros(3, dtype=np.int32)
    mis = 0
    seen = 0
    ok = True
    if indicator != "none":
        itg.set_filter(indicator, FILTER_LAMBDA, filter_S0(ps.deg), FILTER_KAPPA)
    try:
        if indicator == "mlp":
            for _ in range(nsteps):
                itg.step(1)
                check(L.lib().frgpu_indicator_stats(prob._h, stats.ctypes.data_as(L._I)))
                mis += int(stats[1])
                seen += ps.nx * ps.ny
        else:
            itg.step(nsteps)
        u = itg.u
    except L.FRGPUError:
        ok = False
        u = None
    return {"ok": ok, "u": u, "misfires": mis, "elements_seen": seen, "dt": itg.dt}


def train_config3(nseeds=64, nsteps=2400, every=240, epochs=20, batch=4096, lr=2e-3, seed=0, log=print):
    """Labels from plain-indicator runs of config 3 (400 x 200, deg 3) over
    `nseeds` seeded vortex strengths (seeds 0..nseeds-1, Mach uniform on
    [0.1, 0.4]); seeds >= nseeds - 8 are held out for validation."""
    import json
    import time

    ps = config3_space()
    t0 = time.time()
    train_seeds = range(0, nseeds - 8)
    val_seeds = range(nseeds - 8, nseeds)
    x, t = build_dataset(ps, train_seeds, nsteps=nsteps, every=every, keep_neg=0.01)
    xv, tv = build_dataset(ps, val_seeds, nsteps=nsteps, every=every, keep_neg=0.01)
    t_data = time.time() - t0
    log(f"dataset: {len(t)} samples ({int(t.sum())} troubled), validation {len(tv)} ({int(tv.sum())}); {t_data:.1f} s")
    xb, tb = balance(x, t, seed=seed)
    m = MLPIndicator(seed=seed)
    t1 = time.time()
    losses = m.train(xb, tb, epochs=epochs, batch=batch, lr=lr, seed=seed)
    t_train = time.time() - t1
    yv = m.forward(xv)
    pred = yv > 0.5
    lab = tv > 0.5
    rec = {
        "config": dict(CONFIG3, nseeds=nseeds, nsteps=nsteps, every=every, epochs=epochs, batch=batch, lr=lr,
                       seed=seed, mach_range=[0.1, 0.4], filter_lambda=FILTER_LAMBDA, kappa=FILTER_KAPPA),
        "samples": int(len(t)), "troubled": int(t.sum()), "balanced_samples": int(len(tb)),
        "loss_per_epoch": [float(v) for v in losses],
        "validation": {"samples": int(len(tv)), "troubled": int(lab.sum()),
                       "accuracy": float(np.mean(pred == lab)),
                       "false_positive": int(np.sum(pred & ~lab)), "false_negative": int(np.sum(~pred & lab))},
        "seconds": {"labels": t_data, "training": t_train},
    }
    log(json.dumps(rec["validation"]))
    return m, rec


# ---------------------------------------------------------------- 1D Burgers ensembles
# The ensemble's indicator is the 1D modal-decay test of
# example/euler_highlevel.jl:37-52 (su = u_N^2 / (sum u^2 + 1e-6), S0 =
# -3 log10(deg), kappa = 4).  Its learned replacement sees 32 features per
# element: the normalised modal energies (slots 0..deg), a degree one-hot
# (slots 8..12) and the energy level against the 1e-6 floor (slot 16).
BURGERS_WEIGHTS = _os.path.join(_os.path.dirname(_os.path.abspath(__file__)), "data", "burgers1d_mlp.npy")
BURGERS_RECORD = _os.path.join(_os.path.dirname(_os.path.abspath(__file__)), "data", "burgers1d_mlp.json")


def burgers_label_run(n_inst, seed, t_samples, cfl=0.4, keep_neg=0.03):
    """Features and plain labels of a config-4-like ensemble (sizes and ICs
    from Philox with `seed`) run with the plain indicator, sampled at the
    times `t_samples`; all troubled elements and `keep_neg` of the others."""
    from .ensemble import Ensemble, config4_sizes

    ne, deg = config4_sizes(n_inst, seed)
    e = Ensemble(ne, deg, precision="fp32")
    e.init_fourier(0.3, seed)
    rng = np.random.default_rng(seed)
    xs, ts = [], []
    t = 0.0
    for ts_ in t_samples:
        e.run(ts_ - t, cfl=cfl, filter=True)
        t = ts_
        x, lab = e.features()
        # rows of instances stopped by a blow-up are not finite: leave them out
        keep = ((lab > 0) | (rng.random(len(lab)) < keep_neg)) & np.all(np.isfinite(x), axis=1)
        xs.append(x[keep])
        ts.append(lab[keep].astype(np.float32))
    return np.concatenate(xs), np.concatenate(ts)


def load_trained_burgers1d() -> "MLPIndicator":
    """The network trained by `train_burgers1d` (shipped with the package)."""
    return MLPIndicator.load(BURGERS_WEIGHTS)


def train_burgers1d(n_inst=512, nseeds=16, t_samples=(0.05, 0.1, 0.15, 0.2, 0.25, 0.3, 0.35, 0.4, 0.45, 0.5),
                    epochs=20, batch=4096, lr=2e-3, seed=0, log=print):
    """Labels from plain-indicator ensembles with Philox seeds 1000..1000+nseeds-1
    (the config-4 bench uses seed 0); the last two seeds are held out."""
    import json
    import time

    t0 = time.time()
    seeds = [1000 + s for s in range(nseeds)]
    parts = [burgers_label_run(n_inst, s, t_samples) for s in seeds]
    x = np.concatenate([p[0] for p in parts[:-2]])
    t = np.concatenate([p[1] for p in parts[:-2]])
    xv = np.concatenate([p[0] for p in parts[-2:]])
    tv = np.concatenate([p[1] for p in parts[-2:]])
    t_data = time.time() - t0
    log(f"dataset: {len(t)} samples ({int(t.sum())} troubled), validation {len(tv)} ({int(tv.sum())}); {t_data:.1f} s")
    xb, tb = balance(x, t, seed=seed)
    m = MLPIndicator(seed=seed)
    t1 = time.time()
    losses = m.train(xb, tb, epochs=epochs, batch=batch, lr=lr, seed=seed)
    t_train = time.time() - t1
    yv = m.forward(xv)
    pred = yv > 0.5
    lab = tv > 0.5
    rec = {
        "config": dict(n_inst=n_inst, seeds=seeds, t_samples=list(t_samples), epochs=epochs, batch=batch, lr=lr,
                       seed=seed, sigma=0.3, cfl=0.4),
        "samples": int(len(t)), "troubled": int(t.sum()), "balanced_samples": int(len(tb)),
        "loss_per_epoch": [float(v) for v in losses],
        "validation": {"samples": int(len(tv)), "troubled": int(lab.sum()),
                       "accuracy": float(np.mean(pred == lab)),
                       "false_positive": int(np.sum(pred & ~lab)), "false_negative": int(np.sum(~pred & lab))},
        "seconds": {"labels": t_data, "training": t_train},
    }
    log(json.dumps(rec["validation"]))
    return m, rec


def main(argv=None):
    import argparse
    import json

    ap = argparse.ArgumentParser(description="train a learned troubled-cell indicator")
    ap.add_argument("--workload", choices=["shock-vortex", "burgers1d"], default="shock-vortex")
    ap.add_argument("--out", default=None)
    ap.add_argument("--record", default=None)
    ap.add_argument("--nseeds", type=int, default=None)
    ap.add_argument("--nsteps", type=int, default=2400)
    ap.add_argument("--epochs", type=int, default=20)
    a = ap.parse_args(argv)
    if a.workload == "burgers1d":
        m, rec = train_burgers1d(nseeds=a.nseeds or 16, epochs=a.epochs)
        a.out = a.out or BURGERS_WEIGHTS
        a.record = a.record or BURGERS_RECORD
    else:
        m, rec = train_config3(nseeds=a.nseeds or 64, nsteps=a.nsteps, epochs=a.epochs)
        a.out = a.out or WEIGHTS
        a.record = a.record or RECORD
    _os.makedirs(_os.path.dirname(a.out), exist_ok=True)
    m.save(a.out)
    with open(a.record, "w") as f:
        json.dump(rec, f, indent=1)


if __name__ == "__main__":
    main()
