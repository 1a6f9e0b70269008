#!/usr/bin/env python3
"""Benchmark: RK-stage DOF-updates/s of the flux-reconstruction hot path.

Workload (one GPU): 2D Euler density wave on periodic [0,1]^2 with 512 x 512
quadrilaterals, p = 3 (16 solution points per element, 16,777,216 DOFs),
gamma = 1.4, rho = 1 + 0.2 sin(2 pi (x + y)), u = v = 1, p = 1, local
Lax-Friedrichs interface flux, SSPRK3 at CFL 0.1.  One bench "step" is one
SSPRK3 time step (three fused residual+stage launches) over the whole mesh.

* ``value``     FP32 compensated form (FP32K), device-resident, CUDA-event timed.
* ``fp64``      plain FP64 form on the same workload, same timing.
* ``e2e``       the same metric through the C ABI with host buffers: the state
                uploaded from host memory and downloaded at the end, and each
                step's dt written and its FP64 conserved sums / wave speed read
                back (frgpu_step_ssprk3 + frgpu_reduce), all inside the timed region.
* ``roofline``  HBM roofline of the dominant kernel (the fused stage kernel).
* ``cpu_baseline`` the CPU FP64 oracle (OpenMP over all host cores) on a bounded
                sample of the same workload.

``--impl reference`` times the reference's CPU algorithm (the oracle port; the
Julia reference cannot run here) on the same config, metric and unit.
Multi-GPU: the path is run as independent replicas (one per rank, no
collective on the data path); ``value`` sums the replicas' DOFs over the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for sub in ("fluxreconstruction.jl_gb300",):
    sys.path.insert(0, os.path.join(ROOT, sub))

METRIC = "RK-stage DOF updates/s on 1 GB300, learned+FP32 vs plain FP64, at matched L2 err"
UNIT = "DOF-updates/s"
NX = NY = 512
DEG = 3
GAMMA = 1.4
CFL = 0.1
NP = DEG + 1
NDOF = NX * NY * NP * NP * 4
WORKLOAD = "2D Euler density wave, periodic [0,1]^2, 512x512 quads, p=3, LF flux, SSPRK3 at CFL 0.1"
# Algorithmic HBM bytes per DOF per RK stage of a fused SSPRK3 step: 8/3 state
# arrays per stage on average (stage 1 reads u^n and writes u1; stages 2 and 3
# read u^n and the stage input and write the result).
BYTES_PER_DOF_STAGE = {"fp32k": 4 * 8 / 3, "fp64": 8 * 8 / 3}
# DRAM bytes (read + write) per stage launch measured by ncu on this workload
# (mean over the three SSPRK3 stages of the FP32K form; the capture of the
# 512x512 p=3 stage kernels kept under profiles/).
NCU_TRAFFIC_PER_LAUNCH = {"fp32k": 188.7e6, "fp64": None}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def density_wave(xpg):
    X, Y = xpg[..., 0], xpg[..., 1]
    rho = 1 + 0.2 * np.sin(2 * np.pi * (X + Y))
    u = np.zeros(X.shape + (4,), order="F")
    u[..., 0] = rho
    u[..., 1] = rho
    u[..., 2] = rho
    u[..., 3] = 1 / (GAMMA - 1) + rho
    return u


def exact_density(xpg, t):
    X, Y = xpg[..., 0], xpg[..., 1]
    return 1 + 0.2 * np.sin(2 * np.pi * (X + Y - 2 * t))


def l2_err(u, xpg, t, dx, dy):
    """RMS of the density error over all solution points against the exact
    solution rho(x - t, y - t) of the density wave."""
    e = u[..., 0] - exact_density(xpg, t)
    return float(np.sqrt(np.mean(e * e)))


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            import tempfile

            fd, self.path = tempfile.mkstemp(prefix="frgpu_clocks_", suffix=".csv")
            self.f = os.fdopen(fd, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        with open(self.path) as f:
            for ln in f:
                parts = [p.strip() for p in ln.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return float("nan")

        sm = np.array([num(r[1]) for r in rows])
        mx = np.array([num(r[2]) for r in rows])
        pw = np.array([num(r[3]) for r in rows])
        loaded = sm[pw > np.nanmax(pw) * 0.5] if np.isfinite(pw).any() else sm
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.nanmedian(loaded if loaded.size else sm)), "sm_max_mhz": float(np.nanmax(mx)),
                "reasons": sorted(reasons), "samples": int(len(rows))}


# --------------------------------------------------------------------------- distributed
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist

    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    # replicas only: the process group carries the barrier and the max of the
    # timings, never data-path traffic, so gloo suffices
    dist.init_process_group("gloo")
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_replicas(advance, K: int, W: int, sync, dist=None, timer=None):
    """W untimed warm-up steps, then K timed steps bracketed by a barrier and a
    device sync on both sides; returns the slowest rank's seconds.
    ``advance(n)`` queues n steps in one call (the library replays its
    captured step graph n times and checks the status once)."""
    if W:
        advance(W)
    sync()
    barrier(dist)
    sync()
    if timer is not None:
        secs = timer(lambda: advance(K))
    else:
        t0 = time.perf_counter()
        advance(K)
        sync()
        secs = time.perf_counter() - t0
    sync()
    barrier(dist)
    return max_over_ranks(dist, secs)


# --------------------------------------------------------------------------- GPU arm
def gpu_arm(args, dist, rank, ws):
    import torch

    import frgpu

    from frgpu import learned

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    ps = frgpu.FRPSpace2D(0, 1, NX, 0, 1, NY, DEG)
    u0 = density_wave(ps.xpg)
    K, W = args.steps, args.warmup
    out = {}
    sampler = ClockSampler(torch.cuda.current_device())
    if rank == 0:
        sampler.start()
    net = learned.load_trained()
    S0 = learned.filter_S0(DEG)
    # (name, precision, indicator): the learned FP32 form and the plain FP64
    # form run the post-step indicator + :l2 filter every step (the filter loop
    # of example/shock-vortex.jl:308-321); "fp32k" is the bare stage kernel
    # the roofline is quoted on
    forms = (("fp32k_learned", "fp32k", "mlp"), ("fp32k", "fp32k", "none"), ("fp64_plain", "fp64", "plain"))
    if args.forms:
        forms = tuple(f for f in forms if f[0] in args.forms.split(","))
    for form, precision, indicator in forms:
        prob = frgpu.FREuler2DProblem(u0, (0, 1), ps, GAMMA, flux="lf", bc="period", precision=precision)
        itg = frgpu.init(prob, dt=1.0)
        dt = itg.cfl_dt(CFL)
        itg.dt = dt
        if indicator == "mlp":
            frgpu._lib.check(frgpu.lib().frgpu_problem_set_mlp(prob._h, net._h, 0.5, 0.0))
        if indicator != "none":
            itg.set_filter(indicator, learned.FILTER_LAMBDA, S0, learned.FILTER_KAPPA)
        stream = torch.cuda.ExternalStream(itg.stream())
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

        def timer(fn):
            ev[0].record(stream)
            fn()
            ev[1].record(stream)
            ev[1].synchronize()
            return ev[0].elapsed_time(ev[1]) / 1e3

        l0 = itg.launches()
        secs = run_replicas(lambda n: itg.step(n), K, W, itg.synchronize, dist, timer)
        launches = itg.launches() - l0
        t_end = (W + K) * dt
        err = l2_err(itg.u, ps.xpg, t_end, ps.dx, ps.dy)
        stage_s = secs / (3 * K)
        total_dofs = NDOF * 3 * K * ws
        out[form] = {"value": total_dofs / secs, "ms_per_step": secs / K * 1e3, "stage_us": stage_s * 1e6,
                     "dt": dt, "t_end": t_end, "rms_err_rho_vs_exact": err, "indicator": indicator,
                     "troubled_last_step": int(np.sum(itg.troubled())) if indicator != "none" else 0,
                     "launches_timed": launches}
        if form == "fp32k_learned" and not args.no_e2e:
            # end to end through the C ABI with host buffers
            # page-locked host FP64 arrays in the reference layout (the copy
            # engine moves them without a staging copy)
            def pinned(shape):
                t = torch.empty(int(np.prod(shape)), dtype=torch.float64, pin_memory=True)
                return t.numpy().reshape(shape, order="F")

            host_u, host_out = pinned(u0.shape), pinned(u0.shape)
            host_u[...] = u0
            sums_steps = []

            def e2e_run():
                itg.u = host_u                       # H2D of the state (host FP64 array)
                for _ in range(K):
                    itg.step(1)                      # H2D of dt inside frgpu_step_ssprk3
                    sums_steps.append(itg.reduce())  # D2H of FP64 sums + wave speed
                return itg.read_u(host_out)          # D2H of the final state

            itg.synchronize()
            barrier(dist)
            t0 = time.perf_counter()
            e2e_run()
            e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
            state_bytes = NDOF * 8
            out["e2e"] = {"value": total_dofs / e2e_s, "unit": UNIT,
                          "h2d_bytes_per_step": (state_bytes + 8 * K) / K,
                          "d2h_bytes_per_step": (state_bytes + 5 * 8 * K) / K,
                          "note": "state uploaded from and downloaded to page-locked host FP64 arrays once per K "
                                  "steps; dt written and conserved sums/max speed read every step"}
        del itg, prob
    clocks = sampler.stop() if rank == 0 else None
    return out, clocks


def _event_timer(stream):
    import torch

    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def timer(fn):
        ev[0].record(stream)
        fn()
        ev[1].record(stream)
        ev[1].synchronize()
        return ev[0].elapsed_time(ev[1]) / 1e3

    return timer


def shock_vortex_entry(steps=100, warmup=5):
    """Config 3: shock-vortex on [0,2]x[0,1], 400x200, p=3, HLL, indicator +
    :l2 filter after every step.  Learned + FP32K against plain FP64 (DOF
    updates/s), the network's misfire rate (judged by the plain test on every
    element of every step), and the L2 distance of each form's final density
    from the plain FP64 run (the FP64 GPU path is bit-identical to the oracle
    in the parity tests)."""
    import torch

    import frgpu
    from frgpu import learned

    ps = learned.config3_space()
    net = learned.load_trained()
    S0 = learned.filter_S0(3)
    ndof = ps.nx * ps.ny * 16 * 4
    out = {"workload": "shock-vortex 400x200 p=3 HLL, Mach 1.1 shock + Mach 0.25 vortex, filter every step",
           "ndof": ndof, "steps": steps}
    finals = {}
    dt = None
    for form, precision, ind in (("learned_fp32k", "fp32k", "mlp"), ("plain_fp32k", "fp32k", "plain"),
                                 ("plain_fp64", "fp64", "plain")):
        prob = learned.shock_vortex_problem(ps, 0.25, precision=precision)
        itg = frgpu.init(prob, dt=1.0)
        if dt is None:
            dt = itg.cfl_dt(0.1)
        itg.dt = dt
        if ind == "mlp":
            frgpu._lib.check(frgpu.lib().frgpu_problem_set_mlp(prob._h, net._h, 0.5, 0.0))
        itg.set_filter(ind, learned.FILTER_LAMBDA, S0, learned.FILTER_KAPPA)
        timer = _event_timer(torch.cuda.ExternalStream(itg.stream()))
        itg.step(warmup)
        itg.synchronize()
        secs = timer(lambda: itg.step(steps))
        rec = {"value": ndof * 3 * steps / secs, "ms_per_step": secs / steps * 1e3}
        if ind == "mlp":
            # misfires over a further stretch of steps, read after each step
            st = np.zeros(3, dtype=np.int32)
            mis = trb = fb = 0
            for _ in range(50):
                itg.step(1)
                frgpu._lib.check(frgpu.lib().frgpu_indicator_stats(prob._h, st.ctypes.data_as(frgpu._lib._I)))
                trb, mis, fb = trb + int(st[0]), mis + int(st[1]), fb + int(st[2])
            rec["misfire_rate"] = mis / (50 * ps.nx * ps.ny)
            rec["troubled_per_step"] = trb / 50
        else:
            itg.step(50)
        finals[form] = itg.u[..., 0]
        out[form] = rec
    # the learned form with the positivity-preserving limiter before every step,
    # the full loop of example/shock-vortex.jl:297-321 (limiter, step, filter)
    prob = learned.shock_vortex_problem(ps, 0.25, precision="fp32k")
    itg = frgpu.init(prob, dt=dt)
    frgpu._lib.check(frgpu.lib().frgpu_problem_set_mlp(prob._h, net._h, 0.5, 0.0))
    itg.set_filter("mlp", learned.FILTER_LAMBDA, S0, learned.FILTER_KAPPA)
    nlim = itg.positive_limiter()
    itg.set_limiter(True)
    timer = _event_timer(torch.cuda.ExternalStream(itg.stream()))
    itg.step(warmup)
    itg.synchronize()
    secs = timer(lambda: itg.step(steps))
    out["learned_fp32k_with_limiter"] = {"value": ndof * 3 * steps / secs, "ms_per_step": secs / steps * 1e3,
                                         "limited_elements_at_start": nlim}
    # the reference's own loop: Midpoint (shock-vortex.jl:294), limiter before
    # and learned filter after every step; DOF updates counted per RK stage (2)
    prob = learned.shock_vortex_problem(ps, 0.25, precision="fp32k")
    itg = frgpu.init(prob, frgpu.Midpoint(), dt=dt)
    frgpu._lib.check(frgpu.lib().frgpu_problem_set_mlp(prob._h, net._h, 0.5, 0.0))
    itg.set_filter("mlp", learned.FILTER_LAMBDA, S0, learned.FILTER_KAPPA)
    itg.set_limiter(True)
    timer = _event_timer(torch.cuda.ExternalStream(itg.stream()))
    itg.step(warmup)
    itg.synchronize()
    secs = timer(lambda: itg.step(steps))
    out["learned_fp32k_midpoint_loop"] = {"value": ndof * 2 * steps / secs, "ms_per_step": secs / steps * 1e3,
                                          "note": "Midpoint + positive_limiter + learned indicator, the loop of "
                                                  "example/shock-vortex.jl:294-321; 2 RK stages per step"}
    ref = finals["plain_fp64"]
    for form in ("learned_fp32k", "plain_fp32k"):
        out[form]["rms_rho_diff_vs_plain_fp64"] = float(np.sqrt(np.mean((finals[form] - ref) ** 2)))
    # matched error: element-mean density of each form against a run on the
    # 2x refined mesh (800 x 400, plain indicator, half the step, same end time),
    # aggregated to the coarse elements
    nsteps_total = warmup + steps + 50
    psf = frgpu.FRPSpace2D(ps.x0, ps.x1, 2 * ps.nx, ps.y0, ps.y1, 2 * ps.ny, 3)
    probf = learned.shock_vortex_problem(psf, 0.25, precision="fp32k")
    itgf = frgpu.init(probf, dt=dt / 2)
    itgf.set_filter("plain", learned.FILTER_LAMBDA, S0, learned.FILTER_KAPPA)
    itgf.step(2 * nsteps_total)
    w1 = np.polynomial.legendre.leggauss(4)[1]
    W = np.outer(w1, w1) / 4

    def means(rho):
        return np.einsum("ijkl,kl->ij", rho, W)

    mf = means(itgf.u[..., 0])
    mf = 0.25 * (mf[0::2, 0::2] + mf[1::2, 0::2] + mf[0::2, 1::2] + mf[1::2, 1::2])
    errs = {form: float(np.sqrt(np.mean((means(finals[form]) - mf) ** 2))) for form in finals}
    out["rms_element_mean_rho_err_vs_refined"] = errs
    out["matched"] = {"ratio_learned_fp32k_to_plain_fp64": errs["learned_fp32k"] / errs["plain_fp64"],
                      "within_1.5x": bool(errs["learned_fp32k"] <= 1.5 * errs["plain_fp64"])}
    out["speedup_learned_fp32k_vs_plain_fp64"] = out["learned_fp32k"]["value"] / out["plain_fp64"]["value"]
    out["dt"] = dt
    out["t_end"] = nsteps_total * dt
    return out


def ensemble_entry(n=4096, t_end=0.5):
    """Config 4: 4096 Burgers instances (ne log-uniform [32,2048], p in 1..5,
    8 random Fourier modes, seed 0) to t = 0.5 in one persistent launch, tiles
    from the autotuner, FP32; the learned 1D indicator when its weights ship,
    else the plain one.  DOF updates/s = sum_i 3 ndof_i steps_i / kernel time."""
    import os as _os

    from frgpu import learned
    from frgpu.ensemble import Ensemble

    e = Ensemble.config4(n, seed=0, precision="fp32")
    have_net = _os.path.exists(learned.BURGERS_WEIGHTS)
    if have_net:
        e.set_mlp(learned.load_trained_burgers1d(), 0.5, 0.0)
    tiles = e.tune(t_probe=0.01)
    out = {"workload": f"{n} Burgers instances, ne log-uniform [32,2048], p 1..5, to t={t_end}, FP32",
           "ndof": e.ndof, "tiles": [int(t) for t in tiles],
           "indicator": "learned" if have_net else "plain"}
    e.run(t_end)
    st = e.stats()
    out["value"] = st["dof_stage_updates"] / (st["ms"] * 1e-3)
    out["ms"] = st["ms"]
    out["max_steps"] = st["max_steps"]
    out["launches_per_run"] = 1
    if have_net:
        out["indicator_stats"] = e.indicator_stats()
        s = out["indicator_stats"]
        out["misfire_rate"] = s["misfires"] / max(s["judged"], 1)
        # the same ensemble with the plain indicator, for comparison
        e2 = Ensemble.config4(n, seed=0, precision="fp32")
        e2.tiles = tiles
        e2.run(t_end)
        st2 = e2.stats()
        out["plain_indicator"] = {"value": st2["dof_stage_updates"] / (st2["ms"] * 1e-3), "ms": st2["ms"]}
    return out


def bgk_entry(steps=400, warmup=5):
    """Config 5: BGK 1D1V, 256 elements on periodic [0,1], p=3, 512 velocity
    midpoints on [-8,8], FP32, tau = Kn in {1e-4, 1e-2}, Maxwellian IC
    rho = 1 + 0.1 sin(2 pi x), U = 1, T = 1, SSPRK3 at dt = 0.1 dx / 8.
    Timed: `steps` steps; moments at t = 0.2 (4096 steps) against the FP64
    path (bit-identical to the oracle in the parity tests)."""
    import torch

    import frgpu
    from frgpu import _lib as L

    ne, nv, deg = 256, 512, 3
    dv = 16 / nv
    v = -8 + (np.arange(nv) + 0.5) * dv
    w = np.full(nv, dv)
    ps = frgpu.FRPSpace1D(0, 1, ne, deg)
    rho = 1 + 0.1 * np.sin(2 * np.pi * ps.xpg)
    f = np.zeros((ne, nv, deg + 1), order="F")
    for k in range(deg + 1):
        f[:, :, k] = rho[:, k, None] * np.sqrt(1 / np.pi) * np.exp(-(v[None, :] - 1) ** 2)
    dt = 0.1 * (1 / ne) / 8
    nfull = int(round(0.2 / dt))
    ndof = ne * nv * (deg + 1)
    out = {"workload": "BGK 1D1V 256 el x 512 vel, p=3, FP32, SSPRK3 to t=0.2", "ndof": ndof, "dt": dt,
           "steps_to_t02": nfull}

    def moments(u):
        return np.stack([np.einsum("ivk,v->ik", u, w * c) for c in (np.ones(nv), v, 0.5 * v * v)])

    for kn in (1e-2, 1e-4):
        rec = {}
        for form, precision, tensor in (("fp32_tensor", "fp32k", 1), ("fp32_cuda_cores", "fp32k", 0),
                                        ("fp64", "fp64", 0)):
            prob = frgpu.FRBGKProblem(f, (0, 1), ps, v, w, kn, precision=precision)
            if precision == "fp32k":
                prob.set_option(L.OPT_BGK_TENSOR, tensor)
            itg = frgpu.init(prob, dt=dt)
            timer = _event_timer(torch.cuda.ExternalStream(itg.stream()))
            itg.step(warmup)
            itg.synchronize()
            secs = timer(lambda: itg.step(steps))
            rec[form] = {"value": ndof * 3 * steps / secs, "stage_us": secs / (3 * steps) * 1e6}
            itg.u = f
            itg.step(nfull)
            rec[form]["moments"] = moments(itg.u)
        ref = rec["fp64"].pop("moments")
        for form in ("fp32_tensor", "fp32_cuda_cores"):
            m = rec[form].pop("moments")
            rec[form]["moment_rel_err_vs_fp64"] = [float(np.max(np.abs(m[q] - ref[q])) / np.max(np.abs(ref[q])))
                                                   for q in range(3)]
        out[f"Kn={kn:g}"] = rec
    return out


TRI_FLOP_PER_CELL_P3 = 2800      # operations of k_tri_rhs<., 3> per cell, counted from the kernel
TRI_BYTES_PER_CELL_P3 = {"fp64": 249, "fp32k": 137}  # own state + residual + geometry + neighbour tables


def tri_entry(nx=1024, steps=20, warmup=3, reps=20, forms=("fp64", "fp32k"), cpu=True):
    """Unstructured triangles: the linear-advection dudt! of
    dev/wave_triangle.jl:44-125 (a = -1) on a periodic triangulated unit square
    of 2 nx^2 right triangles, p = 3 (10 Williams-Shunn-Jameson points per
    cell, the golden tri_quadrature(3) points), SSPRK3 at dt = 0.05 h.  Timed:
    `reps` residuals of the device state and `steps` SSPRK3 steps, per form;
    the oracle's residual on all host cores over a 128 x 128 sample beside it."""
    import torch

    import frgpu

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    q = np.load(os.path.join(ROOT, "tests", "golden", "tri_quadrature.npz"))
    deg = 3
    xpl, wp = np.stack([q["r3"], q["s3"]], axis=1), q["w3"]

    def space(n):
        pts, cid, key, ct = frgpu.tri_square_mesh(n, n, periodic=True)
        return frgpu.TriFRPSpace(pts, cid, deg, xpl, wp, key, ct)

    sp = space(nx)
    X, Y = sp.xpg[..., 0], sp.xpg[..., 1]
    u = np.asfortranarray(1.0 + 0.5 * np.sin(2 * np.pi * X) * np.cos(2 * np.pi * Y))
    del X, Y
    ndof = sp.ncell * sp.np
    dt = 0.05 / nx
    out = {"workload": f"triangles: linear advection (a = -1), periodic unit square, {sp.ncell} cells "
                       f"({nx}x{nx} squares x 2), p=3, SSPRK3", "ndof": ndof, "cells": sp.ncell}
    for form in forms:
        prob = frgpu.TriAdvectionProblem(u, sp, -1.0, precision=form)
        timer = _event_timer(torch.cuda.ExternalStream(prob.stream()))
        for _ in range(warmup):
            prob.rhs_device()
        secs = timer(lambda: [prob.rhs_device() for _ in range(reps)]) / reps
        prob.step(warmup, dt)
        l0 = prob.launches()
        secs_step = timer(lambda: prob.step(steps, dt)) / steps
        rec = {"value": ndof / secs_step, "unit": "DOF-updates/s", "step_ms": secs_step * 1e3,
               "rhs_us": secs * 1e6, "rhs_dof_per_s": ndof / secs,
               "achieved_gflops": TRI_FLOP_PER_CELL_P3 * sp.ncell / secs / 1e9,
               "achieved_gbs_compulsory": TRI_BYTES_PER_CELL_P3[form] * sp.ncell / secs / 1e9,
               "launches_per_step": (prob.launches() - l0) / steps}
        peak, kind = measured_peaks()
        gbs = rec["achieved_gbs_compulsory"]
        rec["roofline"] = {"bound": "fp64 pipe" if form == "fp64" else "latency (neighbour gathers)",
                           "hbm": {"achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                                   "peak_kind": kind},
                           "flops": {"achieved": rec["achieved_gflops"] / 1e3, "unit": "TFLOP/s",
                                     "note": "FP64 against GB300's nominal 1.25 TFLOP/s FP64 (not measured)"
                                     if form == "fp64" else "FP32 CUDA cores"},
                           "kernel": f"k_tri_rhs<{'double' if form == 'fp64' else 'float'},3>"}
        out[form] = rec
        del prob
    if not cpu:
        return out
    # the oracle's residual on the host cores, on a smaller mesh
    ss = space(128)
    P = O.TriProblem(deg, -1.0, ss.dl, ss.lf, ss.phi, ss.J, ss.iJ, ss.nb_cell, ss.nb_face, ss.nb_point,
                     ss.cell_type)
    us = np.asfortranarray(1.0 + 0.5 * np.sin(2 * np.pi * ss.xpg[..., 0]))
    P.rhs(us)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < 3.0:
        P.rhs(us)
        n += 1
    cpu = ss.ncell * ss.np * n / (time.perf_counter() - t0)
    out["cpu_oracle_rhs_dof_per_s"] = {"value": cpu, "cores": O.get_threads(),
                                       "sample": f"{n} residuals of a {ss.ncell}-cell mesh, FP64 oracle"}
    return out


def cpu_baseline(target_s=12.0, nthreads=None):
    """The oracle (FP64, OpenMP) on the full 512x512 p=3 mesh, timed over as many
    SSPRK3 steps as fit in about target_s seconds (at least one)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    cores = nthreads or os.cpu_count() or 1
    O.set_threads(cores)
    po = O.Space2D(0, 1, NX, 0, 1, NY, DEG)
    u = density_wave(po.xpg)
    P = O.Problem(O.EULER2D, po, flux=O.FLUX_LF, gamma=GAMMA)
    dt = 1e-5
    t0 = time.perf_counter()
    u = P.ssprk3(u, dt, 1)
    t1 = time.perf_counter() - t0
    n = max(1, int(target_s / max(t1, 1e-3)) - 1)
    t0 = time.perf_counter()
    P.ssprk3(u, dt, n)
    secs = time.perf_counter() - t0
    return {"value": NDOF * 3 * n / secs, "unit": UNIT, "cores": O.get_threads(), "kind": "port",
            "sample": f"{n} SSPRK3 step(s) ({3 * n} RK stages) of the full 512x512 p=3 workload, FP64 oracle, "
                      f"OpenMP over elements"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    # profiling aids: run a subset of the forms (comma list of fp32k_learned,
    # fp32k, fp64_plain) and/or skip the end-to-end leg; the line then only
    # carries the forms that ran
    ap.add_argument("--forms", default="")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the shock-vortex, ensemble and BGK entries")
    # profiling aid: run one of the other workloads alone (small sizes through --steps / --instances)
    ap.add_argument("--workload", choices=["shock_vortex", "ensemble", "bgk", "triangles"], default=None)
    ap.add_argument("--instances", type=int, default=4096)
    ap.add_argument("--tri-nx", type=int, default=1024, help="triangles: squares per side (2 nx^2 cells)")
    args = ap.parse_args()
    ws, rank, _ = dist_env()
    dist = init_dist(ws)

    if args.workload is not None:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        if args.workload == "shock_vortex":
            r = shock_vortex_entry(steps=args.steps, warmup=args.warmup)
        elif args.workload == "ensemble":
            r = ensemble_entry(n=args.instances, t_end=0.5)
        elif args.workload == "triangles":
            # FP32K first, so that a profiler's first residual launch is the FP32K one
            r = tri_entry(nx=args.tri_nx, steps=args.steps, warmup=args.warmup, reps=args.steps,
                          forms=("fp32k", "fp64"), cpu=False)
        else:
            r = bgk_entry(steps=args.steps, warmup=args.warmup)
        print(json.dumps({"partial_run": True, "workload": args.workload, "result": r}), flush=True)
        return

    if args.impl == "reference":
        if rank != 0:
            return
        K = max(1, args.steps)
        cb = cpu_baseline(target_s=min(60.0, 0.5 * (K + args.warmup)))
        line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": NDOF * 3 / cb["value"] * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": {"workload": WORKLOAD, "form": "reference CPU algorithm (oracle port)"},
                "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    res, clocks = gpu_arm(args, dist, rank, ws)
    if rank != 0:
        return
    if args.forms or args.no_e2e:
        print(json.dumps({"metric": METRIC, "unit": UNIT, "partial_run": True, "forms": res, "clocks": clocks}),
              flush=True)
        return
    peak, peak_kind = measured_peaks()
    lrn = res["fp32k_learned"]
    f32 = res["fp32k"]
    f64 = res["fp64_plain"]
    bytes_launch = NDOF * BYTES_PER_DOF_STAGE["fp32k"]
    achieved = bytes_launch / (f32["stage_us"] * 1e-6) / 1e9
    traffic = NCU_TRAFFIC_PER_LAUNCH["fp32k"]
    ratio = lrn["rms_err_rho_vs_exact"] / max(f64["rms_err_rho_vs_exact"], 1e-300)
    line = {
        "metric": METRIC, "value": lrn["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": lrn["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "form": "learned indicator + FP32 residual with compensated SSPRK3 "
                   "combination; the :l2 modal filter runs after every step",
                   "ndof": NDOF, "dt": lrn["dt"], "l2_flush": "inputs larger than L2: every stage streams "
                   ">= 2 state arrays of 67 MB (FP32) / 134 MB (FP64)", "parallelism": f"replicas x{ws}"},
        "fp64_plain": {"value": f64["value"], "ms_per_step": f64["ms_per_step"], "dtype": "f64",
                       "rms_err_rho_vs_exact": f64["rms_err_rho_vs_exact"],
                       "note": "plain FP64 residual + plain modal-decay indicator and filter every step"},
        "fp32k_no_indicator": {"value": f32["value"], "ms_per_step": f32["ms_per_step"],
                               "stage_us": f32["stage_us"]},
        "speedup_vs_fp64_plain": lrn["value"] / f64["value"],
        "accuracy": {"rms_err_rho_vs_exact": {"learned_fp32k": lrn["rms_err_rho_vs_exact"],
                                              "fp64_plain": f64["rms_err_rho_vs_exact"]},
                     "ratio": ratio, "matched": bool(ratio <= 1.5),
                     "troubled_last_step": {"learned_fp32k": lrn["troubled_last_step"],
                                            "fp64_plain": f64["troubled_last_step"]}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": "k_euler2d<float,4,LF,FP32K,stage> (fused residual + SSPRK3 stage)",
                     "bytes_per_launch": bytes_launch},
        "e2e": res["e2e"],
        "gpu_launches": lrn["launches_timed"],
        "clocks": clocks,
    }
    if not args.no_configs:
        # the other workloads of the spec, each on its own clock (not part of `value`)
        line["configs"] = {}
        for name, fn in (("shock_vortex_400x200_p3", shock_vortex_entry), ("burgers_ensemble_4096", ensemble_entry),
                         ("bgk_256x512_p3", bgk_entry), ("triangles_advection_2M_cells_p3", tri_entry)):
            try:
                line["configs"][name] = fn()
            except Exception as e:  # report, do not lose the headline line
                line["configs"][name] = {"error": f"{type(e).__name__}: {e}"}
    if not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = cpu_baseline()
        except Exception as e:  # the oracle needs gcc on the host
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {e}"}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
