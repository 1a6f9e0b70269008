#!/usr/bin/env python3
"""Benchmark: RK-stage DOF-updates/s of the flux-reconstruction hot path.

Headline workload (one GPU): the 2D Euler shock-vortex on [0,2] x [0,1] with
400 x 200 quadrilaterals, p = 3 (16 solution points per element, 5,120,000
DOFs), gamma = 1.4, a stationary Mach 1.1 normal shock at x = 0.5 and a Mach
0.25 isentropic vortex of radius 0.075 at (0.25, 0.5), HLL interface flux,
fixed inflow on the left and copy ghosts elsewhere, the troubled-cell
indicator + :l2 modal filter after every step (example/shock-vortex.jl:294-330
with SSPRK3), SSPRK3 at CFL 0.1.  One bench "step" is one SSPRK3 time step
(three fused residual + stage launches, the indicator and filter fused into the
third) over the whole mesh.

* ``value``      learned indicator + FP32 residual with compensated stage sums
                 (FP32K), device-resident, CUDA-event timed per step with L2
                 flushed before every step (the 20 MB state would otherwise stay
                 in the 129 MB L2).
* ``accuracy``   each form's density error (src/tools.jl:47-53 L2 and L-inf,
                 and the quadrature L2) against a converged FP64 solution (the
                 FP64 form on the 2x refined mesh), the matched-error ratio
                 learned FP32K / plain FP64 (target <= 1.5), and each form's
                 difference from the FP64 oracle on the same mesh.
* ``e2e``        the headline form through the C ABI with host buffers: state
                 uploaded from page-locked host memory, every step's dt written
                 and its FP64 conserved sums read back, the state downloaded at
                 the end.  ``e2e_rhs`` times the drop-in rhs!(du, u, p, t) with
                 host FP64 arrays per residual call (the path of
                 OrdinaryDiffEq's solve with host arrays).
* ``roofline``   HBM roofline of the fused FP32K stage kernel on the 512 x 512
                 density wave (the workload the HBM target is set on); the
                 headline kernel's own figures sit in ``configs``.
* ``cpu_baseline`` the CPU FP64 oracle (OpenMP over all host cores) running the
                 plain form of the headline workload; its final state also
                 checks the FP64 GPU form bit for bit.

``--impl reference`` times the reference's CPU algorithm (the oracle port; the
Julia reference cannot run here) on the same config, metric and unit.
Multi-GPU: the path is run as independent replicas (one per rank, no
collective on the data path); ``value`` sums the replicas' DOFs over the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes
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
GAMMA = 1.4
CFL = 0.1
DEG = 3
NP = DEG + 1
# headline: shock-vortex 400 x 200
SV_NX, SV_NY = 400, 200
SV_NDOF = SV_NX * SV_NY * NP * NP * 4
SV_MACH = 0.25
WORKLOAD = ("2D Euler shock-vortex on [0,2]x[0,1], 400x200 quads, p=3, HLL flux, stationary Mach 1.1 normal shock "
            "at x=0.5 + Mach 0.25 isentropic vortex (r=0.075) at (0.25,0.5), indicator + :l2 modal filter after "
            "every step, SSPRK3 at CFL 0.1")
# density wave 512 x 512: the roofline workload
NX = NY = 512
NDOF = NX * NY * NP * NP * 4
WAVE_WORKLOAD = "2D Euler density wave, periodic [0,1]^2, 512x512 quads, p=3, LF flux, SSPRK3 at CFL 0.1"
# filter of example/shock-vortex.jl:308-321
LAM, KAPPA = 5e-4, 9.0
S0 = -3.0 * math.log10(DEG)
# Algorithmic HBM bytes per DOF per RK stage of a fused SSPRK3 step: 8/3 state
# arrays per stage on average (stage 1 reads u^n and writes u1; stages 2 and 3
# read u^n and the stage input and write the result).
BYTES_PER_DOF_STAGE = {"fp32k": 4 * 8 / 3, "fp64": 8 * 8 / 3}
# DRAM bytes (read + write) per stage launch of the bare FP32K stage kernel on
# the 512 x 512 density wave, mean over the three SSPRK3 stages, from the ncu
# capture summarised in profiles/euler2d_stage_tiles16x4_512x512_p3.md.
NCU_TRAFFIC_PER_LAUNCH = {"fp32k": 187.0e6, "fp64": None}
L2_FLUSH_BYTES = 512 << 20  # four times the 129 MB L2


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


def rms(a, b):
    d = np.asarray(a) - np.asarray(b)
    return float(np.sqrt(np.mean(d * d)))


def host_cfl_dt(u, dx, dy, cfl=CFL, g=GAMMA):
    """dt = cfl / max over points of (|u| + c)/dx + (|v| + c)/dy, on the host, so
    that both arms of the bench and the oracle take the same step."""
    U = u[..., 1] / u[..., 0]
    V = u[..., 2] / u[..., 0]
    p = (g - 1) * (u[..., 3] - 0.5 * (u[..., 1] * U + u[..., 2] * V))
    c = np.sqrt(g * p / u[..., 0])
    return cfl / float(np.max((np.abs(U) + c) / dx + (np.abs(V) + c) / dy))


def shock_vortex_initial(xpg):
    from frgpu import learned  # numpy only: the initial state and inflow of the workload

    return learned.shock_vortex_state(xpg, SV_MACH, GAMMA)


def sv_space_host():
    """Element centres and solution points of the 400 x 200 mesh without the library."""
    xpl = np.polynomial.legendre.leggauss(NP)[0]
    dx, dy = 2.0 / SV_NX, 1.0 / SV_NY
    xc = (np.arange(SV_NX) + 0.5) * dx
    yc = (np.arange(SV_NY) + 0.5) * dy
    X = xc[:, None, None, None] + 0.5 * dx * xpl[None, None, :, None]
    Y = yc[None, :, None, None] + 0.5 * dy * xpl[None, None, None, :]
    return np.stack(np.broadcast_arrays(X, Y), axis=-1), dx, dy


def headline_config(dt, ws):
    return {"workload": WORKLOAD, "mesh": [SV_NX, SV_NY], "deg": DEG, "ndof": SV_NDOF, "dt": dt,
            "l2_flush": "L2 flushed before every timed step (a 512 MB device buffer written): the 20 MB FP32 "
                        "state would otherwise stay L2-resident",
            "parallelism": f"replicas x{ws}"}


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


class L2Flush:
    """Writes a device buffer four times the size of L2 on a stream, so that the
    next launch starts from a cold L2."""

    def __init__(self):
        import torch

        self.torch = torch
        self.buf = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def __call__(self, stream):
        with self.torch.cuda.stream(stream):
            self.buf.fill_(1.0)


def flushed_steps(itg, K, stream, flush):
    """K steps, each queued (without a host wait) between two CUDA events after
    an L2 flush; returns the summed device seconds of the steps.  The status of
    all K steps is checked once at the end."""
    import torch

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    for a, b in ev:
        flush(stream)
        a.record(stream)
        itg.step_async(1)
        b.record(stream)
    itg.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / 1e3


def pinned(torch, shape):
    """A page-locked host FP64 array of the reference layout (the copy engine
    reads and writes it directly)."""
    t = torch.empty(int(np.prod(shape)), dtype=torch.float64, pin_memory=True)
    return t.numpy().reshape(shape, order="F")


def same_ops(oracle_space, gpu_space):
    """Give the oracle the library's operator values (the two setup codes agree
    to the last bit or so), so that residuals and steps compare bit for bit."""
    for f in ("ll", "lr", "dl", "dhl", "dhr", "V", "iV", "wp"):
        setattr(oracle_space, f, np.array(getattr(gpu_space, f), dtype=np.float64))
    return oracle_space


# --------------------------------------------------------------------------- headline arm
SV_FORMS = (("learned_fp32k", "fp32k", "mlp"), ("plain_fp32k", "fp32k", "plain"), ("plain_fp64", "fp64", "plain"))


def sv_problem(ps, precision, indicator, net, dt):
    import frgpu
    from frgpu import learned

    prob = learned.shock_vortex_problem(ps, SV_MACH, precision=precision)
    itg = frgpu.init(prob, dt=dt)
    if indicator == "mlp":
        frgpu._lib.check(frgpu.lib().frgpu_problem_set_mlp(prob._h, net._h, learned.DECISION_THRESHOLD, 0.0))
    itg.set_filter(indicator, LAM, S0, KAPPA)
    return prob, itg


def headline_arm(args, dist, rank, ws, dt):
    """The three forms of the shock-vortex workload: timed steps (L2 flushed
    before each), e2e through the ABI, the drop-in rhs! with host arrays, and
    the accuracy runs (acc_steps from the initial state; a 2x refined FP64 run
    is the converged solution)."""
    import torch

    import frgpu
    from frgpu import learned

    ps = learned.config3_space()
    net = learned.load_trained()
    u0 = learned.shock_vortex_state(ps.xpg, SV_MACH, GAMMA)[0]
    K, W = args.steps, args.warmup
    flush = L2Flush()
    out = {}
    for form, precision, ind in SV_FORMS:
        prob, itg = sv_problem(ps, precision, ind, net, dt)
        stream = torch.cuda.ExternalStream(itg.stream())
        if W:
            itg.step(W)
        itg.synchronize()
        torch.cuda.synchronize()
        barrier(dist)
        l0 = itg.launches()
        secs = flushed_steps(itg, K, stream, flush)
        launches = itg.launches() - l0
        torch.cuda.synchronize()
        barrier(dist)
        secs = max_over_ranks(dist, secs)
        rec = {"value": SV_NDOF * 3 * K * ws / secs, "ms_per_step": secs / K * 1e3, "launches_timed": launches,
               "precision": precision, "indicator": ind}
        if ind == "mlp":
            st = np.zeros(3, dtype=np.int32)
            frgpu._lib.check(frgpu.lib().frgpu_indicator_stats(prob._h, st.ctypes.data_as(frgpu._lib._I)))
            rec["last_step_troubled_misfires_fallbacks"] = [int(x) for x in st]
        out[form] = rec
        if form == "learned_fp32k" and not args.no_e2e:
            out["e2e"] = e2e_integrator(torch, itg, u0, K, stream, flush, dist, ws, W)
        del itg, prob
    if not args.no_e2e:
        out["e2e_rhs"] = e2e_rhs(torch, ps, u0, K, flush, dist, ws)
    out["accuracy_runs"] = accuracy_runs(ps, net, dt, args.acc_steps)
    return out


def e2e_integrator(torch, itg, u0, K, stream, flush, dist, ws, W=0):
    """The headline form end to end through the public API: the state uploaded
    from a page-locked host FP64 array, K steps each queued and then reading
    back its status word with its FP64 conserved sums and wave speed in one
    synchronisation (frgpu_step_ssprk3_async + frgpu_reduce, which reports the
    step's status), the state downloaded at the end.  L2 is flushed before each
    step, outside the timing.  W untimed warm-up steps of the same calls come
    first (they capture the reduction's graphs of both state buffers)."""
    host_u, host_out = pinned(torch, u0.shape), pinned(torch, u0.shape)
    host_u[...] = u0
    for _ in range(W):
        itg.step_async(1)
        itg.reduce()
    itg.synchronize()
    barrier(dist)
    secs = 0.0
    t0 = time.perf_counter()
    itg.u = host_u                              # H2D of the state
    secs += time.perf_counter() - t0
    for _ in range(K):
        flush(stream)
        itg.synchronize()
        t0 = time.perf_counter()
        itg.step_async(1)                       # one step queued (dt already on the device)
        itg.reduce()                            # D2H of the status word + FP64 sums + wave speed
        secs += time.perf_counter() - t0
    t0 = time.perf_counter()
    itg.read_u(host_out)                        # D2H of the state
    secs += time.perf_counter() - t0
    secs = max_over_ranks(dist, secs)
    state_bytes = SV_NDOF * 8
    # per step: the 4-byte status word (frgpu_step_ssprk3) and the 6 doubles of
    # frgpu_reduce come back; dt is written once (it does not change)
    return {"value": SV_NDOF * 3 * K * ws / secs, "unit": UNIT,
            "h2d_bytes_per_step": (state_bytes + 8) / K,
            "d2h_bytes_per_step": (state_bytes + (4 + 6 * 8) * K) / K,
            "note": "learned FP32K form through the C ABI: state uploaded from and downloaded to page-locked host "
                    "FP64 arrays once per K steps; every step reads back its status word and the FP64 conserved "
                    "sums and wave speed; host wall-clock, L2 flushed before every step outside the timing"}


def e2e_rhs(torch, ps, u0, K, flush, dist, ws):
    """The drop-in rhs!(du, u, p, t) (frgpu_rhs) with page-locked host FP64
    arrays, called once per RK stage as OrdinaryDiffEq's solve does with host
    arrays: every call copies u to the device, evaluates the residual and copies
    du back.  The stage combination on the host is the caller's and is not
    timed.  DOF-updates/s = DOFs / seconds per call."""
    import frgpu
    from frgpu import learned

    res = {}
    n = max(3, 3 * min(K, 20))
    for precision in ("fp64", "fp32k"):
        prob = learned.shock_vortex_problem(ps, SV_MACH, precision=precision)
        u, du = pinned(torch, u0.shape), pinned(torch, u0.shape)
        u[...] = u0
        h = ctypes.c_void_p()
        frgpu._lib.check(frgpu.lib().frgpu_problem_stream(prob._h, ctypes.byref(h)))
        stream = torch.cuda.ExternalStream(h.value)
        prob.f(du, u)
        secs = 0.0
        for _ in range(n):
            flush(stream)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            prob.f(du, u)
            secs += time.perf_counter() - t0
        secs = max_over_ranks(dist, secs)
        res[precision] = {"value": SV_NDOF * n * ws / secs, "unit": UNIT, "us_per_call": secs / n * 1e6,
                          "h2d_bytes_per_call": SV_NDOF * 8, "d2h_bytes_per_call": SV_NDOF * 8}
        del prob
    res["note"] = ("frgpu_rhs with page-locked host FP64 arrays u and du in the reference layout, one call per RK "
                   "stage; the host-side stage combination is not timed; L2 flushed before every call")
    return res


def accuracy_runs(ps, net, dt, nsteps):
    """acc_steps steps of each form from the initial state; the converged
    solution is the FP64 form (plain indicator) on the 2x refined mesh (800 x
    400, dt / 2, 2 acc_steps steps), evaluated at the coarse solution points."""
    import frgpu

    finals = {}
    stats = {}
    for form, precision, ind in SV_FORMS:
        prob, itg = sv_problem(ps, precision, ind, net, dt)
        st = np.zeros(3, dtype=np.int32)
        trb = mis = fb = 0
        for _ in range(nsteps):
            itg.step(1)
            frgpu._lib.check(frgpu.lib().frgpu_indicator_stats(prob._h, st.ctypes.data_as(frgpu._lib._I)))
            trb += int(st[0])
            if ind == "mlp":
                mis, fb = mis + int(st[1]), fb + int(st[2])
        stats[form] = {"filterings": trb, "troubled_per_step": trb / nsteps}
        if ind == "mlp":
            stats[form].update({"misfire_rate": mis / (nsteps * ps.nx * ps.ny),
                                "fallback_rate": fb / (nsteps * ps.nx * ps.ny)})
        finals[form] = itg.u
        del itg, prob
    from frgpu import learned

    psf = frgpu.FRPSpace2D(ps.x0, ps.x1, 2 * ps.nx, ps.y0, ps.y1, 2 * ps.ny, DEG)
    prob, itg = sv_problem(psf, "fp64", "plain", net, dt / 2)
    itg.step(2 * nsteps)
    truth = frgpu.refined_at_coarse_points(itg.u, ps.xpl)
    del itg, prob
    return finals, truth, stats


def accuracy_report(ps, finals, truth, stats, oracle_final=None):
    """Density errors (variable 1, as the reference's examples report them) of
    each form against the converged solution, in the src/tools.jl:47-53 forms
    (dx = the element area) and as the quadrature L2; the matched-error ratio;
    and, given the oracle's final state on the same mesh, each form's
    difference from it."""
    import frgpu

    w1 = np.polynomial.legendre.leggauss(NP)[1]
    area = ps.dx * ps.dy
    rep = {"truth": "FP64 form, plain indicator, on the 2x refined mesh (800x400, dt/2, same end time), evaluated "
                    "at the 400x200 solution points; the FP64 form is bit-identical to the FP64 oracle "
                    "(tests/test_parity_full.py)",
           "variable": "density", "forms": {}}
    for form, u in finals.items():
        r, t = u[..., 0], truth[..., 0]
        rep["forms"][form] = {"L2_quadrature": frgpu.quadrature_L2_error(r, t, ps.dx, ps.dy, w1),
                              "L2_tools_jl": frgpu.L2_error(r, t, area),
                              "Linf_tools_jl": frgpu.Linf_error(r, t, area), **stats.get(form, {})}
    e = {f: v["L2_quadrature"] for f, v in rep["forms"].items()}
    ratio = e["learned_fp32k"] / max(e["plain_fp64"], 1e-300)
    rep["matched"] = {"ratio_learned_fp32k_to_plain_fp64": ratio, "bound": 1.5, "matched": bool(ratio <= 1.5),
                      "ratio_plain_fp32k_to_plain_fp64": e["plain_fp32k"] / max(e["plain_fp64"], 1e-300)}
    fl = {f: v.get("filterings") for f, v in rep["forms"].items()}
    if fl.get("learned_fp32k") is not None and fl.get("plain_fp32k"):
        rep["learned_vs_plain_fp32k"] = {
            "filterings_ratio": fl["learned_fp32k"] / fl["plain_fp32k"],
            "l2_error_ratio": e["learned_fp32k"] / max(e["plain_fp32k"], 1e-300),
            "note": "both indicators fused into the third stage on the same features; the network's gain is "
                    "fewer filter applications at the plain test's accuracy"}
    if oracle_final is not None:
        ref = oracle_final
        scale = float(np.max(np.abs(ref)))
        rep["vs_fp64_oracle_same_mesh"] = {
            f: {"bit_identical": bool(np.array_equal(u, ref)),
                "L2_rel": float(np.sqrt(np.mean((u - ref) ** 2)) / scale),
                "Linf_rel": float(np.max(np.abs(u - ref)) / scale)} for f, u in finals.items()}
    return rep


# --------------------------------------------------------------------------- density wave (roofline)
def density_wave_entry(args, dist, ws):
    """The 512 x 512 density wave: the bare FP32K stage kernels (the roofline
    entry), the learned FP32K form and the plain FP64 form with the indicator
    and filter every step; each timed over K steps of one graph replay loop
    (every stage streams more than L2 holds)."""
    import torch

    import frgpu
    from frgpu import learned

    ps = frgpu.FRPSpace2D(0, 1, NX, 0, 1, NY, DEG)
    u0 = density_wave(ps.xpg)
    K, W = args.steps, args.warmup
    net = learned.load_trained()
    out = {"workload": WAVE_WORKLOAD, "ndof": NDOF}
    for form, precision, indicator in (("fp32k", "fp32k", "none"), ("fp32k_learned", "fp32k", "mlp"),
                                       ("fp64", "fp64", "none"), ("fp64_plain", "fp64", "plain")):
        prob = frgpu.FREuler2DProblem(u0, (0, 1), ps, GAMMA, flux="lf", bc="period", precision=precision)
        itg = frgpu.init(prob, dt=1.0)
        dt = itg.cfl_dt(CFL)
        itg.dt = dt
        if indicator == "mlp":
            frgpu._lib.check(frgpu.lib().frgpu_problem_set_mlp(prob._h, net._h, learned.DECISION_THRESHOLD, 0.0))
        if indicator != "none":
            itg.set_filter(indicator, LAM, S0, KAPPA)
        timer = _event_timer(torch.cuda.ExternalStream(itg.stream()))
        secs = run_replicas(lambda n: itg.step(n), K, W, itg.synchronize, dist, timer)
        t_end = (W + K) * dt
        out[form] = {"value": NDOF * 3 * K * ws / secs, "ms_per_step": secs / K * 1e3,
                     "stage_us": secs / (3 * K) * 1e6, "dt": dt,
                     "rms_err_rho_vs_exact": rms(itg.u[..., 0], exact_density(ps.xpg, t_end))}
        del itg, prob
    peak, kind = measured_peaks()
    bytes_launch = NDOF * BYTES_PER_DOF_STAGE["fp32k"]
    achieved = bytes_launch / (out["fp32k"]["stage_us"] * 1e-6) / 1e9
    out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                       "traffic": NCU_TRAFFIC_PER_LAUNCH["fp32k"], "peak_kind": peak_kind_label(kind),
                       "kernel": "k_euler2d<float,4,LF,FP32K,stage> (fused residual + SSPRK3 stage)",
                       "workload": WAVE_WORKLOAD, "bytes_per_launch": bytes_launch,
                       "bytes_per_dof_stage": BYTES_PER_DOF_STAGE["fp32k"]}
    p64 = FMA_PEAKS.get("fp64", 0.0)
    fl = E2D_FP64_FLOP_PER_DOF_STAGE * NDOF / (out["fp64"]["stage_us"] * 1e-6)
    out["fp64_roofline"] = {"bound": "fp64 pipe", "achieved": fl / 1e12, "peak": p64 / 1e12, "unit": "TFLOP/s",
                            "frac": fl / max(p64, 1.0), "flop_per_dof_stage": E2D_FP64_FLOP_PER_DOF_STAGE,
                            "kernel": "k_euler2d<double,4,LF,FP64,stage>",
                            "peak_kind": "measured (frgpu_fma_peak, FP64 FMA, this run)"}
    out["accuracy_note"] = ("FP32K's error here is its rounding floor (about 2e-7 RMS in density against the exact "
                            "solution), FP64's is round-off (about 5e-13): the discretisation error of p = 3 on "
                            "512^2 over t < 0.01 is below both, so the matched-error gate applies to the shock-vortex "
                            "workload instead")
    return out


FMA_PEAKS = {}


def indicator_entry(steps=50, warmup=5):
    """The troubled-cell indicators on the shock-vortex workload (400 x 200, p = 3,
    FP32K): ms per SSPRK3 step (L2 flushed before each) with the learned network
    fused into the third stage (warp-level mma.sync), with the network as a
    kernel of its own after the step (tcgen05 tensor cores, TMEM accumulators),
    and with the plain modal-decay test fused."""
    import torch

    import frgpu
    from frgpu import _lib as L
    from frgpu import learned

    ps = learned.config3_space()
    net = learned.load_trained()
    xpg, dx, dy = sv_space_host()
    dt = host_cfl_dt(shock_vortex_initial(xpg)[0], dx, dy)
    flush = L2Flush()
    out = {"workload": WORKLOAD}
    for name, ind, fuse in (("learned_fused_mma_sync", "mlp", 1), ("learned_separate_tcgen05", "mlp", 0),
                            ("plain_fused", "plain", 1)):
        prob, itg = sv_problem(ps, "fp32k", ind, net, dt)
        prob.set_option(L.OPT_FUSED_INDICATOR, fuse)
        itg.step(warmup)
        itg.synchronize()
        st = torch.cuda.ExternalStream(itg.stream())
        out[name] = {"ms_per_step": flushed_steps(itg, steps, st, flush) / steps * 1e3}
        del itg, prob
    return out


def measure_fma_peaks():
    """FP64 / FP32 / FP32-pair FMA throughput of this GPU (frgpu_fma_peak)."""
    import frgpu

    for k in ("fp64", "fp32", "fp32x2"):
        FMA_PEAKS[k] = frgpu.fma_peak(k)
    return {"fp64": FMA_PEAKS["fp64"] / 1e12, "fp32": FMA_PEAKS["fp32"] / 1e12, "fp32x2": FMA_PEAKS["fp32x2"] / 1e12,
            "unit": "TFLOP/s", "how": "8 independent FMA chains per thread, 8 CTAs of 256 threads per SM, best of "
                                      "3 CUDA-event timed launches after one warm-up"}


def peak_kind_label(kind):
    return "measured (MEASURED_PEAKS.json hbm_gbs)" if kind == "measured" else "fallback"


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
        out["learned_vs_plain"] = {
            "throughput_ratio": out["value"] / out["plain_indicator"]["value"],
            "note": "a loss on this workload: the 1D plain test is a 6-point modal transform per element, the "
                    "network 12 kFLOP per element; elements in the plain test's sigma = 1 region skip the network "
                    "(76-84 % of the 16-element halves), the network reproduces the plain decisions on the rest "
                    "(misfire rate above) and saves no filter work here"}
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
        for form, precision, tensor in (("fp32_tensor", "fp32k", 1), ("fp32_tcgen05", "fp32k", 2),
                                        ("fp32_cuda_cores", "fp32k", 0), ("fp64", "fp64", 0)):
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
        for form in ("fp32_tensor", "fp32_tcgen05", "fp32_cuda_cores"):
            m = rec[form].pop("moments")
            rec[form]["moment_rel_err_vs_fp64"] = [float(np.max(np.abs(m[q] - ref[q])) / np.max(np.abs(ref[q])))
                                                   for q in range(3)]
        out[f"Kn={kn:g}"] = rec
    return out


def dev_scripts_entry(cpu=True):
    """Two reference scripts through their drop-in paths, FP64, wall clock per
    step on the device against the oracle on all host cores:
    * example/advection_kinetic.jl: the kinetic problem (100 elements on
      [-1, 1], p = 2, 28 velocities, density-only BGK closure, tau = 0.002) to
      t = 0.5 at the script's dt = 0.0005 with a stabilised method (RKC2: the
      spectral radius by the power method, then the stage count, every step, as
      ROCK4 does); 1000 steps on the GPU, a 100-step sample on the oracle;
    * dev/curve_euler.jl: the polar grid's 58 x 48 active elements, p = 2, its
      central flux with c = 40 dt, Midpoint at dt = 0.002, the script's 50 steps
      (the oracle runs the same 50; the two final states are compared)."""
    import frgpu

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    out = {}
    # advection_kinetic.jl
    nx, deg, nu = 100, 2, 28
    ps = frgpu.FRPSpace1D(-1, 1, nx, deg)
    dv = 10 / nu
    v = -5 + (np.arange(nu) + 0.5) * dv
    w = np.full(nu, dv)
    rho0 = 1 - np.sin(np.pi * ps.xpg)
    f = np.zeros((nx, nu, deg + 1), order="F")
    for k in range(deg + 1):
        f[:, :, k] = rho0[:, k, None] * np.sqrt(1 / np.pi) * np.exp(-(v[None, :] - 1.0) ** 2)
    dt, n = 0.0005, 1000
    itg = frgpu.init(frgpu.FRBGKProblem(f, (0, 0.5), ps, v, w, 0.002, closure="density", a=1.0), frgpu.RKC2(),
                     dt=dt)
    itg.step(5)
    itg.u = f
    itg.stages = []
    t0 = time.perf_counter()
    itg.step(n)
    gpu_s = time.perf_counter() - t0
    rec = {"workload": "advection_kinetic.jl: 100 el x 28 vel, p=2, tau=0.002, RKC2 at dt=0.0005 to t=0.5",
           "ndof": int(f.size), "steps": n, "gpu_ms_per_step": gpu_s / n * 1e3,
           "stages_used": sorted(set(int(x) for x in itg.stages)),
           "gpu_dof_updates_per_s": f.size * float(np.mean(itg.stages)) * n / gpu_s}
    if cpu:
        po = same_ops(O.Space1D(-1, 1, nx, deg), ps)
        po.J = np.array(ps.J)
        P = O.Problem(O.BGK1D, po, tau=0.002, a=1.0, velo=v, weights=w, bgk_closure=1)
        alg = frgpu.RKC2()
        u, d = f.copy(order="F"), None
        m = 100
        t0 = time.perf_counter()
        for _ in range(m):
            r, _, d = P.spectral_radius(u, alg.maxiter, d)
            al, be, mu, de, _, _ = alg.coefficients(dt * r)
            u = P.rock(u, dt, 1, al, be, mu, de)
        rec["cpu_ms_per_step"] = (time.perf_counter() - t0) / m * 1e3
        rec["cpu_sample"] = f"{m} steps on the oracle, {O.get_threads()} threads"
        rec["gpu_vs_cpu"] = rec["cpu_ms_per_step"] / rec["gpu_ms_per_step"]
    out["advection_kinetic"] = rec
    # curve_euler.jl
    nr, nt, deg = 60, 50, 2
    G_CURVE, C_DISS = 5 / 3, 40 * 0.002
    ps2 = frgpu.FRPSpace2D(0, 1, nr, 0, 1, nt, deg)
    V = frgpu.polar_vertices(1.0, 6.0, nr, 0.0, np.pi, nt)
    iJ = frgpu.quad_metric(ps2.xpl, V)
    xpg = frgpu.quad_points(ps2.xpl, V)
    # the script's u0: a density bump at (0, 3), at rest, prim = [rho, 0, 0, 1] (p = rho / 2)
    rho = np.maximum(np.exp(-10 * (xpg[..., 0] ** 2 + (xpg[..., 1] - 3.0) ** 2)), 1e-2)
    u0 = np.zeros(rho.shape + (4,), order="F")
    u0[..., 0] = rho
    u0[..., 3] = 0.5 * rho / (G_CURVE - 1)
    ub = np.asfortranarray(u0[:nr - 2, :nt - 2])
    iJb = np.asfortranarray(iJ[:nr - 2, :nt - 2])
    psb = frgpu.FRPSpace2D(0, 1, nr - 2, 0, 1, nt - 2, deg)
    prob = frgpu.FREuler2DProblem(ub, (0, 1), psb, G_CURVE, flux="central", bc="dirichlet")
    prob.set_metric(iJb)
    prob.set_flux_dissipation(C_DISS)
    mid = frgpu.Midpoint()
    itg = frgpu.init(prob, mid, dt=0.002)
    itg.step(3)
    itg.u = ub
    itg.synchronize()
    t0 = time.perf_counter()
    itg.step(50)
    itg.synchronize()
    gpu_s = time.perf_counter() - t0
    rec = {"workload": "curve_euler.jl: 58 x 48 active elements of the polar grid, p=2, central flux, Midpoint "
                       "at dt=0.002, 50 steps", "ndof": int(ub.size), "gpu_ms_per_step": gpu_s / 50 * 1e3}
    if cpu:
        po2 = same_ops(O.Space2D(0, 1, nr - 2, 0, 1, nt - 2, deg), psb)
        P2 = O.Problem(O.EULER2D, po2, gamma=G_CURVE, flux=O.FLUX_CENTRAL, bc=O.BC_DIRICHLET, flux_c=C_DISS)
        P2.set_metric(iJb)
        t0 = time.perf_counter()
        ref = P2.erk(ub, 0.002, 50, mid.A, mid.b)
        rec["cpu_ms_per_step"] = (time.perf_counter() - t0) / 50 * 1e3
        rec["gpu_vs_cpu"] = rec["cpu_ms_per_step"] / rec["gpu_ms_per_step"]
        rec["bit_identical_to_oracle"] = bool(np.array_equal(itg.u, ref))
    out["curve_euler"] = rec
    return out


# FP64 floating-point operations (dadd + dmul + 2 dfma, ncu instruction counters;
# profiles/fp64_flops_512x512_p3.md): k_tri_rhs<double, 3> per cell, and the
# 2D Euler stage kernel k_euler2d<double, 4, LF, FP64, stage> per DOF and stage
# (mean of the three SSPRK3 stages on the 512 x 512 density wave)
TRI_FLOP_PER_CELL_P3 = 3090
E2D_FP64_FLOP_PER_DOF_STAGE = 70.8
TRI_BYTES_PER_CELL_P3 = {"fp64": 249, "fp32k": 137}  # own state + residual + geometry + neighbour tables


def tri_entry(nx=1024, steps=20, warmup=3, reps=20, forms=("fp64", "fp32k"), cpu=True):
    """Unstructured triangles: the linear-advection dudt! of
    dev/wave_triangle.jl:44-125 (a = -1) on a periodic triangulated unit square
    of 2 nx^2 right triangles, p = 3 (10 Williams-Shunn-Jameson points per
    cell, tri_quadrature(3)), SSPRK3 at dt = 0.05 h.  Timed:
    `reps` residuals of the device state and `steps` SSPRK3 steps, per form;
    the oracle's residual on all host cores over a 128 x 128 sample beside it."""
    import torch

    import frgpu

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    deg = 3

    def space(n):
        pts, cid, key, ct = frgpu.tri_square_mesh(n, n, periodic=True)
        return frgpu.TriFRPSpace(pts, cid, deg, key=key, cell_type=ct)

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
               "flops_per_cell": TRI_FLOP_PER_CELL_P3,
               "achieved_gbs_compulsory": TRI_BYTES_PER_CELL_P3[form] * sp.ncell / secs / 1e9,
               "launches_per_step": (prob.launches() - l0) / steps}
        peak, kind = measured_peaks()
        gbs = rec["achieved_gbs_compulsory"]
        rec["roofline"] = {"bound": "fp64 pipe" if form == "fp64" else "latency (neighbour gathers)",
                           "hbm": {"achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                                   "peak_kind": kind},
                           "flops": {"achieved": rec["achieved_gflops"] / 1e3, "unit": "TFLOP/s",
                                     "peak": FMA_PEAKS.get(form == "fp64" and "fp64" or "fp32x2", 0) / 1e12,
                                     "frac": rec["achieved_gflops"] * 1e9 /
                                     max(FMA_PEAKS.get(form == "fp64" and "fp64" or "fp32x2", 0), 1.0),
                                     "note": "against the FMA throughput measured by frgpu_fma_peak in this run"
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


def headline_cpu(dt, nsteps, gpu_space=None, nthreads=None):
    """The oracle (FP64, OpenMP over all host cores) on the headline workload's
    plain form: nsteps of (SSPRK3 step, plain indicator + :l2 filter), the loop
    of example/shock-vortex.jl:294-321 with SSPRK3.  Given the library's space,
    the oracle takes its operator values and solution points, so that its final
    state is comparable bit for bit with the FP64 GPU form.  Returns the timing
    record and the final state."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    cores = nthreads or os.cpu_count() or 1
    O.set_threads(cores)
    po = O.Space2D(0, 2, SV_NX, 0, 1, SV_NY, DEG)
    xpg = po.xpg
    if gpu_space is not None:
        same_ops(po, gpu_space)
        xpg = gpu_space.xpg
    u, upstream = shock_vortex_initial(xpg)
    P = O.Problem(O.EULER2D, po, gamma=GAMMA, flux=O.FLUX_HLL,
                  bcs=[O.BC_FIXED, O.BC_COPY, O.BC_COPY, O.BC_COPY],
                  fixed_states=[upstream, [0] * 4, [0] * 4, [0] * 4], ghosts_per_step=1)
    t0 = time.perf_counter()
    uf = P.ssprk3_filtered(u, dt, nsteps, LAM, S0, KAPPA)
    secs = time.perf_counter() - t0
    rec = {"value": SV_NDOF * 3 * nsteps / secs, "unit": UNIT, "cores": O.get_threads(), "kind": "port",
           "sample": f"{nsteps} steps (SSPRK3 + plain indicator + :l2 filter; {3 * nsteps} RK stages) of the full "
                     f"400x200 p=3 shock-vortex workload from its initial state, FP64 oracle, OpenMP over elements",
           "ms_per_step": secs / nsteps * 1e3}
    return rec, uf


def reference_arm(args):
    """The reference's CPU algorithm (the oracle port: the Julia reference cannot
    run here) on the headline workload: W warm-up and K timed steps of the
    plain FP64 form with the indicator + filter after every step."""
    xpg, dx, dy = sv_space_host()
    dt = host_cfl_dt(shock_vortex_initial(xpg)[0], dx, dy)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.set_threads(os.cpu_count() or 1)
    po = O.Space2D(0, 2, SV_NX, 0, 1, SV_NY, DEG)
    u, upstream = shock_vortex_initial(po.xpg)
    P = O.Problem(O.EULER2D, po, gamma=GAMMA, flux=O.FLUX_HLL,
                  bcs=[O.BC_FIXED, O.BC_COPY, O.BC_COPY, O.BC_COPY],
                  fixed_states=[upstream, [0] * 4, [0] * 4, [0] * 4], ghosts_per_step=1)
    K = max(1, args.steps)
    if args.warmup:
        u = P.ssprk3_filtered(u, dt, args.warmup, LAM, S0, KAPPA)
    t0 = time.perf_counter()
    P.ssprk3_filtered(u, dt, K, LAM, S0, KAPPA)
    secs = time.perf_counter() - t0
    value = SV_NDOF * 3 * K / secs
    cb = {"value": value, "unit": UNIT, "cores": O.get_threads(), "kind": "port",
          "sample": f"{K} timed steps after {args.warmup} warm-up steps of the full 400x200 p=3 shock-vortex "
                    f"workload (SSPRK3 + plain indicator + :l2 filter), FP64 oracle, OpenMP over elements"}
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs / K * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": headline_config(dt, args.gpus),
            "form": "reference CPU algorithm: plain FP64 residual, SSPRK3, plain modal-decay indicator + :l2 "
                    "filter every step (oracle port)",
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--acc-steps", type=int, default=300,
                    help="steps of the accuracy runs (and of the CPU baseline) from the initial state")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the density-wave, ensemble, BGK and triangle entries")
    # profiling aid: run one workload alone (small sizes through --steps / --instances)
    ap.add_argument("--workload", choices=["density_wave", "ensemble", "bgk", "triangles", "indicator"], default=None)
    ap.add_argument("--instances", type=int, default=4096)
    ap.add_argument("--tri-nx", type=int, default=1024, help="triangles: squares per side (2 nx^2 cells)")
    args = ap.parse_args()
    ws, rank, _ = dist_env()

    if args.impl == "reference":
        # rank 0 alone times the CPU reference; the other ranks have no work
        if rank == 0:
            print(json.dumps(reference_arm(args)), flush=True)
        return

    dist = init_dist(ws)
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if args.workload is not None:
        measure_fma_peaks()
        if args.workload == "density_wave":
            r = density_wave_entry(args, None, 1)
        elif args.workload == "ensemble":
            r = ensemble_entry(n=args.instances, t_end=0.5)
        elif args.workload == "indicator":
            r = indicator_entry(steps=args.steps, warmup=args.warmup)
        elif args.workload == "triangles":
            # FP32K first, so that a profiler's first residual launch is the FP32K one
            r = tri_entry(nx=args.tri_nx, steps=args.steps, warmup=args.warmup, reps=args.steps,
                          forms=("fp32k", "fp64"), cpu=False)
        else:
            r = bgk_entry(steps=args.steps, warmup=args.warmup)
        print(json.dumps({"partial_run": True, "workload": args.workload, "result": r}), flush=True)
        return

    from frgpu import learned

    xpg, dx, dy = sv_space_host()
    dt = host_cfl_dt(shock_vortex_initial(xpg)[0], dx, dy)
    sampler = ClockSampler(torch.cuda.current_device())
    if rank == 0:
        sampler.start()
    fma_peaks = measure_fma_peaks()
    res = headline_arm(args, dist, rank, ws, dt)
    configs = {}
    if not args.no_configs:
        # the other workloads of the spec, each on its own clock (not part of `value`)
        for name, fn in (("density_wave_512x512_p3", lambda: density_wave_entry(args, dist, ws)),
                         ("indicators_400x200_p3", indicator_entry),
                         ("burgers_ensemble_4096", ensemble_entry), ("bgk_256x512_p3", bgk_entry),
                         ("triangles_advection_2M_cells_p3", tri_entry),
                         ("reference_scripts_rock_curve", dev_scripts_entry)):
            try:
                configs[name] = fn()
            except Exception as e:  # report, do not lose the headline line
                configs[name] = {"error": f"{type(e).__name__}: {e}"}
    clocks = sampler.stop() if rank == 0 else None
    if rank != 0:
        return
    ps = learned.config3_space()
    finals, truth, stats = res.pop("accuracy_runs")
    cpu, oracle_final = None, None
    if not args.no_cpu_baseline:
        try:
            cpu, oracle_final = headline_cpu(dt, args.acc_steps, ps)
        except Exception as e:  # the oracle needs gcc on the host
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {e}"}
    acc = accuracy_report(ps, finals, truth, stats, oracle_final)
    acc["steps_from_initial_state"] = args.acc_steps
    acc["t_end"] = args.acc_steps * dt
    peak, kind = measured_peaks()
    lrn, p32, p64 = res["learned_fp32k"], res["plain_fp32k"], res["plain_fp64"]
    step_bytes = 3 * SV_NDOF * BYTES_PER_DOF_STAGE["fp32k"]
    sv = {"workload": WORKLOAD, "ndof": SV_NDOF,
          "headline_step_roofline": {
              "bound": "hbm", "kernel": "k_euler2d<float,4,HLL,FP32K,stage> x3, learned indicator fused in stage 3",
              "achieved": step_bytes / (lrn["ms_per_step"] * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
              "frac": step_bytes / (lrn["ms_per_step"] * 1e-3) / 1e9 / peak, "bytes_per_step": step_bytes,
              "peak_kind": peak_kind_label(kind)}}
    configs = {"shock_vortex_400x200_p3": sv, **configs}
    dw = configs.get("density_wave_512x512_p3", {})
    line = {
        "metric": METRIC, "value": lrn["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": lrn["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": headline_config(dt, ws),
        "form": "learned troubled-cell indicator (fused into the third stage, with the :l2 filter) + FP32 residual "
                "with compensated SSPRK3 stage sums",
        "plain_fp64": {**p64, "dtype": "f64"},
        "plain_fp32k": {**p32, "dtype": "f32"},
        "speedup_vs_plain_fp64": lrn["value"] / p64["value"],
        "learned_time_cost_vs_plain_fp32k": p32["value"] / lrn["value"],
        "accuracy": acc,
        "roofline": dw.get("roofline"),
        "e2e": res.get("e2e"),
        "e2e_rhs": res.get("e2e_rhs"),
        "fp64_peak_measured": fma_peaks,
        "fp64_forms_vs_fp64_peak": {
            "density_wave_fp64": (dw.get("fp64_roofline") or {}).get("frac"),
            "triangles_fp64": ((configs.get("triangles_advection_2M_cells_p3") or {}).get("fp64") or {})
            .get("roofline", {}).get("flops", {}).get("frac")},
        "gpu_launches": lrn["launches_timed"],
        "clocks": clocks,
        "cpu_baseline": cpu,
        "configs": configs,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
