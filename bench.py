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
# DRAM bytes (read + write) per stage launch measured by ncu on this workload;
# summarised in profiles/euler2d_stage_512x512_p3.md.  None until captured.
NCU_TRAFFIC_PER_LAUNCH = {"fp32k": None, "fp64": None}


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
            os.makedirs(os.path.join(ROOT, "gpurun_out"), exist_ok=True)
            self.path = os.path.join(ROOT, "gpurun_out", f"clocks_bench_{os.getpid()}.csv")
            self.f = open(self.path, "w")
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
            host_u = np.asfortranarray(u0)
            sums_steps = []

            def e2e_run():
                itg.u = host_u                       # H2D of the state (host FP64 array)
                for _ in range(K):
                    itg.step(1)                      # H2D of dt inside frgpu_step_ssprk3
                    sums_steps.append(itg.reduce())  # D2H of FP64 sums + wave speed
                return itg.u                         # D2H of the final state

            itg.synchronize()
            barrier(dist)
            t0 = time.perf_counter()
            e2e_run()
            e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
            state_bytes = NDOF * 8
            out["e2e"] = {"value": total_dofs / e2e_s, "unit": UNIT,
                          "h2d_bytes_per_step": (state_bytes + 8 * K) / K,
                          "d2h_bytes_per_step": (state_bytes + 5 * 8 * K) / K,
                          "note": "state uploaded from and downloaded to host FP64 arrays once per K steps; "
                                  "dt written and conserved sums/max speed read every step"}
        del itg, prob
    clocks = sampler.stop() if rank == 0 else None
    return out, clocks


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
    args = ap.parse_args()
    ws, rank, _ = dist_env()
    dist = init_dist(ws)

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
    if not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = cpu_baseline()
        except Exception as e:  # the oracle needs gcc on the host
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {e}"}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
