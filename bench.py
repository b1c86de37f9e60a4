#!/usr/bin/env python3
"""Benchmark: leapfrog site-updates/s of the InflationEasy lattice at 256^3.

Workload (hilltop, the reference's params.analytic.txt with ns = 0.965, seed 8,
N = 256, L = 10, dt = 1e-3): Bunch-Davies initial conditions generated on the
device, then the leapfrog loop of src/evolution.cpp:937-945 (Friedmann update +
kick + drift of every site) run by the engine.  A step is one leapfrog step of
the whole 256^3 lattice; value = steps * 256^3 / device time.  The lattice
state (384 MB in FP64) is larger than L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference] [--form fp64]

--impl reference times the reference's own CPU algorithm for the same step
(the oracle port of it, oracle/ieo.c, OpenMP on all host cores; the reference
source tree is not on the GPU host) on the same workload.
With torchrun (N > 1) every rank runs its own independent lattice on its own
GPU (replicas: the path has no cross-lattice exchange), weak scaling.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "inflation-easy_gb300"
for p in (str(PKG), str(ROOT / "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

N_DEFAULT = 256
WORKLOAD = dict(L=10.0, dt=1e-3, V0=3.338e-13, ns=0.965, phi0=0.0935, dphi0=0.000796, seed=8)
METRIC = "site-updates/s at 256^3 (leapfrog: Friedmann + kick + drift per site)"
UNIT = "site-updates/s"
# algorithmic HBM bytes per site of each kernel of one FP64 step
BYTES_KICK_FP64 = 32   # read f, fd; write f, fd
BYTES_REDUCE_FP64 = 8  # read f


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.path = Path(tempfile.mkstemp(prefix="clocks_", suffix=".csv")[1])
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() in ("active", "1"):
                    reasons.add(name)
        self.path.unlink(missing_ok=True)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_lattice(iegpu, N):
    w = WORKLOAD
    lat = iegpu.Lattice(N, w["L"], w["dt"], w["V0"], w["ns"])
    H = lat.bunch_davies(w["seed"], w["phi0"], w["dphi0"])
    bg = iegpu.Bg(0.0, 1.0, H, 0.0, 1.0)
    lat.evolve_fields(0.5 * w["dt"], bg)   # first half drift, src/evolution.cpp:935
    return lat, bg


def cpu_baseline(N, threads, target_s=10.0):
    """The oracle port of the reference step on the host cores, bounded sample."""
    import numpy as np

    import ieo
    p = ieo.hilltop_params(N, ns=WORKLOAD["ns"], calculate_SIGW=0)
    o = ieo.Oracle(p, threads=threads)
    rng = np.random.default_rng(1)
    o.f[:] = WORKLOAD["phi0"] + 5e-8 * rng.standard_normal(N ** 3)
    o.fd[:] = WORKLOAD["dphi0"] + 5e-8 * rng.standard_normal(N ** 3)
    s = o.scalars
    s.a, s.astep, s.ad = 1.0, 1.0, 0.5773
    o.set_scalars(s)
    o.leapfrog_steps(1)
    t0 = time.perf_counter()
    o.leapfrog_steps(1)
    t1 = time.perf_counter() - t0
    steps = max(2, int(target_s / max(t1, 1e-3)))
    t0 = time.perf_counter()
    o.leapfrog_steps(steps)
    dt = time.perf_counter() - t0
    return {"value": steps * N ** 3 / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} leapfrog steps of the {N}^3 hilltop lattice (oracle/ieo.c, OpenMP kick/drift, "
                      f"serial energy sums as in the reference), {dt:.1f} s"}


def reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import ieo
    N = args.n
    threads = os.cpu_count() or 1
    p = ieo.hilltop_params(N, ns=WORKLOAD["ns"], calculate_SIGW=0)
    o = ieo.Oracle(p, threads=threads)
    import numpy as np
    rng = np.random.default_rng(1)
    o.f[:] = WORKLOAD["phi0"] + 5e-8 * rng.standard_normal(N ** 3)
    o.fd[:] = WORKLOAD["dphi0"] + 5e-8 * rng.standard_normal(N ** 3)
    s = o.scalars
    s.a, s.astep, s.ad = 1.0, 1.0, 0.5773
    o.set_scalars(s)
    o.leapfrog_steps(max(1, min(args.warmup, 3)))
    t0 = time.perf_counter()
    o.leapfrog_steps(1)
    t1 = time.perf_counter() - t0
    steps = args.steps
    budget = 150.0
    capped = steps * t1 > budget
    if capped:
        steps = max(1, int(budget / t1))
    t0 = time.perf_counter()
    o.leapfrog_steps(steps)
    dt = time.perf_counter() - t0
    value = steps * N ** 3 / dt
    sample = (f"{steps} leapfrog steps of the {N}^3 hilltop lattice" +
              (f" (of {args.steps} requested, capped at ~{budget:.0f} s)" if capped else ""))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"hilltop leapfrog, N={N}^3, FP64, reference algorithm on {threads} host threads",
                       "N": N},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def engine_arm(args):
    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    import numpy as np

    import iegpu
    N = args.n
    lat, bg = make_lattice(iegpu, N)
    af = 1e30  # time a fixed number of steps
    lat.leapfrog(af, args.warmup, bg)
    bg.astep = bg.a  # the loop's "astep = a", src/evolution.cpp:944
    if dist:
        dist.barrier()
    launches0 = lat.launches
    cvd = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].strip()
    with Clocks(int(cvd) if cvd.isdigit() else local) as clk:
        lat.timer_start()
        taken = lat.leapfrog(af, args.steps, bg)
        ms = lat.timer_stop()
    bg.astep = bg.a
    launches = lat.launches - launches0
    assert taken == args.steps
    tmax = ms
    if dist:
        import torch
        t = torch.tensor([ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tmax = float(t.item())
        dist.barrier()
    value = ws * args.steps * N ** 3 / (tmax * 1e-3)

    # dominant kernel, timed live with CUDA events around each launch
    prof_steps = min(50, args.steps)
    ms_red, ms_kick = lat.profile_leapfrog(af, prof_steps, bg)
    bg.astep = bg.a
    kick_ms = ms_kick / prof_steps
    red_ms = ms_red / prof_steps
    achieved = BYTES_KICK_FP64 * N ** 3 / (kick_ms * 1e-3) / 1e9
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    traffic = None
    try:
        tr = json.loads((ROOT / "profiles" / "ncu_traffic.json").read_text())
        if "kick_fp64_bytes_per_site" in tr:
            traffic = tr["kick_fp64_bytes_per_site"] * N ** 3
    except (OSError, ValueError):
        pass

    # end to end through the C ABI: host buffers in, steps, host buffers out
    f_host = lat.download(iegpu.F)
    fd_host = lat.download(iegpu.FD)
    pinned = "numpy"
    try:
        import torch
        tf = torch.from_numpy(f_host).pin_memory()
        tfd = torch.from_numpy(fd_host).pin_memory()
        f_host, fd_host = tf.numpy(), tfd.numpy()
        pinned = "pinned"
    except Exception:
        pass
    e2e_steps = args.steps
    t0 = time.perf_counter()
    lat.upload(iegpu.F, f_host)
    lat.upload(iegpu.FD, fd_host)
    lat.leapfrog(af, e2e_steps, bg)
    f_out = lat.download(iegpu.F)
    fd_out = lat.download(iegpu.FD)
    te2e = time.perf_counter() - t0
    if dist:
        import torch
        t = torch.tensor([te2e], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        te2e = float(t.item())
    assert np.isfinite(f_out[:4]).all() and np.isfinite(fd_out[:4]).all()
    bytes_state = 2 * 8 * N ** 3
    e2e = {"value": ws * e2e_steps * N ** 3 / te2e, "unit": UNIT, "h2d_bytes_per_step": bytes_state / e2e_steps,
           "d2h_bytes_per_step": bytes_state / e2e_steps,
           "note": f"iegpu_upload(f, fd) + iegpu_leapfrog({e2e_steps} steps) + iegpu_download(f, fd), "
                   f"{pinned} host buffers, wall clock"}
    if rank != 0:
        return 0
    cpu = cpu_baseline(N, os.cpu_count() or 1) if ws == 1 else None
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tmax / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"hilltop leapfrog, N={N}^3, plain FP64 form (params.analytic.txt, ns=0.965, "
                                   f"seed 8, device Bunch-Davies initial conditions)",
                       "N": N, "form": "fp64", "l2": "state 384 MB > L2 129 MB: no flush needed",
                       "parallelism": f"replicas x{ws}"},
            "forms": {"fp64": {"value": value, "ms_per_step": tmax / args.steps}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "kernel": "k_kick (FP64 kick + drift)",
                         "algorithmic_bytes_per_site": BYTES_KICK_FP64, "kernel_ms": kick_ms,
                         "reduce_kernel_ms": red_ms, "peak_source": f"{peak_src} hbm_gbs (MEASURED_PEAKS.json)"},
            "gpu_launches": launches, "clocks": clk.summary(), "e2e": e2e}
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    ws, rank, local = dist_env()
    if ws > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    if args.impl == "reference":
        return reference_arm(args)
    return engine_arm(args)


if __name__ == "__main__":
    sys.exit(main())
