#!/usr/bin/env python3
"""Benchmark: leapfrog site-updates/s of the InflationEasy lattice at 256^3.

Workload (hilltop, the reference's params.analytic.txt with ns = 0.965, seed 8,
N = 256, L = 10, dt = 1e-3): Bunch-Davies initial conditions generated on the
device, then the leapfrog loop of src/evolution.cpp:937-945 (Friedmann update +
kick + drift of every site) run by the engine.  A step is one leapfrog step of
the whole 256^3 lattice; value = steps * 256^3 / device time.  The lattice
state (384 MB in FP64) is larger than L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

The headline value is the plain FP64 form, the reference's own precision and
per-site arithmetic (like for like with the reference arm).  Beside it, under
"forms": the split form (FP32 perturbations about an FP64 background) and the
compensated split form (the same with Kahan residuals carried from step to
step) on the same workload, each with its error statement against the FP64
form over a whole run (inflation to af = 512 and the deltaN stage: P_dphi and
P_zeta per k-bin, <dphi^2>, H(t) at every save); the batched ensemble (512 x 32^3 + 64 x 64^3 +
8 x 128^3 lattices, USR table potential, advanced together, against the same
number of steps of one lattice of each size alone, and its deltaN stage); the
SIGW split step at 256^3 and 512^3 with the Omega_GW comparison against the
FP64 form; the post-inflation phase; the FFT + binning, deltaN and RK4
kernels.

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
# batched ensemble: 512 seeds at 32^3 + 64 at 64^3 + 8 at 128^3, USR table
# potential (params.numerical.txt), split form
ENSEMBLE = ((32, 512), (64, 64), (128, 8))
USR = dict(L=10.0, dt=1e-3, V0=3e-9, phi0=2.9181235049318586, dphi0=-0.06727651095116181, dN=1e-4, Nend=2.0)
TABLES = ROOT / "tests" / "golden" / "inputs"   # the reference's inputs/*.dat
METRIC = "site-updates/s at 256^3: FP64 plain vs split-FP32 vs batched; % of HBM peak"
UNIT = "site-updates/s"
# algorithmic HBM bytes per site of the dominant kernel of one step
BYTES_STEP_SPLIT = 16  # split form: read dphi, dpi; write dphi, dpi (FP32)
BYTES_STEP_COMP = 24   # compensated split form: 16 + read and write the bf16 residuals of dphi and dpi
BYTES_STEP_FP64 = 32   # plain FP64 form: read f, fd; write f, fd
# FP64 thread instructions per site of one plain FP64 leapfrog step (k_lsum:
# six DADD and one DMUL of the Laplacian, the sums' products on the integer
# pipes; k_kick: six DMUL, four DADD; hilltop) and per deltaN site-step
# (k_deltaN, hilltop, from ncu)
FP64_INST_STEP = 17
# FP64 thread instructions of one 3D FFT at 256^3, forward or inverse (ncu:
# DADD + DMUL + DFMA of the three radix-2 passes and the row unpacking; each
# butterfly is four DMUL and eight DADD in the reference's order)
FFT_FP64_INST_256 = 1.3155e9
# FP64 thread instructions per site of one RK4 step (four k_rk_rhs at 20.1,
# three one-term k_rk_combine at 8 and the final four-term one at 20) and of
# one post-inflation step (k_post_kick 12, k_post_sigw 124, k_drift<SIGW> 8),
# hilltop, from ncu (DADD + DMUL + DFMA thread instructions of each kernel)
RK4_FP64_INST_SITE = 124.4
POST_FP64_INST_SITE = 144.0
DN_FP64_INST = 25
BYTES_STEP_SIGW = 112  # split form with SIGW: 16 + read and write 6 h_ij and 6 h_ij' (FP32)
BYTES_STEP_POST = 128  # post-inflation phase: read and write f, fd (FP64) and 6 h_ij, 6 h_ij' (FP32)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_device(environ):
    """Under torchrun every rank is a replica on its own GPU: the local rank
    selects it unless CUDA_VISIBLE_DEVICES is already set for the process."""
    ws = int(environ.get("WORLD_SIZE", "1"))
    if ws > 1 and "CUDA_VISIBLE_DEVICES" not in environ:
        return str(int(environ.get("LOCAL_RANK", "0")))
    return None


def ranks_max(value, dist):
    """The slowest replica sets the time: max of a per-rank float over ranks."""
    if not dist:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


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


def cpu_usr_step_ms(N, tables, threads, target_s=1.0):
    """ms per leapfrog step of one N^3 USR lattice in the oracle port of the
    reference on the host cores (a bounded sample; CPU baseline of the batched
    form)."""
    import numpy as np

    import ieo
    p = ieo.usr_params(N, calculate_SIGW=0)
    o = ieo.Oracle(p, tables, threads=threads)
    rng = np.random.default_rng(2)
    o.f[:] = USR["phi0"] + 1e-6 * rng.standard_normal(N ** 3)
    o.fd[:] = USR["dphi0"] + 1e-6 * rng.standard_normal(N ** 3)
    s = o.scalars
    s.a, s.astep, s.ad = 1.0, 1.0, 1.0
    o.set_scalars(s)
    o.leapfrog_steps(1)
    t0 = time.perf_counter()
    o.leapfrog_steps(1)
    t1 = time.perf_counter() - t0
    steps = max(2, int(target_s / max(t1, 1e-4)))
    t0 = time.perf_counter()
    o.leapfrog_steps(steps)
    return 1e3 * (time.perf_counter() - t0) / steps


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


def measure_form(iegpu, form, N, steps, warmup, clocks_index, e2e_too, dist=None, settle_s=0.0, tail_s=0.0,
                 usr=False):
    """Times `steps` leapfrog steps of one form; returns a dict of figures.
    With clocks_index set, nvidia-smi samples the SM clocks from settle_s
    seconds of untimed steps before the warm-up to tail_s seconds of untimed
    steps after the timed region, so the samples bracket it."""
    import numpy as np
    w = dict(USR, ns=0.97, seed=8) if usr else WORKLOAD
    lat = iegpu.Lattice(N, w["L"], w["dt"], w["V0"], w["ns"], form=form,
                        potential=iegpu.POT_TABLE if usr else iegpu.POT_HILLTOP)
    if usr:
        lat.set_table(*usr_tables())
    H = lat.bunch_davies(w["seed"], w["phi0"], w["dphi0"])
    bg = iegpu.Bg(0.0, 1.0, H, 0.0, 1.0)
    lat.evolve_fields(0.5 * w["dt"], bg)   # first half drift, src/evolution.cpp:935
    af = 1e30  # a fixed number of steps is timed
    shape = lat.autotune(bg) if form != iegpu.FORM_FP64 else None
    clk = Clocks(clocks_index) if clocks_index is not None else None
    if clk:
        clk.__enter__()

    def hold(seconds):
        t_end = time.perf_counter() + seconds
        while time.perf_counter() < t_end:
            lat.leapfrog(af, 16, bg)
            bg.astep = bg.a

    hold(settle_s)
    lat.leapfrog(af, warmup, bg)
    bg.astep = bg.a  # the loop's "astep = a", src/evolution.cpp:944
    if dist:
        dist.barrier()
    launches0 = lat.launches
    lat.timer_start()
    taken = lat.leapfrog(af, steps, bg)
    ms = lat.timer_stop()   # synchronises the lattice's stream
    if dist:
        dist.barrier()
    bg.astep = bg.a
    launches = lat.launches - launches0
    hold(tail_s)
    if clk:
        clk.__exit__(None, None, None)
    assert taken == steps
    tmax = ranks_max(ms, dist)
    out = {"ms": tmax, "launches": launches, "clocks": clk.summary() if clk else None, "shape": shape}
    # per-kernel device time, CUDA events around each launch (same stream)
    prof_steps = min(50, steps)
    ms0, ms1 = lat.profile_leapfrog(af, prof_steps, bg)
    bg.astep = bg.a
    out["kernel_ms"] = ms1 / prof_steps
    out["aux_ms"] = ms0 / (prof_steps if form == iegpu.FORM_FP64 else 1)
    if e2e_too:
        # end to end through the C ABI: host buffers in, steps, host buffers out
        f_host = lat.download(iegpu.F)
        fd_host = lat.download(iegpu.FD)
        f_out, fd_out = np.empty_like(f_host), np.empty_like(fd_host)
        pinned = "numpy"
        try:
            import torch
            f_host = torch.from_numpy(f_host).pin_memory().numpy()
            fd_host = torch.from_numpy(fd_host).pin_memory().numpy()
            f_out = torch.from_numpy(f_out).pin_memory().numpy()
            fd_out = torch.from_numpy(fd_out).pin_memory().numpy()
            pinned = "pinned"
        except Exception:
            pass
        # the buffers exist before the timed region, as a caller stepping a
        # lattice repeatedly would keep them
        t0 = time.perf_counter()
        lat.upload(iegpu.F, f_host)
        lat.upload(iegpu.FD, fd_host)
        lat.leapfrog(af, steps, bg)
        lat.download(iegpu.F, out=f_out)
        lat.download(iegpu.FD, out=fd_out)
        te2e = ranks_max(time.perf_counter() - t0, dist)
        assert np.isfinite(f_out[:4]).all() and np.isfinite(fd_out[:4]).all()
        out["e2e_s"] = te2e
        out["pinned"] = pinned
    lat.close()
    return out


def usr_tables():
    import numpy as np
    return tuple(np.loadtxt(TABLES / n) for n in ("field_values.dat", "potential.dat", "potential_derivative.dat"))


def measure_ensemble(iegpu, steps, warmup, peak):
    """The batched form: every lattice of the ensemble advanced `steps` leapfrog
    steps together, timed in both modes (one kernel per lattice size per
    step, the sizes side by side in CUDA graphs; one cooperative launch per 64
    steps over a queue of every lattice's tiles), then the deltaN stage, zeta
    spectra and the pooled zeta histogram;
    against the same number of steps of one lattice of each size run alone
    (the sequential way: one lattice after another)."""
    w = USR
    tables = usr_tables()
    Ns = [n for n, c in ENSEMBLE for _ in range(c)]
    sites = sum(n ** 3 for n in Ns)
    ens = iegpu.Ensemble(Ns, w["L"], w["dt"], w["V0"], potential=iegpu.POT_TABLE)
    ens.set_table(*tables)
    hub = ens.bunch_davies(list(range(1, len(Ns) + 1)), w["phi0"], w["dphi0"])
    bg = ens.bgs(hub)
    ens.evolve_fields(0.5 * w["dt"], bg)
    ens.leapfrog(1e30, warmup, bg)   # the first call runs the per-size launch-shape autotuner
    for b in range(len(Ns)):
        bg[b].astep = bg[b].a
    shape = ens.autotune(bg)
    modes = {}
    for persistent in (False, True):
        # per-size launches (CUDA graphs, autotuned shapes), then one
        # cooperative launch per 64 steps over the mixed queue
        ens.set_persistent(persistent)
        ens.leapfrog(1e30, warmup, bg)
        for b in range(len(Ns)):
            bg[b].astep = bg[b].a
        launches0 = ens.launches
        ens.timer_start()
        taken = ens.leapfrog(1e30, steps, bg)
        ms_mode = ens.timer_stop()
        assert int(taken.min()) == steps
        for b in range(len(Ns)):
            bg[b].astep = bg[b].a
        modes["persistent" if persistent else "per_size"] = (ms_mode, ens.launches - launches0)
    best = min(modes, key=lambda k: modes[k][0])
    ms, launches = modes[best]
    ens.set_persistent(False)
    prof_steps = min(20, steps)
    _, kms = ens.profile(prof_steps, bg)
    for b in range(len(Ns)):
        bg[b].astep = bg[b].a
    t0 = time.perf_counter()
    ens.deltaN(bg, w["dN"], w["Nend"])
    t_dn = time.perf_counter() - t0
    t0 = time.perf_counter()
    spectra = ens.zeta_spectra()
    t_sp = time.perf_counter() - t0
    hists = {n: ens.zeta_histogram(n, 200, 10.0) for n, _ in ENSEMBLE}
    ens.close()
    # one lattice of each size alone, the same number of steps
    seq = {}
    for n, _ in ENSEMBLE:
        lat = iegpu.Lattice(n, w["L"], w["dt"], w["V0"], potential=iegpu.POT_TABLE, form=iegpu.FORM_SPLIT)
        lat.set_table(*tables)
        H = lat.bunch_davies(1, w["phi0"], w["dphi0"])
        b1 = iegpu.Bg(0.0, 1.0, H, 0.0, 1.0)
        lat.evolve_fields(0.5 * w["dt"], b1)
        lat.leapfrog(1e30, warmup, b1)
        b1.astep = b1.a
        lat.timer_start()
        lat.leapfrog(1e30, steps, b1)
        seq[n] = lat.timer_stop() / steps
        lat.close()
    t_seq = sum(c * steps * seq[n] for n, c in ENSEMBLE)
    # the same one lattice of each size in the plain FP64 form, and the oracle
    # port of the reference on the host cores (a bounded CPU-baseline sample of
    # a few steps per size)
    seq64, cpu = {}, {}
    for n, _ in ENSEMBLE:
        lat = iegpu.Lattice(n, w["L"], w["dt"], w["V0"], potential=iegpu.POT_TABLE, form=iegpu.FORM_FP64)
        lat.set_table(*tables)
        H = lat.bunch_davies(1, w["phi0"], w["dphi0"])
        b1 = iegpu.Bg(0.0, 1.0, H, 0.0, 1.0)
        lat.evolve_fields(0.5 * w["dt"], b1)
        lat.leapfrog(1e30, warmup, b1)
        b1.astep = b1.a
        lat.timer_start()
        lat.leapfrog(1e30, steps, b1)
        seq64[n] = lat.timer_stop() / steps
        lat.close()
        cpu[n] = cpu_usr_step_ms(n, tables, os.cpu_count() or 1)
    t_seq64 = sum(c * steps * seq64[n] for n, c in ENSEMBLE)
    t_cpu = sum(c * steps * cpu[n] for n, c in ENSEMBLE)
    # HBM figure from the timed region (the faster mode), 16 B per site-update
    achieved = BYTES_STEP_SPLIT * sites * steps / (ms * 1e-3) / 1e9
    mode_figs = {k: {"ms_per_step": v[0] / steps, "gpu_launches": v[1],
                     "frac_of_measured_hbm": BYTES_STEP_SPLIT * sites * steps / (v[0] * 1e-3) / 1e9 / peak}
                 for k, v in modes.items()}
    return {"workload": "512 x 32^3 + 64 x 64^3 + 8 x 128^3 lattices, USR table potential (params.numerical.txt), "
                        "split form, device Bunch-Davies initial conditions, seeds 1..584",
            "lattices": len(Ns), "sites": sites, "steps": steps,
            "site_updates_per_s": steps * sites / (ms * 1e-3), "ms_per_step": ms / steps,
            "mode": best, "modes": mode_figs,
            "achieved_gbs": achieved, "frac_of_measured_hbm": achieved / peak,
            "frac_source": "timed region of the faster mode (CUDA events), 16 B per site-update",
            "per_size_kernel_ms_isolated": kms / prof_steps,
            "gpu_launches": launches,
            "shapes": {str(n): [int(shape["rows"][Ns.index(n)]), int(shape["prefetch"][Ns.index(n)]),
                                int(shape["chunks"][Ns.index(n)])] for n, _ in ENSEMBLE},
            "sequential_ms_per_step": {str(n): seq[n] for n, _ in ENSEMBLE},
            "sequential_site_updates_per_s": steps * sites / (t_seq * 1e-3),
            "lattices_per_s_over_sequential": t_seq / ms,
            "sequential_fp64_ms_per_step": {str(n): seq64[n] for n, _ in ENSEMBLE},
            "lattices_per_s_over_sequential_fp64": t_seq64 / ms,
            "cpu_oracle_ms_per_step": {str(n): cpu[n] for n, _ in ENSEMBLE},
            "cpu_oracle_cores": os.cpu_count() or 1,
            "lattices_per_s_over_cpu_oracle": t_cpu / ms,
            "deltaN_stage_s": t_dn, "zeta_spectra_s": t_sp,
            "zeta_sigma": {str(n): hists[n]["sigma"] for n, _ in ENSEMBLE},
            "zeta_outside_10sigma": {str(n): [int(x) for x in hists[n]["outside"]] for n, _ in ENSEMBLE},
            "zeta_spectra_lattices": len(spectra)}


def measure_batched_steps(iegpu, steps, warmup, shapes=None):
    """The batched form's leapfrog steps alone (512 x 32^3 + 64 x 64^3 +
    8 x 128^3, USR, per-size launches with the autotuned shapes): a short run
    for profilers, without the deltaN stage or the comparisons.  shapes
    ("N:rows:prefetch:chunks,..."): fixed launch shapes instead of the
    autotuner's, whose trial timings mean nothing under a profiler."""
    w = USR
    Ns = [n for n, c in ENSEMBLE for _ in range(c)]
    ens = iegpu.Ensemble(Ns, w["L"], w["dt"], w["V0"], potential=iegpu.POT_TABLE)
    ens.set_table(*usr_tables())
    hub = ens.bunch_davies(list(range(1, len(Ns) + 1)), w["phi0"], w["dphi0"])
    bg = ens.bgs(hub)
    ens.evolve_fields(0.5 * w["dt"], bg)
    if shapes:
        for t in shapes.split(","):
            ens.set_shape(*(int(v) for v in t.split(":")))
    ens.leapfrog(1e30, warmup, bg)   # without fixed shapes, the first call autotunes them
    for b in range(len(Ns)):
        bg[b].astep = bg[b].a
    # the autotuner again on the warmed-up state, as measure_ensemble does (or the fixed shapes)
    shape = ens.shapes() if shapes else ens.autotune(bg)
    ens.leapfrog(1e30, warmup, bg)
    for b in range(len(Ns)):
        bg[b].astep = bg[b].a
    ens.timer_start()
    taken = ens.leapfrog(1e30, steps, bg)
    ms = ens.timer_stop()
    assert int(taken.min()) == steps
    ens.close()
    return {"ms_per_step": ms / steps, "site_updates_per_s": steps * sum(n ** 3 for n in Ns) / (ms * 1e-3),
            "shapes": {str(n): [int(shape["rows"][Ns.index(n)]), int(shape["prefetch"][Ns.index(n)]),
                                int(shape["chunks"][Ns.index(n)])] for n, _ in ENSEMBLE}}


def measure_sigw(iegpu, N, steps, warmup, peak):
    """The split form with the SIGW tensor modes on (config: USR table
    potential, 6 h_ij components and their momenta in FP32): K steps, and one
    GW spectrum (TT projection and shell binning) of the evolved h'."""
    w = USR
    lat = iegpu.Lattice(N, w["L"], w["dt"], w["V0"], potential=iegpu.POT_TABLE, form=iegpu.FORM_SPLIT, sigw=True)
    lat.set_table(*usr_tables())
    H = lat.bunch_davies(8, w["phi0"], w["dphi0"])
    bg = iegpu.Bg(0.0, 1.0, H, 0.0, 1.0)
    lat.evolve_fields(0.5 * w["dt"], bg)
    lat.leapfrog(1e30, warmup, bg)
    bg.astep = bg.a
    lat.timer_start()
    taken = lat.leapfrog(1e30, steps, bg)
    ms = lat.timer_stop()
    assert taken == steps
    bg.astep = bg.a
    # the reference's float accumulators, as the program uses them; the first
    # call also builds the per-bin mode lists of this lattice size (once)
    lat.gw_spectrum_ref(1, 1.0)
    t0 = time.perf_counter()
    counts, f2, _ = lat.gw_spectrum_ref(1, 1.0)
    t_gw = time.perf_counter() - t0
    lat.close()
    per_step = ms / steps
    achieved = BYTES_STEP_SIGW * N ** 3 / (per_step * 1e-3) / 1e9
    return {"workload": f"SIGW on, N={N}^3, USR table potential, split form (FP32 dphi/dpi and 6 h_ij + h_ij')",
            "steps": steps, "ms_per_step": per_step, "site_updates_per_s": N ** 3 / (per_step * 1e-3),
            "algorithmic_bytes_per_site": BYTES_STEP_SIGW, "achieved_gbs": achieved,
            "frac_of_measured_hbm": achieved / peak, "gw_spectrum_s": t_gw, "gw_bins": int((counts > 0).sum())}


def measure_post_inflation(iegpu, N, steps, warmup, peak, fp64_rate=None):
    """The post-inflation phase (radiation era, plain FP64 form, SIGW on): the
    hilltop lattice's device initial conditions turned into Phi by
    initialize_post_inflation (without deltaN), then K leapfrog steps of the
    fd kick, the Hessian-sourced tensor kick and the drift."""
    w = WORKLOAD
    lat = iegpu.Lattice(N, w["L"], w["dt"], w["V0"], w["ns"], form=iegpu.FORM_FP64, sigw=True)
    H = lat.bunch_davies(w["seed"], w["phi0"], w["dphi0"])
    bg = iegpu.Bg(0.0, 1.0, H, 0.0, 1.0)
    lat.initialize_post_inflation(bg, 1.0, 1.0 / 3.0, from_deltaN=False)
    dt = 0.001   # dt_post_inflation of the reference's presets
    lat.evolve_fields(0.5 * dt, bg)
    lat.post_inflation_leapfrog(1e30, dt, warmup, bg)
    lat.timer_start()
    taken = lat.post_inflation_leapfrog(1e30, dt, steps, bg)
    ms = lat.timer_stop()
    assert taken == steps
    lat.close()
    per_step = ms / steps
    achieved = BYTES_STEP_POST * N ** 3 / (per_step * 1e-3) / 1e9
    return {"workload": f"post-inflation phase, N={N}^3, plain FP64 form with SIGW (omega = 1/3, from the hilltop "
                        f"device initial conditions)",
            "steps": steps, "ms_per_step": per_step, "site_updates_per_s": N ** 3 / (per_step * 1e-3),
            "algorithmic_bytes_per_site": BYTES_STEP_POST, "achieved_gbs": achieved,
            "frac_of_measured_hbm": achieved / peak,
            "bound": "fp64", "fp64_inst_per_site": POST_FP64_INST_SITE,
            "fp64_frac_of_measured_rate": (POST_FP64_INST_SITE * N ** 3 / (per_step * 1e-3) / fp64_rate
                                           if fp64_rate else None),
            "note": "three kernels per step (fd kick, tensor kick with the 19-point Hessian source, drift), "
                    "FP64 per-site arithmetic in the reference's order"}


def measure_split_error(N, workdir):
    """The split forms' error statement over a whole run at N^3 (hilltop
    preset, seed 8, af = 2N, deltaN stage): the host program run in the FP64
    form and in each split form from the same device initial conditions,
    every save compared; plus how many sites' deltaN is a whole dN step off."""
    import form_error as fe
    text = fe.preset_text(fe.HILLTOP, N)
    t0 = time.perf_counter()
    ref = fe.run_program(text, Path(workdir) / "fp64", "fp64")
    secs = {"fp64": time.perf_counter() - t0}
    out = {}
    for form in ("split", "split_comp"):
        t0 = time.perf_counter()
        got = fe.run_program(text, Path(workdir) / form, form)
        secs[form] = time.perf_counter() - t0
        err = fe.compare(ref, got)
        err["deltaN_steps_off"] = fe.deltaN_steps_off(ref, got, fe.HILLTOP["dN"])
        err.pop("H_per_save", None)
        err["workload"] = (f"hilltop, N={N}^3, seed 8, inflation to af={2 * N} and the deltaN stage (dN=1e-7, "
                           f"Nend=1e-3), {form} vs plain FP64 form from the same device initial conditions")
        out[form] = err
    out["program_s"] = secs
    return out


def measure_sigw_error(N, workdir):
    """Config: SIGW on, USR table, N^3: Omega_GW(k) per k-bin at every save,
    split against the plain FP64 form (host program, same device initial
    conditions, inflation to af = 2N, no deltaN stage)."""
    import form_error as fe
    text = fe.preset_text(fe.USR, N, calculate_SIGW=1, perform_deltaN=0)
    t0 = time.perf_counter()
    ref = fe.run_program(text, Path(workdir) / "sigw_fp64", "fp64", inputs=TABLES)
    t1 = time.perf_counter()
    got = fe.run_program(text, Path(workdir) / "sigw_split", "split", inputs=TABLES)
    t2 = time.perf_counter()
    err = fe.compare(ref, got)
    out = {"workload": f"USR table, SIGW on, N={N}^3, seed 8, inflation to af={2 * N}, split vs plain FP64 form",
           "Omega_GW": fe.compare_omega_gw(ref, got, USR["L"]),
           "spectrumGW": err.get("spectrumGW"), "spectrumGWdot": err.get("spectrumGWdot"),
           "P_dphi": err["P_dphi"], "H_max": err["H_max"], "saves": err["saves"],
           "program_s": {"fp64": t1 - t0, "split": t2 - t1}}
    return out


def measure_kernels(iegpu, N, fp64_rate, peak):
    """The hot path's other kernels at N^3 (FP64): one forward + inverse 3D FFT
    with the shell binning of the modes (16 B/site per transform, 8 B/site per
    binning), the deltaN integration (register resident, FP64 operations per
    site-step) and one RK4 step (336 B/site)."""
    import numpy as np
    w = WORKLOAD
    out = {}
    lat = iegpu.Lattice(N, w["L"], w["dt"], w["V0"], w["ns"], form=iegpu.FORM_FP64)
    H = lat.bunch_davies(w["seed"], w["phi0"], w["dphi0"])
    bg = iegpu.Bg(0.0, 1.0, H, 0.0, 1.0)
    lat.evolve_fields(0.5 * w["dt"], bg)
    # FFT forward + inverse (the spectrum's pair) and the binning
    lat.spectrum(iegpu.F)
    reps = 5
    ms_dir = {1: 0.0, -1: 0.0}
    for _ in range(reps):
        for sgn in (1, -1):
            lat.timer_start()
            lat.fft(iegpu.F, sgn)
            ms_dir[sgn] += lat.timer_stop() / reps
    ms_fft = 0.5 * (ms_dir[1] + ms_dir[-1])
    t0 = time.perf_counter()
    for _ in range(reps):
        lat.spectrum(iegpu.F)
    ms_spec = 1e3 * (time.perf_counter() - t0) / reps
    gbs = 16 * N ** 3 / (ms_fft * 1e-3) / 1e9
    out["fft"] = {"ms_per_transform": ms_fft, "ms_forward": ms_dir[1], "ms_inverse": ms_dir[-1],
                  "algorithmic_bytes_per_site": 16, "achieved_gbs": gbs,
                  "frac_of_measured_hbm": gbs / peak,
                  "bound": "fp64" if N == 256 else None,
                  "fp64_inst_per_transform": FFT_FP64_INST_256 if N == 256 else None,
                  "fp64_frac_of_measured_rate": (FFT_FP64_INST_256 / (ms_fft * 1e-3) / fp64_rate
                                                 if N == 256 and fp64_rate else None),
                  "spectrum_ms": ms_spec,
                  "note": "ffteasy-exact radix-2 passes in FP64; spectrum = forward FFT + binning + inverse FFT "
                          "(the reference's spectraf), wall clock with its read-back"}
    # the FP32 transform (the GW spectra's, one h component; 8 B/site per transform)
    with iegpu.Lattice(N, w["L"], w["dt"], w["V0"], w["ns"], form=iegpu.FORM_FP64, sigw=True) as lh:
        lh.upload(iegpu.H(0), np.random.default_rng(3).standard_normal(N ** 3).astype(np.float32))
        lh.fft(iegpu.H(0), 1)
        lh.fft(iegpu.H(0), -1)
        lh.timer_start()
        for _ in range(reps):
            lh.fft(iegpu.H(0), 1)
            lh.fft(iegpu.H(0), -1)
        ms_f32 = lh.timer_stop() / (2 * reps)
    gbs32 = 8 * N ** 3 / (ms_f32 * 1e-3) / 1e9
    out["fft_f32"] = {"ms_per_transform": ms_f32, "algorithmic_bytes_per_site": 8, "achieved_gbs": gbs32,
                      "frac_of_measured_hbm": gbs32 / peak,
                      "note": "the same ffteasy passes in FP32 (one h_ij component of the GW spectra); each of the "
                              "3 passes and the unpacking reads and writes the array once, about 4x the algorithmic "
                              "bytes"}
    # deltaN: hilltop preset, dN = 1e-7
    lat.initializeN(bg.a)
    phiref = lat.get_phiref()
    steps = 2000
    lat.deltaN_steps(1e-7, 20, phiref)
    lat.timer_start()
    lat.deltaN_steps(1e-7, steps, phiref)
    ms_dn = lat.timer_stop()
    site_steps = steps * N ** 3
    out["deltaN"] = {"site_steps_per_s": site_steps / (ms_dn * 1e-3), "steps": steps,
                     "fp64_inst_per_site_step": DN_FP64_INST,
                     "fp64_inst_per_s": DN_FP64_INST * site_steps / (ms_dn * 1e-3),
                     "fp64_frac_of_measured_rate": DN_FP64_INST * site_steps / (ms_dn * 1e-3) / fp64_rate,
                     "note": "k_deltaN, hilltop, per-site state in registers (0 B/site-step of HBM); the FP64 "
                             "operation count per site-step is from ncu (DADD+DMUL+DFMA thread instructions)"}
    lat.close()
    # RK4 (inflation_integrator = rk4), FP64 form
    lat = iegpu.Lattice(N, w["L"], w["dt"], w["V0"], w["ns"], form=iegpu.FORM_FP64)
    H = lat.bunch_davies(w["seed"], w["phi0"], w["dphi0"])
    bg = iegpu.Bg(0.0, 1.0, H, 0.0, 1.0)
    lat.rk4(1e30, 2, bg)
    nrk = 10
    lat.timer_start()
    lat.rk4(1e30, nrk, bg)
    ms_rk = lat.timer_stop() / nrk
    gbs = 336 * N ** 3 / (ms_rk * 1e-3) / 1e9
    out["rk4"] = {"ms_per_step": ms_rk, "site_updates_per_s": N ** 3 / (ms_rk * 1e-3),
                  "algorithmic_bytes_per_site": 336, "achieved_gbs": gbs, "frac_of_measured_hbm": gbs / peak,
                  "bound": "fp64", "fp64_inst_per_site": RK4_FP64_INST_SITE,
                  "fp64_frac_of_measured_rate": (RK4_FP64_INST_SITE * N ** 3 / (ms_rk * 1e-3) / fp64_rate
                                                 if fp64_rate else None)}
    lat.close()
    return out


def engine_arm(args):
    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    import iegpu
    N = args.n
    cvd = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].strip()
    smi_index = int(cvd) if cvd.isdigit() else local
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    traffic = {}
    try:
        traffic = json.loads((ROOT / "profiles" / "ncu_traffic.json").read_text())
    except (OSError, ValueError):
        pass
    if args.only == "kernels":
        rate = iegpu.measure_fp64_rate(1)
        r = measure_kernels(iegpu, N, rate, peak)
        r["post_inflation"] = measure_post_inflation(iegpu, N, 10, 3, peak, rate)
        if rank == 0:
            print(json.dumps({"only": args.only, "N": N, **r}), flush=True)
        return 0
    if args.only == "batched":
        r = measure_batched_steps(iegpu, args.steps, args.warmup, args.shapes)
        if rank == 0:
            print(json.dumps({"only": args.only, "steps": args.steps, "warmup": args.warmup, **r}), flush=True)
        return 0
    if args.only in ("split", "split_comp", "sigw"):
        # one form's timed steps alone (a short run for profilers); no other forms, no CPU baseline
        if args.only == "sigw":
            r = measure_sigw(iegpu, N, args.steps, args.warmup, peak)
            ms = r["ms_per_step"]
        else:
            form = iegpu.FORM_SPLIT if args.only == "split" else iegpu.FORM_SPLIT_COMP
            r = measure_form(iegpu, form, N, args.steps, args.warmup, None, False, dist, usr=args.usr)
            ms = r["ms"] / args.steps
        if rank == 0:
            extra = {"gw_spectrum_s": r["gw_spectrum_s"]} if args.only == "sigw" else {}
            print(json.dumps({"only": args.only, "usr": args.usr, "N": N, "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": ms, "site_updates_per_s": N ** 3 / (ms * 1e-3), **extra}), flush=True)
        return 0
    # the FP64 pipe's measured rate (thread instructions per second), the
    # plain FP64 form's compute roofline
    fp64_rate = iegpu.measure_fp64_rate(1) if not args.headline_only else None

    # headline: the plain FP64 form (the reference's precision and per-site
    # arithmetic); the clocks are sampled from 1.5 s before to 0.5 s after the
    # timed region
    if args.headline_only:
        fp = measure_form(iegpu, iegpu.FORM_FP64, N, args.steps, args.warmup, None, False, dist)
    else:
        fp = measure_form(iegpu, iegpu.FORM_FP64, N, args.steps, args.warmup, smi_index, True, dist,
                          settle_s=1.5, tail_s=0.5)
    value = ws * args.steps * N ** 3 / (fp["ms"] * 1e-3)
    if args.headline_only:
        # the FP64 step alone (a short run for profilers); no forms, no CPU baseline
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                              "warmup": args.warmup, "ms_per_step": fp["ms"] / args.steps,
                              "higher_is_better": True, "dtype": "f64", "data": "synthetic",
                              "config": {"workload": f"hilltop leapfrog, N={N}^3, plain FP64 form", "N": N,
                                         "form": "fp64"}, "gpu_launches": fp["launches"],
                              "headline_only": True}), flush=True)
        return 0
    # the split form on the same workload
    sp = measure_form(iegpu, iegpu.FORM_SPLIT, N, args.steps, args.warmup, None, False, dist)
    sp_value = ws * args.steps * N ** 3 / (sp["ms"] * 1e-3)
    spc = measure_form(iegpu, iegpu.FORM_SPLIT_COMP, N, args.steps, args.warmup, None, False, dist)
    spc_value = ws * args.steps * N ** 3 / (spc["ms"] * 1e-3)
    if rank != 0:
        return 0
    with tempfile.TemporaryDirectory(prefix="ie_bench_") as wd:
        err = measure_split_error(N, wd) if not args.quick else None
        sigw_err = measure_sigw_error(N, wd) if not args.quick else None
    ens = measure_ensemble(iegpu, max(20, min(args.steps // 30, 500)), args.warmup, peak)
    sigw = measure_sigw(iegpu, N, max(10, min(args.steps // 75, 200)), args.warmup, peak)
    sigw512 = measure_sigw(iegpu, 512, 20, 5, peak) if not args.quick else None
    post = measure_post_inflation(iegpu, N, max(10, min(args.steps // 300, 100)), args.warmup, peak, fp64_rate)
    kern = measure_kernels(iegpu, N, fp64_rate, peak)

    step_ms = fp["ms"] / args.steps
    achieved = BYTES_STEP_FP64 * N ** 3 / (step_ms * 1e-3) / 1e9
    inst_rate = FP64_INST_STEP * N ** 3 / (step_ms * 1e-3)
    tr = traffic.get("fp64_step_bytes_per_site")
    # split form: the step kernel's average launch duration over its timed
    # region (one priming reduction, timed on its own, taken out)
    sp_kernel_ms = (sp["ms"] - sp["aux_ms"]) / args.steps
    sp_achieved = BYTES_STEP_SPLIT * N ** 3 / (sp_kernel_ms * 1e-3) / 1e9
    sp_tr = traffic.get("split_step_bytes_per_site")
    spc_kernel_ms = (spc["ms"] - spc["aux_ms"]) / args.steps
    spc_achieved = BYTES_STEP_COMP * N ** 3 / (spc_kernel_ms * 1e-3) / 1e9
    bytes_state = 2 * 8 * N ** 3
    e2e = {"value": ws * args.steps * N ** 3 / fp["e2e_s"], "unit": UNIT,
           "h2d_bytes_per_step": bytes_state / args.steps, "d2h_bytes_per_step": bytes_state / args.steps,
           "note": f"iegpu_upload(f, fd) + iegpu_leapfrog({args.steps} steps) + iegpu_download(f, fd), FP64 form, "
                   f"{fp['pinned']} host buffers (allocated before the timed region), wall clock"}
    cpu = cpu_baseline(N, os.cpu_count() or 1) if ws == 1 else None
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"hilltop leapfrog, N={N}^3, plain FP64 form (params.analytic.txt, ns=0.965, "
                                   f"seed 8, device Bunch-Davies initial conditions)",
                       "N": N, "form": "fp64", "l2": "state > L2 (129 MB) each step: no flush needed",
                       "parallelism": f"replicas x{ws}"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None if tr is None else tr * N ** 3,
                         "kernel": "k_lsum + k_kick (one FP64 leapfrog step: stored Laplacian and exact Friedmann "
                                   "sums, then kick + drift)",
                         "algorithmic_bytes_per_site": BYTES_STEP_FP64, "kernel_ms": step_ms,
                         "kernel_ms_source": "timed region (CUDA events on the lattice's stream) divided by the steps",
                         "kernel_ms_isolated": {"k_lsum": fp["aux_ms"], "k_kick": fp["kernel_ms"]},
                         "peak_source": f"{peak_src} hbm_gbs (MEASURED_PEAKS.json)",
                         "compute_bound": "fp64",
                         "fp64": {"inst_per_site": FP64_INST_STEP, "achieved_inst_per_s": inst_rate,
                                  "peak_inst_per_s": fp64_rate, "frac": inst_rate / fp64_rate,
                                  "peak_source": "measured: iegpu_measure_fp64_rate (independent DADD chains on "
                                                 "every SM)",
                                  "note": "GB300's FP64 pipe bounds this form: the FP64 thread instructions per "
                                          "site of both kernels are from ncu; the lattice sums and the division "
                                          "by B^2 run on the integer pipes"}},
            "gpu_launches": fp["launches"], "clocks": fp["clocks"], "e2e": e2e,
            "forms": {"split": {"value": sp_value, "ms_per_step": sp["ms"] / args.steps,
                                "over_fp64": sp_value / value,
                                "roofline": {"achieved": sp_achieved, "frac": sp_achieved / peak,
                                             "kernel": "k_split_rows4_persist", "kernel_ms": sp_kernel_ms,
                                             "kernel_ms_isolated": sp["kernel_ms"],
                                             "algorithmic_bytes_per_site": BYTES_STEP_SPLIT,
                                             "traffic": None if sp_tr is None else sp_tr * N ** 3},
                                "shape": sp["shape"], "gpu_launches": sp["launches"],
                                "error": err["split"] if err else None},
                      "split_comp": {"value": spc_value, "ms_per_step": spc["ms"] / args.steps,
                                     "over_fp64": spc_value / value,
                                     "roofline": {"achieved": spc_achieved, "frac": spc_achieved / peak,
                                                  "kernel": "k_split_rows4_persist (compensated)",
                                                  "kernel_ms": spc_kernel_ms, "kernel_ms_isolated": spc["kernel_ms"],
                                                  "algorithmic_bytes_per_site": BYTES_STEP_COMP},
                                     "shape": spc["shape"], "gpu_launches": spc["launches"],
                                     "error": err["split_comp"] if err else None,
                                     "note": "dphi, dpi in FP32 plus their Kahan residuals in bf16, carried from "
                                             "step to step"},
                      "error_program_s": err["program_s"] if err else None,
                      "batched": ens, "sigw": dict(sigw, error=sigw_err), "sigw_512": sigw512,
                      "post_inflation": post, "kernels": kern}}
    line["metric_note"] = ("value: plain FP64 form at 256^3 (like for like with the reference arm); forms.split, "
                           "forms.split_comp: the split forms on the same workload and their whole-run errors "
                           "against FP64; "
                           "forms.batched: the ensemble (site-updates/s, lattices/s over sequential runs)")
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=15000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--quick", action="store_true", help="skip the whole-run error statements and 512^3")
    ap.add_argument("--headline-only", action="store_true",
                    help="time the plain FP64 step only and print a short line (for profiler runs)")
    ap.add_argument("--only", choices=["split", "split_comp", "sigw", "batched", "kernels"], default=None,
                    help="time one other form alone (at --n; batched: the ensemble's steps) and print a short line "
                         "(for profiler runs)")
    ap.add_argument("--usr", action="store_true", help="with --only split|split_comp: the USR table potential")
    ap.add_argument("--shapes", default=None,
                    help="with --only batched: fixed launch shapes N:rows:prefetch:chunks,... (for profiler runs)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    ws, rank, local = dist_env()
    dev = replica_device(os.environ)
    if dev is not None:
        os.environ["CUDA_VISIBLE_DEVICES"] = dev
    if args.impl == "reference":
        return reference_arm(args)
    return engine_arm(args)


if __name__ == "__main__":
    sys.exit(main())
