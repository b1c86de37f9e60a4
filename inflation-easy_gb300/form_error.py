"""Error statement of the split form against the plain FP64 form.

The host program (ie_gpu_main, the reference's main() driving the engine
through the C ABI) is run twice on one parameter file, with `form = fp64` and
`form = split`, from the same device Bunch-Davies initial conditions (same
seed): inflation to af, the deltaN stage, and every output of the reference's
save()/saveN().  The full-precision outputs (dump/precise.txt: means, P_dphi,
P_zeta, the GW spectra) are then compared save by save:

  P_dphi, P_zeta, Omega_GW inputs   relative deviation per k-bin (bins >= 1)
  <dphi^2>                          relative deviation of the variance, formed
                                    from the spectrum by Parseval
                                    (sum over bins >= 1 of count x P)
  a, H, <phi>                       relative deviation at every save

The plain FP64 form is the reference's arithmetic (bit-exact with the oracle
in its engine-arithmetic mode), so this is the split form's error against
FP64.  The reference's own spectra come from src/output.cpp:297-406
(spectraf), :1140-1169 (spectraN), :466-648 (GW); its means from :204-269.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
MAIN = PKG / "_build" / "ie_gpu_main"


# The reference's presets (params.analytic.txt with ns = 0.965, the value the
# hilltop workloads use; params.numerical.txt for the USR table).
HILLTOP = dict(seed=8, dt=0.001, V0=3.338e-13, ns=0.965, initial_field=0.0935, initial_derivative=0.000796, L=10.0,
               output_freq=500, output_infrequent_freq=500, nbins=256, dN=1e-7, Nend=0.001, numerical_potential=0)
USR = dict(seed=8, dt=0.001, V0=3e-9, initial_field=2.9181235049318586, initial_derivative=-0.06727651095116181,
           L=10.0, output_freq=500, output_infrequent_freq=500, nbins=256, dN=1e-4, Nend=2.0, numerical_potential=1)


def preset_text(preset: dict, N: int, **overrides) -> str:
    """params.txt text of a preset at N points per side (deltaN on, SIGW off
    unless overridden)."""
    kv = dict(preset, N=N, perform_deltaN=1, calculate_SIGW=0, screen_updates=0, output_spectra=1,
              output_histogram=1, output_energy=1)
    kv.update(overrides)
    return "".join(f"{k} = {v}\n" for k, v in kv.items())


def run_program(params_text: str, workdir: Path, form: str, inputs: Path | None = None) -> Path:
    """Runs ie_gpu_main in workdir with `form` and device initial conditions;
    returns workdir.  `inputs` is the folder of the tabulated potential."""
    workdir = Path(workdir)
    workdir.mkdir(parents=True, exist_ok=True)
    (workdir / "params.txt").write_text(params_text + f"\nform = {form}\nic_on_host = 0\n")
    if inputs is not None and not (workdir / "inputs").exists():
        os.symlink(inputs, workdir / "inputs")
    (workdir / "dump").mkdir(exist_ok=True)
    r = subprocess.run([str(MAIN), "params.txt", "results", "dump"], cwd=workdir, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"ie_gpu_main ({form}) failed: {r.stdout[-1000:]}{r.stderr[-1000:]}")
    return workdir


def _precise(path: Path) -> dict:
    out: dict = {}
    for line in path.read_text().splitlines():
        tag, *vals = line.split()
        out.setdefault(tag, []).append(np.array([float(v) for v in vals]))
    return out


def _counts(path: Path) -> np.ndarray:
    """Bin counts of the first spectrum block of a spectra*.dat file."""
    counts = []
    for line in path.read_text().splitlines():
        if not line.strip():
            break
        counts.append(int(line.split()[1]))
    return np.array(counts, dtype=np.int64)


def _bins(got: list, ref: list) -> np.ndarray:
    """Relative deviation per bin (rows: saves); bins where the reference is 0
    get the absolute value."""
    a, b = np.array(got), np.array(ref)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(b != 0, np.abs(a / b - 1.0), np.abs(a))


def _summary(dev: np.ndarray) -> dict:
    """max over saves and bins >= 1, its bin, the median and the 99th
    percentile over bins of the per-bin maximum."""
    per_bin = dev[:, 1:].max(axis=0)
    return {"max": float(per_bin.max()), "bin_of_max": int(per_bin.argmax()) + 1,
            "median": float(np.median(per_bin)), "p99": float(np.percentile(per_bin, 99)),
            "saves": int(dev.shape[0])}


def compare(ref_dir: Path, got_dir: Path) -> dict:
    """The split form's deviations (got_dir) from the FP64 form (ref_dir)."""
    r = _precise(Path(ref_dir) / "dump" / "precise.txt")
    g = _precise(Path(got_dir) / "dump" / "precise.txt")
    out: dict = {}
    assert len(r["means"]) == len(g["means"]), "different number of saves"
    # columns that are 0 in the reference (the time of the first save) get
    # the absolute deviation
    rel = _bins(g["means"], r["means"])
    out["a_max"] = float(rel[:, 1].max())
    out["phibar_max"] = float(rel[:, 2].max())
    out["H_max"] = float(rel[:, 4].max())
    out["H_per_save"] = [float(x) for x in rel[:, 4]]
    out["saves"] = int(rel.shape[0])
    out["P_dphi"] = _summary(_bins(g["spectrum"], r["spectrum"]))
    counts = _counts(Path(ref_dir) / "results" / "spectra.dat")
    var_r = np.array([np.sum(counts[1:] * x[1:len(counts)]) for x in r["spectrum"]])
    var_g = np.array([np.sum(counts[1:] * x[1:len(counts)]) for x in g["spectrum"]])
    out["dphi2_max"] = float(np.max(np.abs(var_g / var_r - 1.0)))
    if "spectrumN" in r:
        out["P_zeta"] = _summary(_bins(g["spectrumN"], r["spectrumN"]))
    for tag in ("spectrumGW", "spectrumGWdot"):
        if tag in r:
            out[tag] = _summary(_bins(g[tag], r[tag]))
    return out


def deltaN_steps_off(ref_dir: Path, got_dir: Path, dN: float) -> dict:
    """How the final deltaN maps (dump/state.bin) of two runs differ, in steps
    of dN: the fraction of sites whose deltaN differs from the reference's by
    a nonzero whole number of steps (after the constant shift of the float
    Nmean, the median difference), and the largest deviation from a whole
    number of steps (in steps)."""
    def dn(d):
        hdr = np.fromfile(Path(d) / "dump" / "state.bin", dtype=np.int32, count=4)
        gs = int(hdr[0]) ** 3
        return np.fromfile(Path(d) / "dump" / "state.bin", dtype=np.float64, count=gs, offset=16 + 64 + 16 * gs)
    x = (dn(got_dir) - dn(ref_dir)) / dN
    x = x - np.median(x)
    k = np.rint(x)
    return {"sites_off": float(np.mean(k != 0)), "off_by_fraction": float(np.max(np.abs(x - k)))}


def omega_gw(precise: dict, L: float) -> np.ndarray:
    """Omega_GW(k) per save as the reference's notebook forms it
    (notebooks/plot.ipynb, section 8) from spectraGW (P_h), spectraGWdot
    (P_h') and the background (a, H of sf.dat):
        Omega_GW = k^3 / (2 pi^2) (P_h' + (k/a)^2 P_h) / (12 H^2),
    k = 2 pi i / L for bin i.  Rows: saves; columns: bins."""
    ph = np.array(precise["spectrumGW"])
    phd = np.array(precise["spectrumGWdot"])
    m = np.array(precise["means"])
    a, H = m[:, 1][:, None], m[:, 4][:, None]
    k = 2.0 * np.pi * np.arange(ph.shape[1]) / L
    return (k ** 3 / (2.0 * np.pi ** 2)) * (phd + (k / a) ** 2 * ph) / (12.0 * H ** 2)


def compare_omega_gw(ref_dir: Path, got_dir: Path, L: float) -> dict:
    """Relative deviation per k-bin of Omega_GW (bins >= 1 with power)."""
    r = omega_gw(_precise(Path(ref_dir) / "dump" / "precise.txt"), L)
    g = omega_gw(_precise(Path(got_dir) / "dump" / "precise.txt"), L)
    return _summary(_bins(list(g), list(r)))
