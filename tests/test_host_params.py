"""The host program's params.txt handling against the oracle's restatement of
the reference's loader (src/runtime_parameters.cpp:17-112, 141-192, 195-365),
with no device: `ie_gpu_main --check-params` prints the resolved values and
the RK45 controls the library derives with iegpu_rk45_effective.

Covered: the reference's defaults for both potentials, integrator names in
any case and as integer codes, invalid integrator values (ignored, with the
reference's warning), and the RK45 sanitisation (non-positive or crossed step
bounds, out-of-range tolerances and safety).
"""
from __future__ import annotations

import ctypes as C
import subprocess

import pytest

from conftest import PKG

MAIN = PKG / "_build" / "ie_gpu_main"

KEYS = ["N", "numerical_potential", "criterion", "seed", "rescale_s", "af", "V0", "rescale_B", "ns",
        "initial_field", "initial_derivative", "L", "dt", "dx", "output_freq", "output_infrequent_freq", "dN",
        "Nend", "horizon_factor", "omega", "dt_post_inflation", "af_post_inflation", "inflation_integrator",
        "deltaN_integrator", "post_inflation_integrator", "rk45_abs_tol", "rk45_rel_tol", "rk45_min_dt",
        "rk45_max_dt", "rk45_safety"]

CASES = {
    "usr_defaults": (32, 1, ""),
    "hilltop_defaults": (64, 0, ""),
    "aliases": (16, 1, "inflation_integrator = LF\ndeltaN_integrator = RKF45\npost_inflation_integrator = 1\n"),
    "more_aliases": (16, 0, "inflation_integrator = Rk4\ndeltaN_integrator = dopri5\n"
                            "post_inflation_integrator = 2\n"),
    "invalid_integrators": (16, 0, "inflation_integrator = rk5\ndeltaN_integrator = 7\n"
                                   "post_inflation_integrator = -1\n"),
    "rk45_sanitised": (16, 1, "dt = 0.002\nrk45_min_dt = -3\nrk45_max_dt = 1e-12\nrk45_safety = 1.5\n"
                              "rk45_abs_tol = 0\nrk45_rel_tol = 1e-9\n"),
    "rk45_given": (16, 0, "rk45_min_dt = 1e-7\nrk45_max_dt = 0.5\nrk45_safety = 0.8\nrk45_abs_tol = 1e-11\n"),
    "derived_overrides": (32, 0, "af = 12.5\nrescale_B = 2e-5\naf_post_inflation = 40\nL = 7.5\nseed = 3\n"
                                 "dt = 0.0005\ncriterion = 0\n"),
}


def _host(path):
    r = subprocess.run([str(MAIN), "--check-params", str(path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = {}
    for line in r.stdout.splitlines():
        k, v = line.split()
        out[k] = float(v)
    return out, r.stderr


def _oracle(oracle_mod, N, numerical, path):
    lib = oracle_mod.load()
    p = oracle_mod.Params()
    lib.ieo_params_defaults(C.byref(p), N, numerical)
    lib.ieo_params_load(C.byref(p), str(path).encode())
    return p


@pytest.mark.parametrize("case", sorted(CASES))
def test_params_match_the_oracle(case, oracle_mod, tmp_path):
    assert MAIN.exists(), "build the engine first (__graft_entry__.build())"
    N, numerical, extra = CASES[case]
    path = tmp_path / "params.txt"
    path.write_text(f"N = {N}\nnumerical_potential = {numerical}\n" + extra)
    got, err = _host(path)
    ref = _oracle(oracle_mod, N, numerical, path)
    for k in KEYS:
        assert got[k] == float(getattr(ref, k)), (case, k, got[k], getattr(ref, k))
    if case == "invalid_integrators":
        assert "Ignoring invalid inflation_integrator 'rk5'" in err
        assert "Ignoring invalid deltaN_integrator '7'" in err


def test_rk45_effective_without_a_device(engine):
    """iegpu_rk45_effective needs no context: the reference's sanitisation."""
    lib = engine.load()
    ctl = engine.Rk45Controls(-1.0, 2e-6, 0.0, -5.0, 1.0)
    out = engine.Rk45Controls()
    assert lib.iegpu_rk45_effective(C.byref(ctl), -0.004, C.byref(out)) == 0
    assert (out.abs_tol, out.rel_tol, out.min_dt, out.max_dt, out.safety) == (1e-8, 2e-6, 0.004 * 1e-6, 0.004, 0.9)


@pytest.mark.parametrize("form", ["split", "split_comp"])
def test_forcing_cutoff_needs_the_fp64_form(form, tmp_path):
    """forcing_cutoff with high_cutoff_index > 0 (src/output.cpp:330-401)
    runs on the plain FP64 form; on the split forms the program stops with a
    message before any device work."""
    assert MAIN.exists(), "build the engine first (__graft_entry__.build())"
    (tmp_path / "params.txt").write_text(f"N = 128\nnumerical_potential = 0\nform = {form}\nforcing_cutoff = 1\n"
                                         "high_cutoff_index = 5.5\n")
    r = subprocess.run([str(MAIN), "params.txt", "results", "dump"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1
    assert "forcing_cutoff runs on the plain FP64 form" in r.stdout + r.stderr
