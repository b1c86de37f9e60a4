"""Pin the oracle against the reference program built from its own sources.

Runs only where the reference tree is available (it is read at build time by
oracle/build_ref.py); elsewhere the committed golden fixtures
(test_oracle_golden.py) carry the same check.  Configurations beyond the
fixtures: hilltop with SIGW, USR without SIGW, USR at N = 32, and the RK4 /
RK45 integrators of the inflation, deltaN and post-inflation loops.
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, INPUTS, ORACLE

sys.path.insert(0, str(ORACLE))
import build_ref  # noqa: E402

pytestmark = pytest.mark.skipif(not build_ref.ref_available(), reason="reference tree not present")

HILL = (GOLDEN / "n16_hilltop" / "params.txt").read_text()
USR = (GOLDEN / "n16_usr_sigw" / "params.txt").read_text()

# (N, numerical, SIGW, post-inflation phase, params text)
CASES = [
    (16, False, True, False, HILL),
    (16, True, False, False, USR),
    (32, True, True, False, USR),
    (16, False, True, True, HILL),
    (16, True, True, False, USR + "inflation_integrator = rk4\n"),
    (16, False, False, False, HILL + "inflation_integrator = rk45\n"),
    # a step large enough for the step control to act: h from 6e-4 to 0.04, one rejection
    (16, False, False, False, HILL.replace("dt = 0.001", "dt = 0.05")
     + "inflation_integrator = rk45\nrk45_abs_tol = 1e-12\nrk45_rel_tol = 1e-10\n"),
    (16, True, True, False, USR + "inflation_integrator = dopri5\nrk45_rel_tol = 1e-7\n"),
    (16, False, True, True, HILL + "post_inflation_integrator = rk4\n"),
    (16, True, True, True, USR + "post_inflation_integrator = rk45\n"),
    (16, False, False, False, HILL + "deltaN_integrator = rk4\n"),
    (16, True, False, False, USR + "deltaN_integrator = rk4\n"),
    (16, False, False, False, HILL + "deltaN_integrator = rk45\n"),
    (16, True, False, False, USR + "deltaN_integrator = rkf45\n"),
]


@pytest.mark.parametrize("N,numerical,sigw,post,text", CASES)
def test_oracle_matches_reference(N, numerical, sigw, post, text, oracle_mod, tmp_path):
    exe = build_ref.build(N, int(numerical), int(sigw), 1, post=int(post))
    wd = tmp_path / "ref"
    wd.mkdir()
    (wd / "params.txt").write_text(text)
    os.symlink(INPUTS, wd / "inputs")
    # the RK right-hand side sums with an OpenMP reduction, whose order follows
    # the thread count; one thread gives the serial loop order the oracle uses
    env = dict(os.environ, OMP_NUM_THREADS="1") if "integrator" in text else None
    subprocess.run([str(exe), str(wd)], check=True, stdout=subprocess.DEVNULL, env=env)
    p = oracle_mod.params_from_text(text, N, numerical, sigw, post=post)
    assert oracle_mod.run_program(p, tmp_path / "results", INPUTS, tmp_path) == 0
    for f in sorted((wd / "results").rglob("*")):
        if f.is_dir() or f.name == "info.dat":
            continue
        rel = f.relative_to(wd / "results")
        assert f.read_bytes() == (tmp_path / "results" / rel).read_bytes(), str(rel)
    assert (wd / "trace.txt").read_text() == (tmp_path / "trace.txt").read_text()
    ref = oracle_mod.read_state(wd / "state.bin")
    got = oracle_mod.read_state(tmp_path / "state.bin")
    for k in ref:
        assert np.array_equal(ref[k], got[k]), k


@pytest.mark.parametrize("N", [8, 16, 32])
def test_oracle_forcing_cutoff_matches_fresh_reference_runs(N, oracle_mod, tmp_path):
    """The reference's spectraf() with the forcing cutoff (src/output.cpp:297-406),
    run afresh (ie_ref --spectraf) on random f and fd other than the committed
    fixtures', for cutoffs across the whole range of |p| (with and without a low
    one): f and fd after the call equal the oracle's bit for bit."""
    exe = build_ref.build(N, 0, 0, 1)
    rng = np.random.default_rng(7000 + N)
    f = rng.standard_normal(N ** 3) * 1e-3 + 0.09
    fd = rng.standard_normal(N ** 3) * 1e-5
    pmax = np.sqrt(3.0) * N / 2
    for q, (hi, lo) in enumerate([(0.3 * pmax, 0.0), (0.55 * pmax, 1.0), (0.8 * pmax, 0.5 * N / 4),
                                  (N / 2, 0.0), (pmax + 1, 0.0)]):
        wd = tmp_path / f"cut{q}"
        (wd / "results").mkdir(parents=True)
        with open(wd / "cut_in.bin", "wb") as fp:
            fp.write(f.tobytes())
            fp.write(fd.tobytes())
            fp.write(np.array([hi, lo]).tobytes())
        subprocess.run([str(exe), "--spectraf", str(wd)], check=True, stdout=subprocess.DEVNULL)
        out = np.fromfile(wd / "cut_out.bin", dtype=np.float64)
        o = oracle_mod.Oracle(oracle_mod.default_params(N, False))
        o.f[:] = f
        o.fd[:] = fd
        o.spectrum_f(hi, lo)
        assert np.array_equal(o.f.view(np.uint64), out[:N ** 3].view(np.uint64)), (N, hi, lo, "f")
        assert np.array_equal(o.fd.view(np.uint64), out[N ** 3:].view(np.uint64)), (N, hi, lo, "fd")
