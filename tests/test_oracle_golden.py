"""The oracle against the golden fixtures made by the reference program.

Each fixture in tests/golden/<case>/ was produced by the unmodified reference
(tests/golden/make_golden.py).  The oracle, run on the same params.txt, must
reproduce every results file byte for byte, the full-precision trace of the
background scalars at each save(), and the final lattice state bit for bit.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, INPUTS

# case: (N, numerical, SIGW, post-inflation phase)
CASES = {
    "n16_hilltop": (16, False, False, False),
    "n16_usr_sigw": (16, True, True, False),
    "n32_hilltop": (32, False, False, False),
    "n16_usr_sigw_post": (16, True, True, True),
    "n16_hilltop_rk4": (16, False, False, False),
    "n16_hilltop_rk45": (16, False, False, False),
    "n16_usr_sigw_post_rk45": (16, True, True, True),
    "n16_usr_dn_rk45": (16, True, False, False),
    "n16_hilltop_cutoff": (16, False, False, False),   # forcing_cutoff = 1, high_cutoff_index = 5.5
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_reproduces_reference_outputs(case, oracle_mod, tmp_path):
    N, numerical, sigw, post = CASES[case]
    src = GOLDEN / case
    p = oracle_mod.params_from_text((src / "params.txt").read_text(), N, numerical, sigw, post=post)
    rc = oracle_mod.run_program(p, tmp_path / "results", INPUTS, tmp_path)
    assert rc == 0
    golden_files = sorted(str(x.relative_to(src / "results")) for x in (src / "results").rglob("*") if x.is_file())
    assert golden_files, "empty fixture"
    for name in golden_files:
        a = (src / "results" / name).read_bytes()
        b = (tmp_path / "results" / name).read_bytes()
        assert a == b, f"{case}: {name} differs"
    assert (src / "trace.txt").read_text() == (tmp_path / "trace.txt").read_text()
    ref = np.load(src / "state.npz")
    got = oracle_mod.read_state(tmp_path / "state.bin")
    for key in ref.files:
        assert np.array_equal(ref[key], got[key]), f"{case}: state {key} differs"


@pytest.mark.parametrize("N", [8, 16])
def test_oracle_forcing_cutoff_matches_reference(N, oracle_mod):
    """spectraf() with the forcing cutoff (src/output.cpp:330-401) on seeded
    random f and fd: the reference's f and fd after the call
    (tests/golden/forcing_cutoff/, made by ie_ref --spectraf), bit for bit,
    for high and low cutoffs (a low one zeroes the k = 0 mode too)."""
    g = np.load(GOLDEN / "forcing_cutoff" / f"cut_n{N}.npz")
    for q, (hi, lo) in enumerate(g["cuts"]):
        o = oracle_mod.Oracle(oracle_mod.default_params(N, False))
        o.f[:] = g["f_in"]
        o.fd[:] = g["fd_in"]
        o.spectrum_f(hi, lo)
        assert np.array_equal(o.f.view(np.uint64), g[f"f_{q}"].view(np.uint64)), (N, hi, lo, "f")
        assert np.array_equal(o.fd.view(np.uint64), g[f"fd_{q}"].view(np.uint64)), (N, hi, lo, "fd")
