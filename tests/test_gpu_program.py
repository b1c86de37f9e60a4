"""End-to-end parity of the host program (ie_gpu_main, which drives the CUDA
engine through the C ABI) with the reference.

1. Against the golden fixtures made by the reference program itself: every
   results file is compared number by number at its printed precision, the
   final lattice state element by element.
2. Against the oracle program on the hilltop workload at N = 64 (the
   reference's own CPU-sized case) and the USR table at N = 32, at full
   precision (details in test_program_full_precision_against_oracle):
     engine-arithmetic oracle: a, H bit for bit; spectra per bin 1e-11
     reference oracle: a, H, <phi> relative 1e-10; P_dphi, P_zeta per k-bin
     relative 1e-8, or twice the reference's own rounding floor where that
     is larger; k-shell bin counts exact
"""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, INPUTS, PKG

pytestmark = pytest.mark.gpu

MAIN = PKG / "_build" / "ie_gpu_main"

CASES = {
    "n16_hilltop": (16, 0, 0),
    "n16_hilltop_rk4": (16, 0, 0),   # inflation_integrator = rk4
    "n16_hilltop_rk45": (16, 0, 0),  # inflation_integrator = rk45, dt = 0.05: the step control acts
    "n16_usr_sigw": (16, 1, 1),
    "n16_usr_dn_rk45": (16, 1, 0),   # deltaN_integrator = rk45
    "n32_hilltop": (32, 0, 0),
    "n16_hilltop_cutoff": (16, 0, 0),   # forcing_cutoff = 1, high_cutoff_index = 5.5
}

# Bounds for the final f (ulp) and the background trace (relative).  With the
# RK45 step control acting, the embedded error estimate magnifies the
# rounding of re-associated sums; the reference itself differs between its own
# 1- and 8-thread runs of n16_hilltop_rk45 by 58626 ulp in f and 1.1e-9 in the
# trace, so that case gets bounds above its own spread.
BOUNDS = {"n16_hilltop_rk45": (1 << 17, 5e-9)}


def run_main(tmp_path, params_text, N, numerical, sigw):
    wd = tmp_path / "gpu"
    wd.mkdir()
    # ic_on_host = 1: the modes are drawn with the host maths library, bit-identical to the reference
    text = params_text + (f"N = {N}\nnumerical_potential = {numerical}\ncalculate_SIGW = {sigw}\nperform_deltaN = 1\n"
                          "ic_on_host = 1\n")
    (wd / "params.txt").write_text(text)
    os.symlink(INPUTS, wd / "inputs")
    (wd / "dump").mkdir()
    r = subprocess.run([str(MAIN), "params.txt", "results", "dump"], cwd=wd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return wd


def parse_numbers(path):
    rows = []
    for line in path.read_text().splitlines():
        if line.strip():
            rows.append([float(x) for x in line.split()])
    return rows


def compare_text(ref_path, got_path, rel, field_std=None):
    a, b = parse_numbers(ref_path), parse_numbers(got_path)
    assert len(a) == len(b), f"{ref_path.name}: {len(a)} vs {len(b)} rows"
    A = np.array([x for r in a for x in r])
    B = np.array([x for r in b for x in r])
    assert A.shape == B.shape, ref_path.name
    if field_std is not None:
        err = np.max(np.abs(A - B)) / field_std
        assert err < rel, f"{ref_path.name}: {err}"
        return
    scale = np.max(np.abs(A)) if A.size else 0.0
    bad = np.abs(A - B) > rel * np.abs(A) + 1e-12 * scale
    assert not bad.any(), f"{ref_path.name}: {A[bad][:5]} vs {B[bad][:5]}"


@pytest.mark.parametrize("case", sorted(CASES))
def test_program_matches_reference_fixtures(case, tmp_path):
    N, num, sigw = CASES[case]
    src = GOLDEN / case
    wd = run_main(tmp_path, (src / "params.txt").read_text(), N, num, sigw)
    ref_state = np.load(src / "state.npz")
    names = sorted(x.name for x in (src / "results").iterdir())
    got_names = sorted(x.name for x in (wd / "results").iterdir() if x.name not in ("info.dat", "output.txt"))
    assert names == got_names
    for name in names:
        if name.startswith("snapshots_2d"):
            key = {"phi": "f", "phidot": "fd", "deltaN": "deltaN"}[name[len("snapshots_2d_"):-4]]
            std = float(np.std(ref_state[key]))
            compare_text(src / "results" / name, wd / "results" / name, 1e-3, field_std=std)
        elif name.startswith("histogram") and not name.startswith("histogramtimes"):
            a = np.concatenate([np.array(r) for r in parse_numbers(src / "results" / name)])
            b = np.concatenate([np.array(r) for r in parse_numbers(wd / "results" / name)])
            assert np.max(np.abs(a - b)) <= 2.0 / N ** 3 + 1e-12, name
        elif name.startswith("spectraGW"):
            compare_text(src / "results" / name, wd / "results" / name, 2e-5)
        else:
            compare_text(src / "results" / name, wd / "results" / name, 2e-6)
    import ieo
    got = ieo.read_state(wd / "dump" / "state.bin")
    # fields: the per-site arithmetic is the reference's, but the lattice sums
    # that feed the Friedmann update are re-associated, so the two runs drift
    # apart by a few units in the last place of the background value
    ref = ref_state["f"]
    d = np.abs(got["f"] - ref)
    ulps = np.max(d / np.spacing(np.abs(ref)))
    print(f"{case} f: max dev {np.max(d):.3e} = {ulps:.0f} ulp of f, std {np.std(ref):.3e}")
    max_ulps, trace_rel = BOUNDS.get(case, (4096, 1e-10))
    assert ulps < max_ulps
    # fd ends the deltaN stage in e-fold units, near zero at many sites, so it
    # is compared against its own spread
    ref = ref_state["fd"]
    d = np.abs(got["fd"] - ref)
    print(f"{case} fd: max dev {np.max(d):.3e}, std {np.std(ref):.3e}")
    assert np.max(d) <= 1e-3 * np.std(ref)
    ref = ref_state["deltaN"]
    zeta = ref - ref.mean()
    d = np.abs(got["deltaN"] - ref)
    print(f"{case} deltaN: max dev {np.max(d):.3e}, std(zeta) {np.std(zeta):.3e}")
    assert np.max(d) / np.std(zeta) < 1e-3
    # background scalars at every save, full precision: t, a, ad, astep (and
    # t, a, Ne, phiref at saveN) relative 1e-10.  ad2 is the Friedmann
    # solution -2ad - 2a/(d(s+1)) (1 - sqrt(1 + x)) with x = O(d): two
    # cancellations, each losing about log10(1/d) digits, turn the ulp-level
    # differences of its inputs into ~1e-9 relative, so it gets 1e-6.
    ta = [l.split() for l in (src / "trace.txt").read_text().splitlines()]
    tb = [l.split() for l in (wd / "dump" / "trace.txt").read_text().splitlines()]
    assert len(ta) == len(tb)
    worst_ad2 = 0.0
    for x, y in zip(ta, tb):
        assert x[0] == y[0]
        for col, (u, v) in enumerate(zip(x[2:] if x[0] == "save" else x[1:], y[2:] if y[0] == "save" else y[1:])):
            u, v = float(u), float(v)
            if x[0] == "save" and col == 3:
                worst_ad2 = max(worst_ad2, abs(u - v) / max(abs(u), 1e-300))
                assert abs(u - v) <= 1e-6 * abs(u) + 1e-300, (x, y)
            else:
                assert abs(u - v) <= trace_rel * abs(u) + 1e-300, (x, y)
    print(f"{case} ad2: max rel dev {worst_ad2:.3e}")


def _precise(path):
    out = {}
    for line in path.read_text().splitlines():
        tag, *vals = line.split()
        out.setdefault(tag, []).append(np.array([float(v) for v in vals]))
    return out


def _bin_dev(got, ref):
    """Largest relative deviation per k-bin over every save (bins where the
    reference is zero: the absolute value)."""
    dev = np.zeros(len(ref[0]))
    for x, y in zip(got, ref):
        with np.errstate(divide="ignore", invalid="ignore"):
            dev = np.maximum(dev, np.where(y != 0, np.abs(x / y - 1), np.abs(x)))
    return dev


@pytest.mark.parametrize("N,numerical,extra", [(64, 0, ""), (32, 1, ""),
                                              # the USR table at 128^3 (its workload's size), inflation
                                              # shortened to af = 1.35 (about 520 steps) and the deltaN
                                              # stage to Nend = 0.1 (1000 steps) so the oracle ends in
                                              # seconds
                                              (128, 1, "af = 1.35\nNend = 0.1\n")])
def test_program_full_precision_against_oracle(N, numerical, extra, tmp_path, oracle_mod):
    """The whole program (inflation to af, deltaN stage, spectra) against the
    oracle program twice:
      * in engine-arithmetic mode (lattice sums formed exactly, as the engine
        forms them): a and H bit for bit at every save, <phi> to 1e-12 (the
        output's sum of the field is a tree sum here and a serial one there),
        P_dphi and P_zeta per k-bin to 1e-11 (the spectra's bin sums
        likewise);
      * in reference mode (serial sums, libm pow): a, H, <phi> relative 1e-10;
        P_dphi and P_zeta per k-bin relative 1e-8, except where the
        reference's own rounding floor is larger.  The floor is measured here
        as the deviation between the two oracle runs, i.e. between two valid
        roundings of the reference's algorithm; a bin whose floor exceeds
        5e-9 is held to twice its floor instead, and is printed.
    Bin counts are exact in both."""
    src = GOLDEN / ("n16_usr_sigw" if numerical else "n16_hilltop")
    text = (src / "params.txt").read_text() + "\n" + extra
    wd = run_main(tmp_path, text, N, numerical, 0)
    p = oracle_mod.params_from_text(text, N, bool(numerical), False)
    od, oe = tmp_path / "oracle", tmp_path / "oracle_engine"
    for d, mode in ((od, False), (oe, True)):
        d.mkdir()
        assert oracle_mod.run_program(p, d / "results", INPUTS, d, engine_arith=mode) == 0
    g, o, e = (_precise(x / "precise.txt") for x in (wd / "dump", od, oe))
    assert len(g["means"]) == len(o["means"]) == len(e["means"])
    for x, y, z in zip(g["means"], o["means"], e["means"]):
        assert np.allclose(x[[1, 2, 4]], y[[1, 2, 4]], rtol=1e-10, atol=0)  # a, <phi>, H
        assert x[1] == z[1] and x[4] == z[4]                                 # a, H
        assert np.allclose(x[2], z[2], rtol=1e-12, atol=0)                   # <phi>
    for tag in ("spectrum", "spectrumN"):
        assert len(g[tag]) == len(o[tag]) == len(e[tag])
        dev_ref = _bin_dev(g[tag], o[tag])
        dev_eng = _bin_dev(g[tag], e[tag])
        floor = _bin_dev(e[tag], o[tag])
        bound = np.where(floor > 5e-9, 2.0 * floor, 1e-8)
        exempt = np.nonzero(floor[1:] > 5e-9)[0] + 1
        print(f"{tag} N={N}: vs engine-mode oracle max {dev_eng[1:].max():.2e}; vs reference max "
              f"{dev_ref[1:].max():.2e}; reference floor max {floor[1:].max():.2e}; bins held to 2x floor: "
              f"{exempt.tolist()}")
        print(f"{tag} N={N} per bin vs reference: " + " ".join(f"{v:.1e}" for v in dev_ref))
        print(f"{tag} N={N} per bin floor:        " + " ".join(f"{v:.1e}" for v in floor))
        assert dev_eng[1:].max() < 1e-11, tag
        assert np.all(dev_ref[1:] <= bound[1:]), tag
    # exact bin counts
    for name in ("spectra.dat", "spectraN.dat"):
        ca = [r[1] for r in parse_numbers(wd / "results" / name)]
        cb = [r[1] for r in parse_numbers(od / "results" / name)]
        assert ca == cb


def test_program_gw_spectra_byte_exact_with_engine_arithmetic(tmp_path, oracle_mod):
    """spectraGW.dat and spectraGWdot.dat of the program (16^3 USR with SIGW,
    inflation to af, deltaN stage) against the oracle program in
    engine-arithmetic mode, byte for byte: h and h' are bit-exact there, and
    the spectra use the reference's float accumulators in its loop order
    (src/output.cpp:478-612), divided and normalised in float as it does."""
    text = (GOLDEN / "n16_usr_sigw" / "params.txt").read_text()
    wd = run_main(tmp_path, text, 16, 1, 1)
    p = oracle_mod.params_from_text(text, 16, True, True)
    d = tmp_path / "oracle_engine"
    d.mkdir()
    assert oracle_mod.run_program(p, d / "results", INPUTS, d, engine_arith=True) == 0
    for name in ("spectraGW.dat", "spectraGWdot.dat"):
        assert (wd / "results" / name).read_bytes() == (d / "results" / name).read_bytes(), name


@pytest.mark.parametrize("case", ["n16_usr_sigw_post", "n16_usr_sigw_post_rk45"])
def test_program_post_inflation_matches_reference_fixture(case, tmp_path):
    """The program with the post-inflation phase on (16^3, USR, SIGW, deltaN;
    leapfrog, or RK45 with post_inflation_integrator = rk45) against the
    reference program's own outputs of that phase (tests/golden/<case>):
    results/post_inflation/* number by number, and the final fields.  The
    phase starts from the deltaN map, which the engine reproduces to
    round-off (its sums are re-associated), so the tolerances are those of
    the inflation outputs above."""
    src = GOLDEN / case
    text = (src / "params.txt").read_text() + "post_inflation = 1\n"
    wd = run_main(tmp_path, text, 16, 1, 1)
    names = sorted(x.name for x in (src / "results" / "post_inflation").iterdir())
    got_names = sorted(x.name for x in (wd / "results" / "post_inflation").iterdir())
    assert names == got_names
    ref_state = np.load(src / "state.npz")
    for name in names:
        a = src / "results" / "post_inflation" / name
        b = wd / "results" / "post_inflation" / name
        A = np.concatenate([np.array(r) for r in parse_numbers(a)])
        B = np.concatenate([np.array(r) for r in parse_numbers(b)])
        assert A.shape == B.shape, name
        rel = np.max(np.abs(A - B) / (np.abs(A) + 1e-300 + 1e-12 * np.max(np.abs(A))))
        print(f"post {name}: max rel dev {rel:.3e}")
        if name.startswith("histogram") and not name.startswith("histogramtimes"):
            assert np.max(np.abs(A - B)) <= 2.0 / 16 ** 3 + 1e-12, name
        elif name.startswith("spectraGW"):
            compare_text(a, b, 2e-5)
        else:
            compare_text(a, b, 2e-6)
    import ieo
    got = ieo.read_state(wd / "dump" / "state.bin")
    for key in ("f", "fd"):
        ref = ref_state[key]
        d = np.max(np.abs(got[key] - ref)) / np.std(ref)
        print(f"post {key}: max dev / std {d:.3e}")
        assert d < 1e-6, key
    for key in ("h", "hd"):
        ref = ref_state[key].astype(np.float64)
        d = np.max(np.abs(got[key].astype(np.float64) - ref)) / np.std(ref)
        print(f"post {key}: max dev / std {d:.3e}")
        assert d < 1e-4, key
    ta = [l.split() for l in (src / "trace.txt").read_text().splitlines() if l.startswith("savep")]
    tb = [l.split() for l in (wd / "dump" / "trace.txt").read_text().splitlines() if l.startswith("savep")]
    assert len(ta) == len(tb) and len(ta) > 2
    for x, y in zip(ta, tb):
        for u, v in zip(x[2:], y[2:]):
            u, v = float(u), float(v)
            assert abs(u - v) <= 1e-10 * abs(u) + 1e-300, (x, y)
