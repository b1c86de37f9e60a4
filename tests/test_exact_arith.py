"""The engine's exact arithmetic on the CPU (no device needed).

inflation-easy_gb300/csrc/exact.cuh holds the two pieces of the plain FP64
form that run on the integer pipes: the exact lattice sum (256-bit fixed
point, rounded once) and the exact division by a fixed divisor (B^2).  Its
host build (tests/native/exact_arith_check.cu, compiled with nvcc) is checked
here: the division bit for bit against IEEE division over random dividends
and divisors, the sum against Python's math.fsum (Shewchuk's correctly
rounded sum) and the oracle's long accumulator, and the sum of exact
products against exact rational arithmetic.
"""
from __future__ import annotations

import math
import shutil
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
CSRC = HERE.parent / "inflation-easy_gb300" / "csrc"


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    exe = tmp_path_factory.mktemp("exact") / "exact_arith_check"
    subprocess.check_call([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off", f"-I{CSRC}",
                           str(HERE / "native" / "exact_arith_check.cu"), "-o", str(exe)])
    return exe


def test_division_by_fixed_divisor_is_ieee(checker):
    out = subprocess.run([str(checker), "div", "12345", "400000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert out.stdout.strip().endswith("mismatches 0"), out.stdout


def _engine_sum(checker, tmp_path, x):
    p = tmp_path / "terms.bin"
    np.ascontiguousarray(x, dtype="<f8").tofile(p)
    out = subprocess.run([str(checker), "sum", str(p)], capture_output=True, text=True, check=True).stdout.split()
    return struct.unpack("<d", bytes.fromhex(out[0])[::-1])[0], int(out[1])


def test_exact_sum_is_the_correctly_rounded_sum(checker, tmp_path, oracle_mod):
    rng = np.random.default_rng(3)
    f = 0.0935 + 1e-6 * rng.standard_normal(20000)
    lap = np.roll(f, 1) + np.roll(f, -1) - 2.0 * f
    cases = [
        f * lap,                                           # the gradient sum's terms
        f * f,                                             # the hilltop potential sum's terms
        rng.standard_normal(50000) * 10.0 ** rng.integers(-40, 8, 50000),
        np.array([1.0, 2.0 ** -53]),                       # a tie, to even
        np.array([1.0, 2.0 ** -53, 2.0 ** -105]),
        np.array([-1.0, -(2.0 ** -53), 3 * 2.0 ** -53]),
        np.array([2.0 ** 29, 2.0 ** 29, -(2.0 ** -150)]),
        np.array([0.1] * 10 + [-0.0]),
        np.array([]),
    ]
    for x in cases:
        s, flags = _engine_sum(checker, tmp_path, x)
        assert flags == 0
        want = math.fsum(x)
        assert s == want, (s, want)
        assert oracle_mod.exact_sum(x) == want


def test_exact_sum_of_products(checker, tmp_path, oracle_mod):
    """Sums of exact products (the engine's sums of f lapl(f), f^2, fd^2)
    against Fractions and the oracle's long accumulator."""
    from fractions import Fraction
    rng = np.random.default_rng(11)
    f = 0.0935 + 1e-6 * rng.standard_normal(3000)
    lap = np.roll(f, 1) + np.roll(f, -1) - 2.0 * f
    cases = [(f, lap), (f, f), (rng.standard_normal(3000) * 1e-3, rng.standard_normal(3000)),
             # a cancelling pair and a small product whose bits all lie above 2^-192
             (np.array([3.0, -3.0, 1e-12]), np.array([1.0 / 3.0, 1.0 / 3.0, 1e-12]))]
    for x, y in cases:
        p = tmp_path / "pairs.bin"
        np.ascontiguousarray(np.stack([x, y], axis=1).ravel(), dtype="<f8").tofile(p)
        out = subprocess.run([str(checker), "sumprod", str(p)], capture_output=True, text=True,
                             check=True).stdout.split()
        got = struct.unpack("<d", bytes.fromhex(out[0])[::-1])[0]
        assert int(out[1]) == 0
        want = float(sum((Fraction(a) * Fraction(b) for a, b in zip(x, y)), Fraction(0)))
        assert got == want
        assert oracle_mod.exact_dot(x, y) == want


def test_exact_sum_drops_bits_below_its_range(checker, tmp_path):
    """The accumulator's least significant bit is 2^-192: a product below it
    adds nothing (lattice terms never come near it)."""
    p = tmp_path / "pairs.bin"
    np.array([1.0, 1.0, 1e-40, 1e-40], dtype="<f8").tofile(p)
    out = subprocess.run([str(checker), "sumprod", str(p)], capture_output=True, text=True, check=True).stdout.split()
    assert struct.unpack("<d", bytes.fromhex(out[0])[::-1])[0] == 1.0


def test_exact_sum_flags_terms_it_cannot_hold(checker, tmp_path):
    _, flags = _engine_sum(checker, tmp_path, np.array([1.0, 2.0 ** 30]))
    assert flags == 2
    _, flags = _engine_sum(checker, tmp_path, np.array([1.0, np.nan]))
    assert flags == 1
