"""The C-ABI library: it loads, exports every entry point include/iegpu.h
declares, answers the calls that need no GPU, and refuses to run the lattice
without one (there is no CPU fallback)."""
from __future__ import annotations

import ctypes as C
import re

import pytest

from conftest import ROOT


def declared_symbols() -> list[str]:
    text = (ROOT / "include" / "iegpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(iegpu_[a-zA-Z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_symbols()
    assert len(names) >= 25
    for must in ("iegpu_create", "iegpu_leapfrog", "iegpu_spectrum", "iegpu_deltaN_steps", "iegpu_gw_spectrum"):
        assert must in names


def test_library_exports_every_declared_symbol(engine):
    lib = engine.load()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_calls_without_device(engine):
    lib = engine.load()
    assert lib.iegpu_version() >= 1
    assert lib.iegpu_strerror(engine.ERANGE).decode().startswith("field value")
    for N in (8, 16, 64, 256, 512):
        assert lib.iegpu_numbins(N) == int(1.73205 * (N // 2)) + 1


def test_create_rejects_bad_config(engine):
    lib = engine.load()
    h = C.c_void_p()
    bad = engine.Config(12, 0, 0, 0, -1, 10.0, 1e-3, 0.0, 1.0, 1.0, 0.97)  # N not a power of two
    assert lib.iegpu_create(C.byref(bad), C.byref(h)) == engine.EINVAL
    assert not h.value


def test_no_cpu_fallback_without_gpu(engine):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(engine.IegpuError):
        engine.Lattice(16, 10.0, 1e-3, 3.338e-13)
