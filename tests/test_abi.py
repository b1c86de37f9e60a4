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


def test_rk_entry_points_reject_null_arguments(engine):
    """The Runge-Kutta entry points check their arguments before any device
    call: a null context returns IEGPU_EINVAL."""
    lib = engine.load()
    bg = engine.Bg(0.0, 1.0, 1.0, 0.0, 1.0)
    ctl = engine.Rk45Controls()
    h, ne, out = C.c_double(1e-3), C.c_double(0.0), C.c_double()
    steps, acc = C.c_int(), C.c_int()
    calls = [
        lambda: lib.iegpu_rk4(None, 2.0, 1, C.byref(bg), C.byref(steps), None),
        lambda: lib.iegpu_rk4_step_inflation(None, 1e-3, C.byref(bg)),
        lambda: lib.iegpu_rk45(None, C.byref(ctl), 2.0, 1, C.byref(h), C.byref(bg), C.byref(steps), None),
        lambda: lib.iegpu_rk45_step_inflation(None, C.byref(ctl), 1e-3, 1e-3, C.byref(out), C.byref(acc),
                                              C.byref(bg)),
        lambda: lib.iegpu_deltaN_rk4_steps(None, 1e-4, 1, 0.0, C.byref(bg)),
        lambda: lib.iegpu_deltaN_rk45(None, C.byref(ctl), 1e-4, 1.0, 1, 0.0, C.byref(h), C.byref(ne), C.byref(bg),
                                      C.byref(steps), None),
        lambda: lib.iegpu_post_inflation_rk4(None, 2.0, 1e-3, 1.0 / 3.0, 1, C.byref(bg), C.byref(steps), None),
        lambda: lib.iegpu_post_inflation_rk45(None, C.byref(ctl), 2.0, 1e-3, 1.0 / 3.0, 1, C.byref(h), C.byref(bg),
                                              C.byref(steps), None),
    ]
    for call in calls:
        assert call() == engine.EINVAL
    assert lib.iegpu_rk45_effective(None, 1e-3, C.byref(ctl)) == engine.EINVAL
    assert lib.iegpu_strerror(engine.ECONVERGE).decode().startswith("RK45")


def test_spectrum_and_ensemble_entry_points_reject_null_arguments(engine):
    """The forcing-cutoff spectrum, the reference-order GW spectrum and the
    ensemble's shape query check their arguments before any device call."""
    lib = engine.load()
    nb = lib.iegpu_numbins(16)
    counts = (C.c_int * nb)()
    f2 = (C.c_double * nb)()
    f2f = (C.c_float * nb)()
    assert lib.iegpu_spectrum_cutoff(None, counts, f2, nb, 5.5, 0.0) == engine.EINVAL
    assert lib.iegpu_gw_spectrum_ref(None, 0, C.c_double(1.0), counts, f2f, f2, nb) == engine.EINVAL
    assert lib.iegpu_ens_shapes(None, None, None, None) == engine.EINVAL
