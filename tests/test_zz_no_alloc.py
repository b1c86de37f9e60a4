"""The allocation-free shell binning, iegpu_shell_spectrum_noalloc.

Some callers cannot allocate device memory: a plugin whose host framework
owns all device memory through its own caching allocator and forbids direct
cudaMalloc, or a process whose fixed memory budget is already spent on the
lattice.  For them the library offers this one entry point, whose scratch is a
fixed array inside the library.
Checked through the C ABI against the context-based iegpu_spectrum on two
calls in a row -- the second call must not see anything the first one left in
the shared array -- at the tolerance the other spectrum tests use: bin counts
exact, per-bin sums relative 1e-12 (only the summation order differs).
This file is collected last on purpose.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("N", [32, 256, 512])
def test_noalloc_matches_context_spectrum(N, engine):
    """N = 512 is the array's limit: 444 bins, the largest shared-memory use of
    the binning kernel (4 warps x 444 bins x 12 B)."""
    torch = pytest.importorskip("torch")
    lib = engine.load()
    nb = lib.iegpu_numbins(N)
    rng = np.random.default_rng(7)
    dev = torch.device("cuda", 0)
    with engine.Lattice(N, 10.0, 1e-3, 3.338e-13) as lat:
        for call, amp in enumerate((1e-6, 3e-5)):
            x = 0.0935 + amp * rng.standard_normal(N ** 3)
            # the existing entry point: forward FFT, binning, inverse FFT
            lat.upload(engine.F, x)
            counts_ref, f2_ref = lat.spectrum(engine.F)
            # the same field's r2c modes, from the existing FFT entry point
            lat.upload(engine.F, x)
            lat.fft(engine.F, 1)
            modes, nyq = lat.download(engine.F, nyquist=True)
            d_modes = torch.from_numpy(modes).to(dev)
            d_nyq = torch.from_numpy(nyq).to(dev)
            d_counts = torch.full((nb,), -1, dtype=torch.int32, device=dev)
            d_f2 = torch.full((nb,), float("nan"), dtype=torch.float64, device=dev)
            stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
            rc = lib.iegpu_shell_spectrum_noalloc(_ptr(d_modes), _ptr(d_nyq), N, _ptr(d_counts), _ptr(d_f2), stream)
            assert rc == engine.OK, call
            torch.cuda.synchronize()
            assert np.array_equal(d_counts.cpu().numpy(), counts_ref), call
            assert np.allclose(d_f2.cpu().numpy(), f2_ref, rtol=1e-12, atol=0), call


def test_noalloc_rejects_sizes_above_its_limit(engine):
    lib = engine.load()
    # the size check comes before any device work; the pointers are never used
    fake = C.c_void_p(16)
    assert lib.iegpu_shell_spectrum_noalloc(fake, fake, 1024, fake, fake, None) == engine.ETOOBIG
    assert lib.iegpu_shell_spectrum_noalloc(fake, fake, 48, fake, fake, None) == engine.EINVAL
