"""Known-answer tests of the oracle's building blocks.

The reference ships no unit tests or golden vectors for these pieces, so the
answers come from closed forms: the Park-Miller sequence, the discrete
Fourier transform (numpy), Parseval, the lattice Laplacian eigenvalue of a
plane wave, the shell-bin multiplicities, and the homogeneous-field
background equation.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

M31 = 2 ** 31 - 1


def test_rng_park_miller_sequence(oracle_mod):
    # src/initialize.cpp:18-31: 99 warm-up calls, then x_{n+1} = 16807 x_n mod (2^31-1)
    for seed in (1, 8, 12345):
        o = oracle_mod.Oracle(oracle_mod.hilltop_params(8, seed=seed))
        got = [o.lib.ieo_rand_uniform(o.h) for _ in range(5)]
        want = [pow(16807, 100 + q, M31) * seed % M31 / M31 for q in range(5)]
        assert got == want


def test_rng_seed_below_one_is_constant(oracle_mod):
    o = oracle_mod.Oracle(oracle_mod.hilltop_params(8, seed=0))
    assert [o.lib.ieo_rand_uniform(o.h) for _ in range(3)] == [0.33] * 3


def _ffteasy_to_dense(out, ny, N):
    """Full complex spectrum F[i, j, k], k = 0..N/2, from the r2c layout."""
    c = out.reshape(N, N, N // 2, 2)
    F = np.empty((N, N, N // 2 + 1), dtype=complex)
    F[:, :, : N // 2] = c[..., 0] + 1j * c[..., 1]
    nyc = ny.reshape(N, N, 2)
    F[:, :, N // 2] = nyc[..., 0] + 1j * nyc[..., 1]
    return F


@pytest.mark.parametrize("N", [8, 16, 32])
def test_fft_forward_is_plus_sign_dft(N, oracle_mod):
    rng = np.random.default_rng(N)
    x = rng.standard_normal(N ** 3)
    f = x.copy()
    ny = np.zeros(2 * N * N)
    oracle_mod.fftrn_d(f, ny, N, 1)
    F = _ffteasy_to_dense(f, ny, N)
    # forward = +1 uses exp(+2 pi i k.x / N): the conjugate of numpy's fftn
    ref = np.conj(np.fft.rfftn(x.reshape(N, N, N)))
    assert np.allclose(F, ref, rtol=1e-12, atol=1e-10 * np.abs(ref).max())


@pytest.mark.parametrize("N", [8, 16, 32])
def test_fft_round_trip_and_parseval(N, oracle_mod):
    rng = np.random.default_rng(100 + N)
    x = rng.standard_normal(N ** 3)
    f = x.copy()
    ny = np.zeros(2 * N * N)
    oracle_mod.fftrn_d(f, ny, N, 1)
    F = _ffteasy_to_dense(f, ny, N)
    w = np.ones(N // 2 + 1)
    w[1:N // 2] = 2.0
    # Parseval with the r2c multiplicities (interior k counted twice)
    assert np.isclose(np.sum(w * np.abs(F) ** 2), N ** 3 * np.sum(x * x), rtol=1e-12)
    oracle_mod.fftrn_d(f, ny, N, -1)
    assert np.allclose(f, x, rtol=0, atol=1e-13)


@pytest.mark.parametrize("N", [8, 16, 64])
def test_bin_counts_closed_form(N, oracle_mod):
    f = np.zeros(N ** 3)
    ny = np.zeros(2 * N * N)
    counts, _ = oracle_mod.bin_spectrum(N, f, ny)
    p = np.fft.fftfreq(N, 1.0 / N).astype(int)
    p[N // 2] = N // 2
    pz = np.arange(N // 2 + 1)
    mag = np.sqrt(p[:, None, None] ** 2 + p[None, :, None] ** 2 + pz[None, None, :] ** 2)
    w = np.where((pz > 0) & (pz < N // 2), 2, 1)[None, None, :] * np.ones_like(mag, dtype=int)
    b = np.floor(mag + 0.5).astype(int)
    nb = int(1.73205 * (N // 2)) + 1
    want = np.bincount(b[b < nb], weights=w[b < nb], minlength=nb).astype(int)
    assert np.array_equal(counts, want)


def test_plane_wave_laplacian_eigenvalue(oracle_mod):
    N = 16
    p = oracle_mod.hilltop_params(N)
    o = oracle_mod.Oracle(p)
    i, j, k = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    px, py, pz = 1, 3, 2
    wave = np.cos(2 * np.pi * (px * i + py * j + pz * k) / N).ravel()
    o.f[:] = wave
    s = o.scalars
    s.a = 1.0
    o.set_scalars(s)
    grad = o.lib.ieo_gradient_energy(o.h)
    lam = 4 * sum(np.sin(np.pi * q / N) ** 2 for q in (px, py, pz))
    # gradient_energy = 0.5 * (-sum f lapl f) / (a dx)^2 / N^3 = 0.5 * lam <f^2> / dx^2
    want = 0.5 * lam * np.mean(wave ** 2) / p.dx ** 2
    assert np.isclose(grad, want, rtol=1e-12)


def test_homogeneous_background_matches_scalar_leapfrog(oracle_mod):
    # With no fluctuations the lattice leapfrog reduces to the background ODE.
    N = 8
    p = oracle_mod.hilltop_params(N)
    o = oracle_mod.Oracle(p)
    phi, dphi = 0.0935, 0.000796
    o.f[:] = phi
    o.fd[:] = dphi
    V = lambda v: p.V0 * (1.0 - (1.0 - p.ns) / 4.0 * v * v) / (p.rescale_B ** 2)
    dV = lambda v: -p.V0 * (1.0 - p.ns) / 2.0 * v / (p.rescale_B ** 2)
    s = o.scalars
    s.a, s.ad, s.astep = 1.0, np.sqrt((0.5 * dphi ** 2 + V(phi)) / 3.0), 1.0
    o.set_scalars(s)
    a, ad = s.a, s.ad
    for _ in range(50):
        d = p.dt / a
        ad2 = (-2 * ad - 2 * a / d / 1.0 * (1 - np.sqrt(1 + 2 * d * ad / a + d * d * a * a * (0.0 + V(phi))))) / d
        ad += 0.5 * d * ad2
        dphi += d * (0.0 - 2.0 * ad / a * dphi - a * a * dV(phi))
        ad += 0.5 * d * ad2
        phi += d * dphi
        a += d * ad
        o.leapfrog_steps(1)
    sc = o.scalars
    assert np.isclose(sc.a, a, rtol=1e-13)
    assert np.allclose(o.f, phi, rtol=1e-13)
    assert np.allclose(o.fd, dphi, rtol=1e-12)
