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


def _hilltop_V(p):
    B2 = p.rescale_B ** 2
    V = lambda v: p.V0 * (1.0 - (1.0 - p.ns) / 4.0 * v * v) / B2
    dV = lambda v: -p.V0 * (1.0 - p.ns) / 2.0 * v / B2
    return V, dV


def test_rk4_inflation_background_is_fourth_order(oracle_mod):
    """With no fluctuations, rk4_step_inflation integrates the homogeneous
    system f'' = -(2 a'/a) f' - a^2 V'(f), a'' = a^3 V(f) - a'^2/a (s = 0).
    Against a tight independent solution its error falls by ~2^4 when the
    step halves."""
    solve_ivp = pytest.importorskip("scipy.integrate").solve_ivp
    N = 8
    p = oracle_mod.hilltop_params(N, inflation_integrator=1)
    V, dV = _hilltop_V(p)
    phi0, dphi0 = 0.0935, 0.000796
    ad0 = np.sqrt((0.5 * dphi0 ** 2 + V(phi0)) / 3.0)
    T = 1.0   # conformal time (s = 0): a ~ 1/(1 - H t) blows up near t = 1.7

    def rhs(_, y):
        f, fd, a, ad = y
        return [fd, -(2.0 * ad / a) * fd - a * a * dV(f), ad, a ** 3 * V(f) - ad * ad / a]

    exact = solve_ivp(rhs, (0.0, T), [phi0, dphi0, 1.0, ad0], method="DOP853", rtol=1e-13, atol=1e-15).y[:, -1]
    errs = []
    for h in (0.1, 0.05, 0.025):
        o = oracle_mod.Oracle(p)
        o.f[:] = phi0
        o.fd[:] = dphi0
        s = o.scalars
        s.t, s.a, s.ad = 0.0, 1.0, ad0
        o.set_scalars(s)
        for _ in range(int(round(T / h))):
            o.rk4_step_inflation(h)
        got = np.array([o.f[0], o.fd[0], o.scalars.a, o.scalars.ad])
        assert np.all(o.f == o.f[0]) and np.all(o.fd == o.fd[0])
        errs.append(np.max(np.abs(got - exact) / np.abs(exact)))
    r1, r2 = errs[0] / errs[1], errs[1] / errs[2]
    assert 12.0 < r1 < 20.0 and 12.0 < r2 < 20.0, errs


def test_rk45_inflation_background_meets_its_tolerance(oracle_mod):
    """rk45 on the same homogeneous system: accepted steps stay within a small
    multiple of the requested relative tolerance of the tight solution."""
    solve_ivp = pytest.importorskip("scipy.integrate").solve_ivp
    p = oracle_mod.hilltop_params(8, inflation_integrator=2, rk45_rel_tol=1e-9, rk45_abs_tol=1e-12,
                                  rk45_max_dt=0.5)
    V, dV = _hilltop_V(p)
    phi0, dphi0 = 0.0935, 0.000796
    ad0 = np.sqrt((0.5 * dphi0 ** 2 + V(phi0)) / 3.0)

    def rhs(_, y):
        f, fd, a, ad = y
        return [fd, -(2.0 * ad / a) * fd - a * a * dV(f), ad, a ** 3 * V(f) - ad * ad / a]

    o = oracle_mod.Oracle(p)
    o.f[:] = phi0
    o.fd[:] = dphi0
    s = o.scalars
    s.t, s.a, s.ad = 0.0, 1.0, ad0
    o.set_scalars(s)
    h, hmax = 0.1, 0.5
    for _ in range(40):
        h = o.rk45_accept(o.rk45_clamp(h, hmax), hmax)
    T = o.scalars.t
    exact = solve_ivp(rhs, (0.0, T), [phi0, dphi0, 1.0, ad0], method="DOP853", rtol=1e-13, atol=1e-15).y[:, -1]
    got = np.array([o.f[0], o.fd[0], o.scalars.a, o.scalars.ad])
    assert np.max(np.abs(got - exact) / np.abs(exact)) < 1e-7


def test_rk4_deltaN_site_matches_an_independent_solution(oracle_mod):
    """One deltaN site in e-fold time, f' = fd, fd' = -(3 - fd^2/2)(fd + V'/V),
    while active: rk4_step_deltaN on a homogeneous lattice against a tight
    solution, fourth order, and deltaN = N_e for a site that never stops."""
    solve_ivp = pytest.importorskip("scipy.integrate").solve_ivp
    p = oracle_mod.hilltop_params(8)          # antimonotonic: active while |f| < |phiref|
    V, dV = _hilltop_V(p)
    f0, fd0, Ntot = 0.0935, 0.02, 0.8

    def rhs(_, y):
        f, fd = y
        return [fd, -(3.0 - 0.5 * fd * fd) * (fd + dV(f) / V(f))]

    exact = solve_ivp(rhs, (0.0, Ntot), [f0, fd0], method="DOP853", rtol=1e-13, atol=1e-16).y[:, -1]
    errs = []
    for h in (0.1, 0.05, 0.025):
        o = oracle_mod.Oracle(p)
        o.f[:] = f0
        o.fd[:] = fd0
        o.deltaN[:] = 0.0
        s = o.scalars
        s.phiref = 10.0
        o.set_scalars(s)
        n = int(round(Ntot / h))
        for _ in range(n):
            o.rk4_step_deltaN(h)
        errs.append(max(abs(o.f[0] - exact[0]) / abs(exact[0]), abs(o.fd[0] - exact[1]) / abs(exact[1])))
        assert np.allclose(o.deltaN, n * h, rtol=1e-13)
    r1, r2 = errs[0] / errs[1], errs[1] / errs[2]
    assert 12.0 < r1 < 20.0 and 12.0 < r2 < 20.0, errs


def test_post_inflation_rk_radiation_background_is_linear(oracle_mod):
    """Radiation era (omega = 1/3, s = 0): a'' = 0, so with a homogeneous
    lattice a(t) = 1 + a'_0 t and a' stays exact under RK4 and RK45."""
    for integ in (1, 2):
        p = oracle_mod.hilltop_params(8, calculate_SIGW=1, post_inflation=1, post_inflation_integrator=integ)
        o = oracle_mod.Oracle(p)
        o.f[:] = 0.01
        o.fd[:] = 0.0
        s = o.scalars
        s.t, s.a, s.ad = 0.0, 1.0, 5.0
        o.set_scalars(s)
        o.set_rk_post(True)
        h = 1e-3
        for _ in range(100):
            if integ == 1:
                o.rk4_step_inflation(h)
            else:
                h = o.rk45_accept(o.rk45_clamp(h, 2e-3), 2e-3)
        sc = o.scalars
        assert sc.ad == 5.0
        assert abs(sc.a - (1.0 + 5.0 * sc.t)) <= 1e-13 * sc.a
        # the 7-point Laplacian of a constant is a rounding residue, not 0
        assert np.allclose(o.f, 0.01, rtol=1e-15) and np.max(np.abs(o.fd)) < 1e-15
