"""Parity of the CUDA engine with the oracle, operation by operation.

Bit-exact where the engine's per-site arithmetic is the reference's (FFT, the
deltaN integration, the float mean of saveN, histograms, bin counts), and for
whole leapfrog trajectories against the oracle in engine-arithmetic mode
(the Friedmann update's lattice sums formed exactly, as the engine forms
them).  Against the reference's serial sums, within stated tolerances:
  * fields after leapfrog steps: max|x_gpu - x_oracle| <= 1e-9 * std(x_oracle)
  * a, ad: relative 1e-12
  * spectrum bins: relative 1e-12 (same modes, different summation order)
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def oracle_state(ieo, N, usr, sigw, tables, steps=0):
    p = ieo.usr_params(N, calculate_SIGW=int(sigw)) if usr else ieo.hilltop_params(N, calculate_SIGW=int(sigw))
    o = ieo.Oracle(p, tables if usr else None)
    o.initialize_all()
    o.evolve_fields(0.5 * p.dt)
    if steps:
        o.leapfrog_steps(steps)
    return p, o


def lattice_like(iegpu, p, o, usr, sigw, tables):
    lat = iegpu.Lattice(p.N, p.L, p.dt, p.V0, p.ns, p.rescale_B,
                        potential=iegpu.POT_TABLE if usr else iegpu.POT_HILLTOP, sigw=sigw)
    if usr:
        lat.set_table(*tables)
    lat.upload(iegpu.F, o.f.copy())
    lat.upload(iegpu.FD, o.fd.copy())
    if sigw:
        for c in range(6):
            lat.upload(iegpu.H(c), o.h_(c).copy())
            lat.upload(iegpu.HD(c), o.hd_(c).copy())
    s = o.scalars
    return lat, iegpu.Bg(s.t, s.a, s.ad, s.ad2, s.astep)


def rel_field_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.std(b), 1e-300))


@pytest.mark.parametrize("N", [8, 16, 32, 64])
def test_fft_bit_exact(N, engine, oracle_mod):
    rng = np.random.default_rng(N)
    with engine.Lattice(N, 10.0, 1e-3, 3.338e-13, sigw=True) as lat:
        x = rng.standard_normal(N ** 3)
        ny = rng.standard_normal(2 * N * N)
        for fwd in (1, -1):
            lat.upload(engine.F, x, ny)
            lat.fft(engine.F, fwd)
            g, gny = lat.download(engine.F, nyquist=True)
            r, rny = x.copy(), ny.copy()
            oracle_mod.fftrn_d(r, rny, N, fwd)
            assert np.array_equal(g, r), f"double fft {fwd}"
            assert np.array_equal(gny, rny)
        xf = rng.standard_normal(N ** 3).astype(np.float32)
        nyf = rng.standard_normal(2 * N * N).astype(np.float32)
        for fwd in (1, -1):
            lat.upload(engine.H(2), xf, nyf)
            lat.fft(engine.H(2), fwd)
            g, gny = lat.download(engine.H(2), nyquist=True)
            r, rny = xf.copy(), nyf.copy()
            oracle_mod.fftrn_f(r, rny, N, fwd)
            assert np.array_equal(g, r), f"float fft {fwd}"
            assert np.array_equal(gny, rny)


@pytest.mark.parametrize("N,usr,sigw", [(16, False, False), (32, False, False), (16, True, False), (16, True, True),
                                        (32, True, True)])
def test_leapfrog_matches_oracle(N, usr, sigw, engine, oracle_mod, tables):
    p, o = oracle_state(oracle_mod, N, usr, sigw, tables)
    lat, bg = lattice_like(engine, p, o, usr, sigw, tables)
    with lat:
        nsteps = 300
        taken, trace = lat.leapfrog(p.af, nsteps, bg, trace=True)
        assert taken == nsteps
        o.leapfrog_steps(nsteps)
        s = o.scalars
        assert abs(bg.a - s.a) <= 1e-12 * s.a
        assert abs(bg.ad - s.ad) <= 1e-12 * abs(s.ad)
        assert abs(bg.t - s.t) <= 1e-12 * s.t
        assert trace[-1] == bg.a
        assert rel_field_err(lat.download(engine.F), o.f) < 1e-9
        assert rel_field_err(lat.download(engine.FD), o.fd) < 1e-9
        if sigw:
            for c in range(6):
                assert rel_field_err(lat.download(engine.H(c)), o.h_(c)) < 1e-5
                assert rel_field_err(lat.download(engine.HD(c)), o.hd_(c)) < 1e-5


@pytest.mark.parametrize("N,usr,sigw", [(16, False, False), (32, False, False), (64, False, False),
                                        (16, True, False), (32, True, False), (16, True, True)])
def test_leapfrog_bit_exact_with_engine_arithmetic(N, usr, sigw, engine, oracle_mod, tables):
    """300 leapfrog steps, engine against the oracle in engine-arithmetic mode:
    the fields, the tensor modes and every background scalar bit for bit.
    This checks each per-site operation (the stencil, V' with the exact
    division by B^2, the kick and drift) and the exact lattice sums over a
    whole trajectory."""
    p, o = oracle_state(oracle_mod, N, usr, sigw, tables)
    o.set_engine_arith(True)
    lat, bg = lattice_like(engine, p, o, usr, sigw, tables)
    with lat:
        nsteps = 300
        taken = lat.leapfrog(p.af, nsteps, bg)
        assert taken == nsteps
        o.leapfrog_steps(nsteps)
        s = o.scalars
        assert (bg.t, bg.a, bg.ad, bg.ad2) == (s.t, s.a, s.ad, s.ad2)
        assert np.array_equal(lat.download(engine.F), o.f)
        assert np.array_equal(lat.download(engine.FD), o.fd)
        if sigw:
            for c in range(6):
                assert np.array_equal(lat.download(engine.H(c)), o.h_(c))
                assert np.array_equal(lat.download(engine.HD(c)), o.hd_(c))


def test_leapfrog_stops_at_af(engine, oracle_mod):
    p, o = oracle_state(oracle_mod, 16, False, False, None)
    lat, bg = lattice_like(engine, p, o, False, False, None)
    with lat:
        af = bg.a * 1.01
        taken = lat.leapfrog(af, 100000, bg)
        assert bg.a > af
        p.af = af
        o2 = oracle_mod.Oracle(p)
        o2.initialize_all()
        o2.evolve_fields(0.5 * p.dt)
        assert o2.leapfrog_steps(100000) == taken


def test_single_step_entry_points(engine, oracle_mod):
    p, o = oracle_state(oracle_mod, 16, False, False, None, steps=10)
    lat, bg = lattice_like(engine, p, o, False, False, None)
    with lat:
        d = o.rescaled_step(o.scalars.astep)
        lat.evolve_derivs(d, bg)
        o.evolve_derivs(d)
        lat.evolve_fields(d, bg)
        o.evolve_fields(d)
        s = o.scalars
        assert abs(bg.ad - s.ad) <= 1e-13 * abs(s.ad)
        assert abs(bg.a - s.a) <= 1e-14 * s.a
        assert rel_field_err(lat.download(engine.F), o.f) < 1e-12


def test_energies_and_means(engine, oracle_mod, tables):
    """kin, gradient and potential energies.  The engine sums exactly, so it
    equals the oracle in engine-arithmetic mode bit for bit, and its sum of
    f lapl(f) is the correctly rounded sum of the exact products f lapl(f)
    (the products are not rounded before they are added).  The reference's
    serial sum of f lapl(f) cancels (the terms are of order |f| |lapl f|, the
    total of order |grad f|^2), so it keeps only about six digits of the
    gradient energy; that is the comparison with the reference mode below."""
    for usr in (False, True):
        p, o = oracle_state(oracle_mod, 16, usr, False, tables, steps=20)
        lat, bg = lattice_like(engine, p, o, usr, False, tables)
        with lat:
            k, g, v = lat.energies(bg)
            ko, go, vo = o.energies()
            assert np.isclose(k, ko, rtol=1e-12) and np.isclose(v, vo, rtol=1e-12)
            assert np.isclose(g, go, rtol=1e-6, atol=1e-12 * abs(vo))
            o.set_engine_arith(True)
            assert (k, g, v) == o.energies()
            o.set_engine_arith(False)
            N = p.N
            f = o.f.reshape(N, N, N)
            lap = (np.roll(f, -1, 2) + np.roll(f, 1, 2) + np.roll(f, -1, 1) + np.roll(f, 1, 1) + np.roll(f, -1, 0)
                   + np.roll(f, 1, 0) - 6.0 * f)
            G = oracle_mod.exact_dot(f.ravel(), lap.ravel())
            a, dx = bg.a, p.L / N
            assert g == 0.5 * (-G) * ((1.0 / (a * dx)) * (1.0 / (a * dx))) / N ** 3
            sf, sfd, sf2 = lat.means()
            assert np.isclose(sf, o.f.sum(), rtol=1e-13)
            assert np.isclose(sfd, o.fd.sum(), rtol=1e-12)
            assert np.isclose(sf2, (o.f ** 2).sum(), rtol=1e-13)


@pytest.mark.parametrize("N", [16, 32, 64])
def test_spectrum_matches_oracle(N, engine, oracle_mod):
    p, o = oracle_state(oracle_mod, N, False, False, None, steps=50)
    lat, bg = lattice_like(engine, p, o, False, False, None)
    with lat:
        counts, f2 = lat.spectrum(engine.F)
        oc, of2 = o.spectrum_f()
        assert np.array_equal(counts, oc)
        assert np.allclose(f2, of2, rtol=1e-12, atol=0)
        # the in-place FFT round trip leaves the same bits as the reference's
        assert np.array_equal(lat.download(engine.F), o.f)


def _bits(x):
    return np.ascontiguousarray(x).view(np.uint64)


@pytest.mark.parametrize("N", [16, 32, 64, 128])
def test_spectrum_forcing_cutoff_matches_oracle(N, engine, oracle_mod):
    """spectraf() with the forcing cutoff (src/output.cpp:330-401): counts
    exact, bin sums 1e-12, and f and fd after the call bit for bit (signs of
    zero included) with the oracle, for a high cutoff alone, one at N/2 (the
    on-axis Nyquist modes stay), and high with low (the low one zeroes the
    k = 0 mode as well)."""
    for hi, lo in ((0.3 * N, 0.0), (N / 2, 0.0), (0.4 * N, 2.5)):
        p, o = oracle_state(oracle_mod, N, False, False, None, steps=20)
        lat, bg = lattice_like(engine, p, o, False, False, None)
        with lat:
            counts, f2 = lat.spectrum_cutoff(hi, lo)
            oc, of2 = o.spectrum_f(hi, lo)
            assert np.array_equal(counts, oc)
            assert np.allclose(f2, of2, rtol=1e-12, atol=0)
            assert np.array_equal(_bits(lat.download(engine.F)), _bits(o.f)), (N, hi, lo, "f")
            assert np.array_equal(_bits(lat.download(engine.FD)), _bits(o.fd)), (N, hi, lo, "fd")


@pytest.mark.parametrize("N", [8, 16])
def test_spectrum_forcing_cutoff_matches_reference(N, engine):
    """The same against the reference's own spectraf() on seeded random f and
    fd (tests/golden/forcing_cutoff/, made by the reference program): f and fd
    after the call bit for bit, for every cutoff pair of the fixture."""
    g = np.load(GOLDEN / "forcing_cutoff" / f"cut_n{N}.npz")
    for q, (hi, lo) in enumerate(g["cuts"]):
        with engine.Lattice(N, 10.0, 1e-3, 3.338e-13) as lat:
            lat.upload(engine.F, g["f_in"].copy())
            lat.upload(engine.FD, g["fd_in"].copy())
            lat.spectrum_cutoff(float(hi), float(lo))
            assert np.array_equal(_bits(lat.download(engine.F)), _bits(g[f"f_{q}"])), (N, hi, lo, "f")
            assert np.array_equal(_bits(lat.download(engine.FD)), _bits(g[f"fd_{q}"])), (N, hi, lo, "fd")


def test_gw_spectrum_matches_oracle(engine, oracle_mod, tables):
    p, o = oracle_state(oracle_mod, 16, True, True, tables, steps=100)
    lat, bg = lattice_like(engine, p, o, True, True, tables)
    with lat:
        for which, tp in ((0, 1.0), (1, p.rescale_B / o.scalars.a)):
            counts, f2 = lat.gw_spectrum(which, tp)
            oc, of2, of2d = o.gw_spectrum(which, tp)
            assert np.array_equal(counts, oc)
            assert np.allclose(f2, of2d, rtol=1e-12, atol=0)
            # the tree-ordered double sums against the reference's float accumulators
            m = oc > 0
            assert np.allclose(f2[m], of2[m], rtol=1e-4)
            # the reference's float accumulators themselves, in its loop order: bit for bit,
            # and the same values summed in double (another order) to 1e-12
            # (both sides' fields have been through one FFT round trip here)
            rc, rf2, rf2d = lat.gw_spectrum_ref(which, tp)
            oc, of2, of2d = o.gw_spectrum(which, tp)
            assert np.array_equal(rc, oc)
            assert np.array_equal(rf2.view(np.uint32), np.asarray(of2, dtype=np.float32).view(np.uint32))
            assert np.allclose(rf2d, of2d, rtol=1e-12, atol=0)
        for c in range(6):
            assert np.array_equal(lat.download(engine.H(c)), o.h_(c))


@pytest.mark.parametrize("N", [16, 32, 64])
def test_gw_spectrum_reference_order_at_sizes(N, engine, oracle_mod, tables):
    """The reference-order GW accumulators at several lattice sizes (random h
    and h' uploaded to both): float sums bit for bit with the oracle's
    write_gw_spectrum_impl, double sums to 1e-12, counts exact."""
    rng = np.random.default_rng(N)
    p = oracle_mod.usr_params(N, calculate_SIGW=1)
    o = oracle_mod.Oracle(p, tables)
    with engine.Lattice(N, p.L, p.dt, p.V0, sigw=True) as lat:
        for c in range(6):
            h = rng.standard_normal(N ** 3).astype(np.float32) * 1e-3
            hd = rng.standard_normal(N ** 3).astype(np.float32) * 1e-3
            o.h_(c)[:] = h
            o.hd_(c)[:] = hd
            lat.upload(engine.H(c), h.copy())
            lat.upload(engine.HD(c), hd.copy())
        for which, tp in ((0, 1.0), (1, 0.37)):
            rc, rf2, rf2d = lat.gw_spectrum_ref(which, tp)
            oc, of2, of2d = o.gw_spectrum(which, tp)
            assert np.array_equal(rc, oc)
            assert np.array_equal(rf2.view(np.uint32), np.asarray(of2, dtype=np.float32).view(np.uint32)), (N, which)
            assert np.allclose(rf2d, of2d, rtol=1e-12, atol=0), (N, which)


@pytest.mark.parametrize("usr", [False, True])
def test_deltaN_bit_exact(usr, engine, oracle_mod, tables):
    p, o = oracle_state(oracle_mod, 16, usr, False, tables, steps=30)
    lat, bg = lattice_like(engine, p, o, usr, False, tables)
    with lat:
        lat.initializeN(o.scalars.a)
        o.initializeN()
        assert np.array_equal(lat.download(engine.FD), o.fd)
        lat.evolve_fieldsN(0.5 * p.dN, 0.0 if usr else 0.0)
        s = o.scalars
        s.phiref = 0.0
        o.set_scalars(s)
        o.evolve_fieldsN(0.5 * p.dN)
        phiref = lat.get_phiref()
        assert phiref == o.get_phiref()
        s = o.scalars
        s.phiref = phiref
        o.set_scalars(s)
        lat.deltaN_steps(p.dN, 400, phiref)
        o.deltaN_steps(400)
        for fld, ref in ((engine.F, o.f), (engine.FD, o.fd), (engine.DELTAN, o.deltaN)):
            assert np.array_equal(lat.download(fld), ref)


def test_saveN_mean_histogram_and_zeroing(engine, oracle_mod):
    N = 16
    rng = np.random.default_rng(5)
    dn = 1e-3 + 1e-6 * rng.standard_normal(N ** 3)
    dn[::7] = 2e-3
    p = oracle_mod.hilltop_params(N)
    o = oracle_mod.Oracle(p)
    o.deltaN[:] = dn
    with engine.Lattice(N, p.L, p.dt, p.V0) as lat:
        lat.upload(engine.DELTAN, dn)
        cutoff = 1.5e-3
        m = lat.saveN_mean(cutoff)
        assert np.float32(m) == np.float32(o.saveN_mean(cutoff))
        lat.shift(engine.DELTAN, float(m))
        x = dn - np.float64(np.float32(m))
        assert np.array_equal(lat.download(engine.DELTAN), x)
        bmin, df, freq = lat.histogram(engine.DELTAN, 256)
        assert bmin == x.min() and df == (x.max() - x.min()) / 256
        b = ((x - bmin) / df).astype(int)
        b[x == x.max()] = 255
        want = np.bincount(b[(b >= 0) & (b < 256)], minlength=256) / N ** 3
        assert np.array_equal(freq, want)
        lat.zero_above(engine.DELTAN, cutoff - m)
        x[x > cutoff - np.float64(np.float32(m))] = 0
        assert np.array_equal(lat.download(engine.DELTAN), x)
        assert np.isclose(lat.sum(engine.DELTAN), x.sum(), rtol=1e-14)


def test_table_range_error_is_reported(engine, oracle_mod, tables):
    p, o = oracle_state(oracle_mod, 8, True, False, tables)
    lat, bg = lattice_like(engine, p, o, True, False, tables)
    with lat:
        f = o.f.copy()
        f[17] = 3.6  # above the top node 3.5
        lat.upload(engine.F, f)
        with pytest.raises(engine.IegpuError) as e:
            lat.leapfrog(p.af, 4, bg)
        assert e.value.code == engine.ERANGE
        assert "outside the numerical potential range" in str(e.value)


@pytest.mark.parametrize("N,usr", [(16, False), (32, True), (64, False)])
def test_device_initial_conditions(N, usr, engine, oracle_mod, tables):
    p = oracle_mod.usr_params(N) if usr else oracle_mod.hilltop_params(N)
    o = oracle_mod.Oracle(p, tables if usr else None)
    o.initialize_all()
    with engine.Lattice(N, p.L, p.dt, p.V0, p.ns, p.rescale_B,
                        potential=engine.POT_TABLE if usr else engine.POT_HILLTOP) as lat:
        if usr:
            lat.set_table(*tables)
        H = lat.bunch_davies(p.seed, p.initial_field, p.initial_derivative)
        # same uniforms, same dispersion; only log/sin/cos come from another
        # maths library, so the fluctuations agree to a few ulps of themselves
        for fld, ref, base in ((engine.F, o.f, p.initial_field), (engine.FD, o.fd, p.initial_derivative)):
            got = lat.download(fld)
            # a fluctuation that differs in its last bits can round the sum
            # background + fluctuation to the neighbouring double
            tol = 1e-12 * np.std(ref) + 2 * np.spacing(abs(base))
            assert np.max(np.abs(got - ref)) <= tol
        assert abs(H - o.scalars.hubble_init) <= 1e-13 * H


@pytest.mark.parametrize("hi,lo", [(5.5, 0.0), (6.0, 2.5)])
def test_device_initial_conditions_with_mode_cutoffs(hi, lo, engine, oracle_mod):
    """set_mode's cutoff (src/initialize.cpp:70): modes with |p| outside
    [low_cutoff_index, high_cutoff_index] get no amplitude; the device draw
    against the oracle's at 32^3, high cutoff alone and with a low one."""
    N = 32
    p = oracle_mod.hilltop_params(N, high_cutoff_index=hi, low_cutoff_index=lo)
    o = oracle_mod.Oracle(p)
    o.initialize_all()
    with engine.Lattice(N, p.L, p.dt, p.V0, p.ns, p.rescale_B) as lat:
        H = lat.bunch_davies(p.seed, p.initial_field, p.initial_derivative, hi, lo)
        for fld, ref, base in ((engine.F, o.f, p.initial_field), (engine.FD, o.fd, p.initial_derivative)):
            got = lat.download(fld)
            tol = 1e-12 * np.std(ref) + 2 * np.spacing(abs(base))
            assert np.max(np.abs(got - ref)) <= tol
        assert abs(H - o.scalars.hubble_init) <= 1e-13 * H
    # the cutoff removed power: the spectrum past the high cutoff is empty
    f = o.f.reshape(N, N, N) - o.f.mean()
    X = np.fft.rfftn(f)
    px = np.fft.fftfreq(N, 1.0 / N)
    pz = np.fft.rfftfreq(N, 1.0 / N)
    k = np.sqrt(px[:, None, None] ** 2 + px[None, :, None] ** 2 + pz[None, None, :] ** 2)
    assert np.max(np.abs(X[k > hi + 1])) <= 1e-9 * np.max(np.abs(X))


def test_device_initial_conditions_seed_semantics(engine, oracle_mod):
    N = 8
    for seed in (0, 1, 12345):
        p = oracle_mod.hilltop_params(N, seed=seed)
        o = oracle_mod.Oracle(p)
        o.initialize_all()
        with engine.Lattice(N, p.L, p.dt, p.V0, p.ns, p.rescale_B) as lat:
            lat.bunch_davies(seed, p.initial_field, p.initial_derivative)
            got = lat.download(engine.F)
            assert np.max(np.abs(got - o.f)) <= 1e-12 * max(np.std(o.f), 1e-300) + 1e-15 * abs(p.initial_field)
