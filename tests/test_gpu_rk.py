"""The Runge-Kutta integrators against the oracle: RK4 and RK45
(Dormand-Prince 5(4) with the reference's step control) for the inflation
loop and the post-inflation loop on the plain FP64 form, and for the
per-site deltaN loop.

Every per-site expression of the stages, the weighted update and the RK45
candidate is the reference's.  The inflation equations combine two lattice
sums per stage, and the RK45 error norm one lattice sum per attempt, in a
different order from the reference, so the tolerances are those of the
leapfrog parity:
  * fields: max|x_gpu - x_oracle| <= 1e-9 * std(x_oracle); h, h': 1e-5
  * t, a, ad: relative 1e-12; the RK45 step carried between steps 1e-10
The post-inflation and deltaN equations have no lattice sums, so RK4 there is
compared bit for bit; deltaN RK45 differs only in the summation order of its
error norm.

With a step large enough for the RK45 controller to act (dt = 0.05 below),
the embedded error estimate is a near-cancelling combination of the stage
derivatives, so the rounding of the re-associated sums reaches the proposed
step at ~1e-10 relative and the trajectory follows.  The reference itself
shows more than that between its own runs on 1 and 8 OpenMP threads (16^3
hilltop, dt = 0.05, to a = 32: a differs by 5.5e-10 relative, f by 58626 ulp).
Those cases use tolerances above that spread: scalars and the step 5e-9
relative, fields 1e-9 of their largest magnitude.
"""
from __future__ import annotations

import numpy as np
import pytest

from test_gpu_parity import lattice_like, rel_field_err

pytestmark = pytest.mark.gpu


def _oracle(ieo, N, usr, sigw, tables):
    kw = dict(calculate_SIGW=int(sigw), inflation_integrator=1)
    p = ieo.usr_params(N, **kw) if usr else ieo.hilltop_params(N, **kw)
    o = ieo.Oracle(p, tables if usr else None)
    o.initialize_all()   # no half drift: the RK4 state is synchronous
    return p, o


def _oracle_loop(o, af, n):
    """The RK4 branch of run_evolution_loop (src/evolution.cpp:948-956)."""
    taken = 0
    while taken < n and o.scalars.a <= af:
        o.rk4_step_inflation(o.rescaled_step(o.scalars.astep))
        s = o.scalars
        s.astep = s.a
        o.set_scalars(s)
        taken += 1
    return taken


def _close(engine, o, lat, bg, sigw, what, controlled=False):
    s = o.scalars
    rs = 5e-9 if controlled else 1e-12
    assert abs(bg.a - s.a) <= rs * s.a, (what, bg.a, s.a)
    assert abs(bg.ad - s.ad) <= rs * abs(s.ad), (what, bg.ad, s.ad)
    assert abs(bg.t - s.t) <= rs * s.t, what
    assert bg.ad2 == s.ad2, what
    for field, ref in ((engine.F, o.f), (engine.FD, o.fd)):
        got = lat.download(field)
        if controlled:
            assert np.max(np.abs(got - ref)) <= 1e-9 * np.max(np.abs(ref)), what
        else:
            assert rel_field_err(got, ref) < 1e-9, what
    if sigw:
        for c in range(6):
            assert rel_field_err(lat.download(engine.H(c)), o.h_(c)) < 1e-5, (what, c)
            assert rel_field_err(lat.download(engine.HD(c)), o.hd_(c)) < 1e-5, (what, c)


@pytest.mark.parametrize("N,usr,sigw", [(16, False, False), (32, False, False), (16, True, False), (16, True, True),
                                        (32, True, True)])
def test_rk4_matches_oracle(N, usr, sigw, engine, oracle_mod, tables):
    p, o = _oracle(oracle_mod, N, usr, sigw, tables)
    lat, bg = lattice_like(engine, p, o, usr, sigw, tables)
    with lat:
        total = 0
        for n in (1, 99, 200):
            taken, trace = lat.rk4(p.af, n, bg, trace=True)
            assert taken == n and trace[-1] == bg.a
            bg.astep = bg.a   # the caller's "astep = a" after its report
            assert _oracle_loop(o, p.af, n) == n
            total += n
            _close(engine, o, lat, bg, sigw, f"after {total} steps")


def test_rk4_single_step_and_stop_at_af(engine, oracle_mod):
    p, o = _oracle(oracle_mod, 16, False, False, None)
    lat, bg = lattice_like(engine, p, o, False, False, None)
    with lat:
        h = 0.75 * p.dt
        lat.rk4_step_inflation(h, bg)
        o.rk4_step_inflation(h)
        s = o.scalars
        assert bg.astep == s.astep
        assert abs(bg.a - s.a) <= 1e-14 * s.a
        assert abs(bg.ad - s.ad) <= 1e-13 * abs(s.ad)
        assert rel_field_err(lat.download(engine.F), o.f) < 1e-12
        assert rel_field_err(lat.download(engine.FD), o.fd) < 1e-12
        af = bg.a * 1.01
        taken = lat.rk4(af, 100000, bg)
        assert bg.a > af and bg.astep == bg.a
        assert _oracle_loop(o, af, 100000) == taken
        assert abs(bg.a - o.scalars.a) <= 1e-12 * bg.a


def test_rk4_table_range_error_is_reported(engine, oracle_mod, tables):
    p, o = _oracle(oracle_mod, 8, True, False, tables)
    lat, bg = lattice_like(engine, p, o, True, False, tables)
    with lat:
        f = o.f.copy()
        f[17] = 3.6  # above the top node 3.5
        lat.upload(engine.F, f)
        with pytest.raises(engine.IegpuError) as e:
            lat.rk4(p.af, 4, bg)
        assert e.value.code == engine.ERANGE
        assert "outside the numerical potential range" in str(e.value)


def test_rk4_needs_the_fp64_form(engine):
    bg = engine.Bg(0.0, 1.0, 1.0, 0.0, 1.0)
    with engine.Lattice(128, 10.0, 1e-3, 3.338e-13, form=engine.FORM_SPLIT) as lat:
        with pytest.raises(engine.IegpuError) as e:
            lat.rk4(2.0, 1, bg)
        assert e.value.code == engine.EUNSUPPORTED


def _oracle_rk45(o, af, n, h):
    """The RK45 branch of run_evolution_loop (src/evolution.cpp:958-985)."""
    taken = 0
    while taken < n and o.scalars.a <= af:
        hmax = o.rk45_hmax(o.rescaled_step(o.scalars.astep))
        h = o.rk45_accept(o.rk45_clamp(h, hmax), hmax)
        s = o.scalars
        s.astep = s.a
        o.set_scalars(s)
        taken += 1
    return taken, h


def _controls(engine, p):
    return engine.Rk45Controls(p.rk45_abs_tol, p.rk45_rel_tol, p.rk45_min_dt, p.rk45_max_dt, p.rk45_safety)


# (N, USR, SIGW, extra parameters): the reference's defaults, and a step large
# enough for the step control to act (h from 6e-4 to 0.04, rejections)
RK45_CASES = [
    (16, False, False, {}),
    (16, True, True, {}),
    (16, False, False, dict(dt=0.05, rk45_abs_tol=1e-12, rk45_rel_tol=1e-10)),
    (32, False, False, dict(dt=0.05, rk45_abs_tol=1e-12, rk45_rel_tol=1e-10)),
]


@pytest.mark.parametrize("N,usr,sigw,extra", RK45_CASES)
def test_rk45_matches_oracle(N, usr, sigw, extra, engine, oracle_mod, tables):
    kw = dict(calculate_SIGW=int(sigw), inflation_integrator=2, **extra)
    p = oracle_mod.usr_params(N, **kw) if usr else oracle_mod.hilltop_params(N, **kw)
    o = oracle_mod.Oracle(p, tables if usr else None)
    o.initialize_all()
    lat, bg = lattice_like(engine, p, o, usr, sigw, tables)
    ctl = _controls(engine, p)
    h0 = o.rescaled_step(o.scalars.astep)
    hg = ho = h0
    controlled = "dt" in extra
    rh = 5e-9 if controlled else 1e-10
    with lat:
        total = 0
        for n in (1, 59, 140):
            taken, hg = lat.rk45(p.af, n, bg, hg, ctl)
            bg.astep = bg.a
            t_o, ho = _oracle_rk45(o, p.af, n, ho)
            assert taken == t_o, (taken, t_o)
            total += taken
            assert abs(hg - ho) <= rh * ho, (hg, ho)
            _close(engine, o, lat, bg, sigw, f"after {total} steps", controlled)
            if taken < n:
                break


def test_rk45_attempts_accept_and_reject(engine, oracle_mod):
    p = oracle_mod.hilltop_params(16, inflation_integrator=2, dt=0.05, rk45_abs_tol=1e-12, rk45_rel_tol=1e-10)
    o = oracle_mod.Oracle(p)
    o.initialize_all()
    lat, bg = lattice_like(engine, p, o, False, False, None)
    ctl = _controls(engine, p)
    with lat:
        f0 = lat.download(engine.F)
        # too large a step for the tolerances: rejected, the state is kept
        acc, hn = lat.rk45_step_inflation(0.1, 0.1, bg, ctl)
        acc_o, hn_o = o.rk45_step_inflation(0.1, 0.1)
        assert not acc and not acc_o
        assert abs(hn - hn_o) <= 5e-9 * hn_o
        assert np.array_equal(lat.download(engine.F), f0) and bg.a == o.scalars.a == 1.0
        # the proposed step is accepted
        acc, hn2 = lat.rk45_step_inflation(hn, 0.1, bg, ctl)
        acc_o, hn2_o = o.rk45_step_inflation(hn_o, 0.1)
        assert acc and acc_o
        assert abs(hn2 - hn2_o) <= 5e-9 * hn2_o
        _close(engine, o, lat, bg, False, "after one accepted attempt", controlled=True)


def test_rk45_failure_to_converge_is_reported(engine, oracle_mod):
    p = oracle_mod.hilltop_params(16, inflation_integrator=2)
    o = oracle_mod.Oracle(p)
    o.initialize_all()
    lat, bg = lattice_like(engine, p, o, False, False, None)
    # tolerances no step can meet, and no room below dt: the first rejection
    # lands on the minimum step
    ctl = engine.Rk45Controls(1e-300, 1e-300, p.dt, p.dt, 0.9)
    with lat:
        with pytest.raises(engine.IegpuError) as e:
            lat.rk45(p.af, 10, bg, p.dt, ctl)
        assert e.value.code == engine.ECONVERGE
        assert "RK45 failed to converge at a=" in str(e.value)


def _post_setup(ieo, engine, N, usr, integrator, tables):
    kw = dict(calculate_SIGW=1, perform_deltaN=1, post_inflation=1, post_inflation_integrator=integrator)
    p = ieo.usr_params(N, **kw) if usr else ieo.hilltop_params(N, **kw)
    o = ieo.Oracle(p, tables if usr else None)
    o.initialize_all()
    o.evolve_fields(0.5 * p.dt)
    o.leapfrog_steps(40)
    rng = np.random.default_rng(N + 11)
    o.deltaN[:] = 1e-3 * rng.standard_normal(N ** 3)
    lat, bg = lattice_like(engine, p, o, usr, True, tables)
    lat.upload(engine.DELTAN, o.deltaN.copy())
    o.initialize_post_inflation()
    lat.initialize_post_inflation(bg, p.horizon_factor, p.omega, True)
    o.set_rk_post(True)
    return p, o, lat, bg


@pytest.mark.parametrize("N,usr", [(16, True), (32, False)])
def test_post_inflation_rk4_bit_exact(N, usr, engine, oracle_mod, tables):
    p, o, lat, bg = _post_setup(oracle_mod, engine, N, usr, 1, tables)
    with lat:
        dt, af = p.dt_post_inflation, p.af_post_inflation
        for n in (1, 60):
            taken = 0
            while taken < n and o.scalars.a <= af:
                o.rk4_step_inflation(dt)
                taken += 1
            assert lat.post_inflation_rk4(af, dt, n, bg, omega=p.omega) == taken
            assert np.array_equal(lat.download(engine.F), o.f)
            assert np.array_equal(lat.download(engine.FD), o.fd)
            for c in range(6):
                assert np.array_equal(lat.download(engine.H(c)), o.h_(c)), c
                assert np.array_equal(lat.download(engine.HD(c)), o.hd_(c)), c
            s = o.scalars
            assert (bg.t, bg.a, bg.ad, bg.ad2) == (s.t, s.a, s.ad, s.ad2)


def test_post_inflation_rk45_matches_oracle(engine, oracle_mod, tables):
    p, o, lat, bg = _post_setup(oracle_mod, engine, 16, True, 2, tables)
    ctl = _controls(engine, p)
    with lat:
        dt, af = p.dt_post_inflation, p.af_post_inflation
        hg = ho = dt
        for n in (1, 60):
            taken = 0
            while taken < n and o.scalars.a <= af:
                hmax = o.rk45_hmax(dt)
                ho = o.rk45_accept(o.rk45_clamp(ho, hmax), hmax)
                taken += 1
            steps, hg = lat.post_inflation_rk45(af, dt, n, bg, hg, omega=p.omega, controls=ctl)
            assert steps == taken
            assert abs(hg - ho) <= 1e-10 * ho
            s = o.scalars
            assert abs(bg.a - s.a) <= 1e-12 * s.a and abs(bg.ad - s.ad) <= 1e-12 * abs(s.ad)
            assert rel_field_err(lat.download(engine.F), o.f) < 1e-9
            assert rel_field_err(lat.download(engine.FD), o.fd) < 1e-9
            for c in range(6):
                assert rel_field_err(lat.download(engine.H(c)), o.h_(c)) < 1e-5
                assert rel_field_err(lat.download(engine.HD(c)), o.hd_(c)) < 1e-5


def test_post_inflation_rk_needs_sigw(engine):
    bg = engine.Bg(0.0, 1.0, 1.0, 0.0, 1.0)
    with engine.Lattice(16, 10.0, 1e-3, 3.338e-13, sigw=False) as lat:
        with pytest.raises(engine.IegpuError):
            lat.post_inflation_rk4(2.0, 1e-3, 1, bg)


def _deltaN_setup(ieo, engine, usr, tables, median_phiref):
    from test_gpu_parity import oracle_state
    p, o2 = oracle_state(ieo, 16, usr, False, tables, steps=30)
    lat, bg = lattice_like(engine, p, o2, usr, False, tables)
    lat.initializeN(o2.scalars.a)
    o2.initializeN()
    phiref = float(np.median(o2.f)) if median_phiref else lat.get_phiref()
    s = o2.scalars
    s.phiref = phiref
    s.Ne = 0.0
    o2.set_scalars(s)
    return p, o2, lat, bg, phiref


# (USR, end surface at the median field value: sites go inactive during the run)
DN_CASES = [(False, False), (True, False), (True, True)]


@pytest.mark.parametrize("usr,median", DN_CASES)
def test_deltaN_rk4_bit_exact(usr, median, engine, oracle_mod, tables):
    """The deltaN stages have no lattice sums: RK4 matches bit for bit."""
    p, o, lat, bg, phiref = _deltaN_setup(oracle_mod, engine, usr, tables, median)
    with lat:
        for n in (1, 399):
            lat.deltaN_rk4_steps(p.dN, n, phiref, bg)
            for _ in range(n):
                o.rk4_step_deltaN(p.dN)
            for fld, ref in ((engine.F, o.f), (engine.FD, o.fd), (engine.DELTAN, o.deltaN)):
                assert np.array_equal(lat.download(fld), ref)
            s = o.scalars
            assert (bg.t, bg.a) == (s.t, s.a)
        if median:
            dn = lat.download(engine.DELTAN)
            assert 0 < np.count_nonzero(dn < dn.max()) < dn.size   # some sites stopped


@pytest.mark.parametrize("usr,median", DN_CASES)
def test_deltaN_rk45_matches_oracle(usr, median, engine, oracle_mod, tables):
    """Per-site stages are bit-exact; only the error norm's summation order
    differs, so the step control agrees to rounding."""
    p, o, lat, bg, phiref = _deltaN_setup(oracle_mod, engine, usr, tables, median)
    ctl = _controls(engine, p)
    with lat:
        hg = ho = p.dN
        Ne = 0.0
        for n in (1, 200):
            steps, hg, Ne = lat.deltaN_rk45(p.dN, p.Nend, n, phiref, hg, Ne, bg, ctl)
            taken = 0
            while taken < n and o.scalars.Ne <= p.Nend:
                hmax = o.rk45_hmax(p.dN)
                ho = o.rk45_accept_deltaN(o.rk45_clamp(ho, hmax), hmax)
                s = o.scalars
                s.Ne += ho
                o.set_scalars(s)
                taken += 1
            assert steps == taken
            s = o.scalars
            assert abs(hg - ho) <= 1e-12 * ho and abs(Ne - s.Ne) <= 1e-12 * s.Ne
            assert abs(bg.a - s.a) <= 1e-12 * s.a and abs(bg.t - s.t) <= 1e-12 * s.t
            for fld, ref in ((engine.F, o.f), (engine.FD, o.fd), (engine.DELTAN, o.deltaN)):
                got = lat.download(fld)
                assert np.max(np.abs(got - ref)) <= 1e-10 * np.max(np.abs(ref)), fld
