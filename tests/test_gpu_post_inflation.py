"""The post-inflation phase on the plain FP64 form (SIGW on) against the
oracle, bit for bit.

The phase has no lattice sums (a'' depends on a and a' only) and the engine
forms its scalars on the host with the reference's expressions, so whole
trajectories are compared exactly: after initialize_post_inflation (from a
deltaN map, or from f and fd without deltaN) and after runs of leapfrog
steps, the fields f, fd, the six h and h', and t, a, ad, ad2.  The runs end
mid-way and on af_post, so the loop condition is covered as well.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(ieo, engine, N, usr, from_deltaN, tables):
    kw = dict(calculate_SIGW=1, perform_deltaN=int(from_deltaN), post_inflation=1)
    p = ieo.usr_params(N, **kw) if usr else ieo.hilltop_params(N, **kw)
    o = ieo.Oracle(p, tables if usr else None)
    o.initialize_all()
    o.evolve_fields(0.5 * p.dt)
    o.leapfrog_steps(40)   # a state with structure in f, fd, h and h'
    rng = np.random.default_rng(N + 7 * int(usr))
    if from_deltaN:
        o.deltaN[:] = 1e-3 * rng.standard_normal(N ** 3)
    lat = engine.Lattice(N, p.L, p.dt, p.V0, p.ns, p.rescale_B,
                         potential=engine.POT_TABLE if usr else engine.POT_HILLTOP, sigw=True)
    if usr:
        lat.set_table(*tables)
    lat.upload(engine.F, o.f.copy())
    lat.upload(engine.FD, o.fd.copy())
    lat.upload(engine.DELTAN, o.deltaN.copy())
    for c in range(6):
        lat.upload(engine.H(c), o.h_(c).copy())
        lat.upload(engine.HD(c), o.hd_(c).copy())
    s = o.scalars
    return p, o, lat, engine.Bg(s.t, s.a, s.ad, s.ad2, s.astep)


def _same(engine, o, lat, bg, what):
    assert np.array_equal(lat.download(engine.F), o.f), f"{what}: f"
    assert np.array_equal(lat.download(engine.FD), o.fd), f"{what}: fd"
    for c in range(6):
        assert np.array_equal(lat.download(engine.H(c)), o.h_(c)), f"{what}: h{c}"
        assert np.array_equal(lat.download(engine.HD(c)), o.hd_(c)), f"{what}: hd{c}"
    s = o.scalars
    assert (bg.t, bg.a, bg.ad, bg.ad2, bg.astep) == (s.t, s.a, s.ad, s.ad2, s.astep), what


@pytest.mark.parametrize("N,usr,from_deltaN", [(16, True, True), (32, False, True), (16, False, False)])
def test_post_inflation_matches_oracle(N, usr, from_deltaN, engine, oracle_mod, tables):
    p, o, lat, bg = _setup(oracle_mod, engine, N, usr, from_deltaN, tables)
    with lat:
        o.initialize_post_inflation()
        lat.initialize_post_inflation(bg, p.horizon_factor, p.omega, from_deltaN)
        _same(engine, o, lat, bg, "initialize_post_inflation")
        dt, af = p.dt_post_inflation, p.af_post_inflation
        o.evolve_fields(0.5 * dt)
        lat.evolve_fields(0.5 * dt, bg)
        total = 0
        for n in (1, 37, 200, 10 ** 6):
            taken = 0
            while taken < n and o.scalars.a <= af:
                o.evolve_derivs_post_inflation(dt)
                o.evolve_fields(dt)
                taken += 1
            assert lat.post_inflation_leapfrog(af, dt, n, bg, omega=p.omega) == taken
            total += taken
            _same(engine, o, lat, bg, f"after {total} steps")
        assert bg.a > af and total > 238


def test_post_inflation_needs_the_fp64_form_with_sigw(engine):
    bg = engine.Bg(0.0, 1.0, 1.0, 0.0, 1.0)
    with engine.Lattice(16, 10.0, 1e-3, 3.338e-13, sigw=False) as lat:
        with pytest.raises(engine.IegpuError):
            lat.initialize_post_inflation(bg)
    with engine.Lattice(16, 10.0, 1e-3, 3.338e-13, sigw=True, form=engine.FORM_SPLIT) as lat:
        with pytest.raises(engine.IegpuError):
            lat.post_inflation_leapfrog(32.0, 1e-3, 1, bg)
