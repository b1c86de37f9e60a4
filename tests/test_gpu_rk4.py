"""The RK4 inflation integrator (inflation_integrator = rk4) on the plain FP64
form against the oracle's rk4_step_inflation.

Every per-site expression of the stages and of the weighted update is the
reference's; the two lattice sums of each right-hand side (sum f lapl f and
sum V(f)) are combined in a different order, so the tolerances are those of
the leapfrog parity:
  * fields: max|x_gpu - x_oracle| <= 1e-9 * std(x_oracle); h, h': 1e-5
  * t, a, ad: relative 1e-12
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


def _close(engine, o, lat, bg, sigw, what):
    s = o.scalars
    assert abs(bg.a - s.a) <= 1e-12 * s.a, (what, bg.a, s.a)
    assert abs(bg.ad - s.ad) <= 1e-12 * abs(s.ad), (what, bg.ad, s.ad)
    assert abs(bg.t - s.t) <= 1e-12 * s.t, what
    assert bg.ad2 == s.ad2, what
    assert rel_field_err(lat.download(engine.F), o.f) < 1e-9, what
    assert rel_field_err(lat.download(engine.FD), o.fd) < 1e-9, what
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
