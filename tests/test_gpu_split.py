"""The split-precision form (FP32 perturbations about an FP64 background)
against the FP64 oracle.

Tolerances (the form's stated error budget):
  * perturbation fields after 300 steps: max|x - x_oracle| <= 1e-4 * std(x_oracle - mean)
  * a, ad, t: relative 1e-9 (FP64 background; lattice sums formed from FP32 data)
  * P_dphi per k-bin (bins >= 1): relative 1e-4; bin counts exact
"""
from __future__ import annotations

import numpy as np
import pytest

from test_gpu_parity import oracle_state

pytestmark = pytest.mark.gpu


def split_like(engine, p, o, usr, sigw, tables):
    lat = engine.Lattice(p.N, p.L, p.dt, p.V0, p.ns, p.rescale_B, form=engine.FORM_SPLIT,
                         potential=engine.POT_TABLE if usr else engine.POT_HILLTOP, sigw=sigw)
    if usr:
        lat.set_table(*tables)
    lat.upload(engine.F, o.f.copy())
    lat.upload(engine.FD, o.fd.copy())
    if sigw:
        for c in range(6):
            lat.upload(engine.H(c), o.h_(c).copy())
            lat.upload(engine.HD(c), o.hd_(c).copy())
    s = o.scalars
    return lat, engine.Bg(s.t, s.a, s.ad, s.ad2, s.astep)


def pert_err(got, ref):
    d = ref - ref.mean()
    return float(np.max(np.abs(got - ref)) / np.std(d))


def test_split_round_trip(engine, oracle_mod):
    p, o = oracle_state(oracle_mod, 32, False, False, None)
    lat, bg = split_like(engine, p, o, False, False, None)
    with lat:
        f = lat.download(engine.F)
        assert pert_err(f, o.f) < 1e-6
        sf, sfd, sf2 = lat.means()
        assert np.isclose(sf, o.f.sum(), rtol=1e-13)
        assert np.isclose(sfd, o.fd.sum(), rtol=1e-12)
        assert np.isclose(sf2, (o.f ** 2).sum(), rtol=1e-12)
        k, g, v = lat.energies(bg)
        ko, go, vo = o.energies()
        assert np.isclose(k, ko, rtol=1e-10) and np.isclose(v, vo, rtol=1e-12)
        assert np.isclose(g, go, rtol=1e-4)


@pytest.mark.parametrize("N,usr,sigw", [(32, False, False), (32, True, False), (16, True, True), (64, False, False),
                                        # N >= 32: the first call autotunes the step kernel's shape on
                                        # trial steps, which must leave the tensors alone
                                        (32, True, True), (64, False, True)])
def test_split_leapfrog_matches_fp64(N, usr, sigw, engine, oracle_mod, tables):
    p, o = oracle_state(oracle_mod, N, usr, sigw, tables)
    lat, bg = split_like(engine, p, o, usr, sigw, tables)
    with lat:
        taken = lat.leapfrog(p.af, 300, bg)
        assert taken == 300
        o.leapfrog_steps(300)
        s = o.scalars
        for got, ref in ((bg.a, s.a), (bg.ad, s.ad), (bg.t, s.t)):
            assert abs(got - ref) <= 1e-9 * abs(ref)
        assert pert_err(lat.download(engine.F), o.f) < 1e-4
        assert pert_err(lat.download(engine.FD), o.fd) < 1e-4
        if sigw:
            for c in range(6):
                h = lat.download(engine.H(c))
                ref = o.h_(c)
                assert np.max(np.abs(h - ref)) <= 1e-3 * np.std(ref)


def test_split_table_beyond_window(engine, oracle_mod, tables):
    """USR table with the background on the table's densest stretch (brackets
    of 2.7e-6 near phi = 2.6826) and perturbations of 3e-4: nearly every site
    lies beyond the window of brackets around phibar, so V' and V come from
    the whole table (far_line).  300 steps against the oracle, the same bars
    as the other leapfrog cases."""
    p, o = oracle_state(oracle_mod, 32, True, False, tables)
    f = o.f
    f[:] = 2.6827 + 4.0 * (f - f.mean())
    lat, bg = split_like(engine, p, o, True, False, tables)
    with lat:
        taken = lat.leapfrog(p.af, 300, bg)
        assert taken == 300
        o.leapfrog_steps(300)
        s = o.scalars
        for got, ref in ((bg.a, s.a), (bg.ad, s.ad), (bg.t, s.t)):
            assert abs(got - ref) <= 1e-9 * abs(ref)
        assert pert_err(lat.download(engine.F), o.f) < 1e-4
        assert pert_err(lat.download(engine.FD), o.fd) < 1e-4


def test_split_spectrum(engine, oracle_mod):
    p, o = oracle_state(oracle_mod, 32, False, False, None, steps=100)
    lat, bg = split_like(engine, p, o, False, False, None)
    with lat:
        counts, f2 = lat.spectrum(engine.F)
        oc, of2 = o.spectrum_f()
        assert np.array_equal(counts, oc)
        assert np.isclose(f2[0], of2[0], rtol=1e-12)
        assert np.allclose(f2[1:], of2[1:], rtol=1e-6)


def test_split_deltaN_stage(engine, oracle_mod, tables):
    p, o = oracle_state(oracle_mod, 16, True, False, tables, steps=30)
    lat, bg = split_like(engine, p, o, True, False, tables)
    with lat:
        lat.initializeN(o.scalars.a)
        o.initializeN()
        lat.evolve_fieldsN(0.5 * p.dN, 0.0)
        o.evolve_fieldsN(0.5 * p.dN)
        phiref = lat.get_phiref()
        s = o.scalars
        s.phiref = o.get_phiref()
        o.set_scalars(s)
        # phi = phibar + (double)dphi carries the FP32 rounding of dphi (~1e-7 of dphi)
        assert abs(phiref - s.phiref) <= 1e-6 * np.std(o.f)
        lat.deltaN_steps(p.dN, 200, phiref)
        o.deltaN_steps(200)
        dn = lat.download(engine.DELTAN)
        assert np.max(np.abs(dn - o.deltaN)) <= 3 * p.dN


def test_split_autotune_keeps_state(engine, oracle_mod):
    p, o = oracle_state(oracle_mod, 64, False, False, None, steps=5)
    lat, bg = split_like(engine, p, o, False, False, None)
    with lat:
        before = lat.download(engine.F)
        shape = lat.autotune(bg)
        assert shape["rows"] in (4, 8) and shape["prefetch"] in (1, 2) and shape["chunks"] >= 1
        assert np.array_equal(lat.download(engine.F), before)
        taken = lat.leapfrog(p.af, 50, bg)
        o.leapfrog_steps(50)
        assert taken == 50
        assert pert_err(lat.download(engine.F), o.f) < 1e-4


@pytest.mark.parametrize("N", [32, 64])
def test_split_whole_plane_kernel(N, engine, oracle_mod, tables):
    """The whole-plane step kernel (N <= 64) against the FP64 oracle and against
    the row-tile kernel on the same state."""
    p, o = oracle_state(oracle_mod, N, True, False, tables)
    out = {}
    for name, shape in (("plane", (N, 4, N // 16)), ("rows", (8, 2, N // 32))):
        lat, bg = split_like(engine, p, o, True, False, tables)
        with lat:
            lat.set_shape(*shape)
            assert lat.leapfrog(p.af, 200, bg) == 200
            out[name] = (lat.download(engine.F), lat.download(engine.FD), bg.as_tuple())
    o.leapfrog_steps(200)
    for name in out:
        assert pert_err(out[name][0], o.f) < 1e-4 and pert_err(out[name][1], o.fd) < 1e-4, name
        assert abs(out[name][2][1] - o.scalars.a) <= 1e-9 * o.scalars.a
    # the two kernels differ only in FP32 summation order
    assert pert_err(out["plane"][0], out["rows"][0]) < 1e-5


@pytest.mark.parametrize("N,shapes", [(128, [(16, 12, 8), (16, 11, 0), (16, 13, 8), (8, 12, 4)]),
                                      (256, [(16, 12, 9), (8, 12, 9)])])
def test_split_bulk_copy_staging_matches(N, shapes, engine, tables):
    """Planes staged by bulk (TMA) copies give the same bits as planes staged
    by cp.async with the same tiling."""
    w = dict(L=10.0, dt=1e-3, V0=3e-9, phi0=2.9181235049318586, dphi0=-0.06727651095116181)
    out = {}
    for sh in shapes + [(sh[0], sh[1] - 10 if sh[1] - 10 in (1, 2) else 2, sh[2]) for sh in shapes]:
        lat = engine.Lattice(N, w["L"], w["dt"], w["V0"], potential=engine.POT_TABLE, form=engine.FORM_SPLIT)
        with lat:
            lat.set_table(*tables)
            lat.set_shape(*sh)
            H = lat.bunch_davies(5, w["phi0"], w["dphi0"])
            bg = engine.Bg(0.0, 1.0, H, 0.0, 1.0)
            lat.evolve_fields(0.5 * w["dt"], bg)
            assert lat.leapfrog(1e30, 30, bg) == 30
            out[sh] = (lat.download(engine.F), lat.download(engine.FD), bg.as_tuple())
    for sh in shapes:
        ref = (sh[0], sh[1] - 10 if sh[1] - 10 in (1, 2) else 2, sh[2])
        if sh[1] - 10 != ref[1]:
            continue   # no cp.async shape with that prefetch depth and rows
        assert np.array_equal(out[sh][0], out[ref][0]) and np.array_equal(out[sh][1], out[ref][1]), sh
        assert out[sh][2] == out[ref][2], sh
    # every staging gives the same trajectory up to FP32 summation order
    base = out[shapes[0]][0]
    for sh, v in out.items():
        assert np.max(np.abs(v[0] - base)) <= 1e-6 * np.std(base - base.mean()), sh


ROWCASE = {False: dict(L=10.0, dt=1e-3, V0=3.338e-13, ns=0.965, phi0=0.0935, dphi0=0.000796),
           True: dict(L=10.0, dt=1e-3, V0=3e-9, ns=0.97, phi0=2.9181235049318586, dphi0=-0.06727651095116181)}


@pytest.mark.parametrize("N,usr,shape", [(128, False, (16, 2, 0)), (128, True, (16, 3, 0)), (256, False, (16, 3, 9)),
                                         (256, False, (4, 2, 7)),
                                         # 512^3 with the table: the five-bracket window cache
                                         (512, True, (8, 2, 0))])
def test_split_row_kernel_matches_fp64(N, usr, shape, engine, tables):
    """The vector row kernel (N >= 128) against the plain FP64 form from the
    same device initial conditions, 300 steps.  With the hilltop potential the
    last CTA of each step forms the friction in double-float arithmetic and the
    FP64 update of the background follows in the next step; with the table it
    runs the precomputed FP64 update.  Fields within 1e-4 of their spread and
    a, ad, t relative 1e-9 after 120 steps; then the a(t) trace of a second
    call within relative 1e-9 of the FP64 run's, and the stop on af at the
    step the FP64 trace puts it."""
    w = ROWCASE[usr]
    pot = engine.POT_TABLE if usr else engine.POT_HILLTOP
    runs, af = {}, 1e30
    for form in (engine.FORM_FP64, engine.FORM_SPLIT):
        lat = engine.Lattice(N, w["L"], w["dt"], w["V0"], w["ns"], potential=pot, form=form)
        if usr:
            lat.set_table(*tables)
        if form == engine.FORM_SPLIT:
            lat.set_shape(*shape)
        H = lat.bunch_davies(7, w["phi0"], w["dphi0"])
        bg = engine.Bg(0.0, 1.0, H, 0.0, 1.0)
        lat.evolve_fields(0.5 * w["dt"], bg)
        # two calls, the second from the first's end state; the split run's
        # second call stops on a(t) crossing af, midway between the FP64 run's
        # a after steps 100 and 101 of that call
        assert lat.leapfrog(1e30, 120, bg) == 120
        fields = (lat.download(engine.F), lat.download(engine.FD), bg.a, bg.ad, bg.t)
        bg.astep = bg.a
        taken, tr = lat.leapfrog(af, 180, bg, trace=True)
        runs[form] = (lat, bg, taken, tr, fields)
        af = 0.5 * (tr[99] + tr[100])
    lf, bf, tf, trf, ff = runs[engine.FORM_FP64]
    ls, bs, ts, trs, fs = runs[engine.FORM_SPLIT]
    with ls, lf:
        # after the first call: fields within 1e-4 of their spread, a, ad, t relative 1e-9
        assert pert_err(fs[0], ff[0]) < 1e-4 and pert_err(fs[1], ff[1]) < 1e-4
        for got, ref in zip(fs[2:], ff[2:]):
            assert abs(got - ref) <= 1e-9 * abs(ref)
        assert tf == 180 and ts == 101
        assert np.all(np.abs(trs - trf[:ts]) <= 1e-9 * trf[:ts])
        assert abs(bs.a - trf[ts - 1]) <= 1e-9 * trf[ts - 1]


@pytest.mark.parametrize("N,usr,shape", [(128, False, (16, 2, 0)), (128, True, (8, 2, 4)), (256, False, (16, 3, 9)),
                                         (512, False, (4, 2, 16))])
def test_split_comp_matches_fp64(N, usr, shape, engine, tables):
    """The compensated split form against the plain FP64 form from the same
    device initial conditions, 400 steps: fields within 1e-4 of their spread
    (and no farther than the plain split form's), a, ad, t relative 1e-9; the
    residuals enter every read of the state (downloads and spectra)."""
    w = ROWCASE[usr]
    pot = engine.POT_TABLE if usr else engine.POT_HILLTOP
    res = {}
    for form in (engine.FORM_FP64, engine.FORM_SPLIT, engine.FORM_SPLIT_COMP):
        lat = engine.Lattice(N, w["L"], w["dt"], w["V0"], w["ns"], potential=pot, form=form)
        with lat:
            if usr:
                lat.set_table(*tables)
            if form != engine.FORM_FP64:
                lat.set_shape(*shape)
            H = lat.bunch_davies(7, w["phi0"], w["dphi0"])
            bg = engine.Bg(0.0, 1.0, H, 0.0, 1.0)
            lat.evolve_fields(0.5 * w["dt"], bg)
            assert lat.leapfrog(1e30, 400, bg) == 400
            res[form] = (lat.download(engine.F), lat.download(engine.FD), bg.as_tuple(), lat.spectrum(engine.F))
    f64, sp, cp = res[engine.FORM_FP64], res[engine.FORM_SPLIT], res[engine.FORM_SPLIT_COMP]
    for q in (0, 1):
        assert pert_err(cp[q], f64[q]) < 1e-4
        assert pert_err(cp[q], f64[q]) <= pert_err(sp[q], f64[q])
    for got, ref in zip(cp[2][:3], f64[2][:3]):
        assert abs(got - ref) <= 1e-9 * abs(ref)
    assert np.array_equal(cp[3][0], f64[3][0])
    assert np.allclose(cp[3][1][1:], f64[3][1][1:], rtol=1e-4)


@pytest.mark.parametrize("N,usr,shape", [(128, False, (16, 3, 0)), (128, True, (8, 2, 4)), (256, False, (16, 3, 9)),
                                         (256, True, (4, 2, 7))])
def test_split_persistent_launch_matches(N, usr, shape, engine, tables):
    _persistent_matches(N, usr, shape, engine, tables, engine.FORM_SPLIT)


@pytest.mark.parametrize("N,usr,shape", [(128, False, (16, 3, 0)), (128, True, (8, 2, 4)), (256, False, (16, 2, 9))])
def test_split_comp_persistent_launch_matches(N, usr, shape, engine, tables):
    _persistent_matches(N, usr, shape, engine, tables, engine.FORM_SPLIT_COMP)


def _persistent_matches(N, usr, shape, engine, tables, form):
    """Many steps per cooperative launch against one launch per step: the
    same fields, a(t) trace, background and steps taken, bit for bit, over
    three calls (150 steps, then 70, then a call stopped by af), so launches
    end mid-call and the buffer parity changes between calls."""
    w = ROWCASE[usr]
    pot = engine.POT_TABLE if usr else engine.POT_HILLTOP
    out = []
    for persist in (False, True):
        lat = engine.Lattice(N, w["L"], w["dt"], w["V0"], w["ns"], potential=pot, form=form)
        if usr:
            lat.set_table(*tables)
        lat.set_shape(*shape)
        lat.set_persistent(persist)
        H = lat.bunch_davies(5, w["phi0"], w["dphi0"])
        bg = engine.Bg(0.0, 1.0, H, 0.0, 1.0)
        lat.evolve_fields(0.5 * w["dt"], bg)
        rec = []
        for steps, af in ((150, 1e30), (70, 1e30), (100, None)):
            if af is None:
                # about 42 steps past the end of the previous call
                prev = rec[-1][1]
                af = prev[-1] + 41.5 * (prev[-1] - prev[-2])
            taken, tr = lat.leapfrog(af, steps, bg, trace=True)
            bg.astep = bg.a
            rec.append((taken, tr, bg.as_tuple(), lat.download(engine.F), lat.download(engine.FD)))
        out.append(rec)
        lat.close()
    for (ta, tra, bga, fa, fda), (tb, trb, bgb, fb, fdb) in zip(*out):
        assert ta == tb and np.array_equal(tra, trb) and bga == bgb
        assert np.array_equal(fa, fb) and np.array_equal(fda, fdb)
    taken = [r[0] for r in out[0]]
    assert taken[:2] == [150, 70] and 0 < taken[2] < 100


def test_split_whole_run_error_128(engine, tmp_path):
    """The split forms' error over a whole run: 128^3 hilltop (the reference's
    params.analytic.txt with ns = 0.965, seed 8), the inflation loop to
    af = 2N = 256 (9603 steps) and the deltaN stage, each split form against
    the plain FP64 form from the same device initial conditions, every save
    compared at full precision.

    deltaN counts whole steps of dN = 1e-7 (src/evolution.cpp:1015-1037), so
    zeta is quantised: a site whose end-of-inflation state moves by a tiny
    amount can cross the end surface one step earlier or later.  The split
    form's FP32 updates round every step, and over ~10^4 steps the rounding
    walks the state by ~100 single roundings; about 1 % of the sites then
    cross one dN step off, which moves the highest-k P_zeta bins by up to
    2e-4.  Apart from those whole steps the deltaN maps agree: with them taken
    out P_zeta matches to 1e-12.  The compensated form (Kahan residuals
    carried from step to step) keeps the state within about one rounding and
    meets the 1e-4 bar on every bin.
    Bars: compensated form: P_zeta and P_dphi per k-bin 1e-4, <dphi^2> 1e-5;
    plain split form: P_dphi per k-bin 1e-4, P_zeta per k-bin 3e-4, the deltaN
    maps equal up to whole dN steps (and the constant of the float Nmean) at
    fewer than 2 % of the sites; both: H and a relative 1e-9."""
    import form_error as fe
    text = fe.preset_text(fe.HILLTOP, 128)
    ref = fe.run_program(text, tmp_path / "fp64", "fp64")
    errs = {}
    for form in ("split", "split_comp"):
        got = fe.run_program(text, tmp_path / form, form)
        errs[form] = err = fe.compare(ref, got)
        flips = fe.deltaN_steps_off(ref, got, 1e-7)
        print(form, {k: v for k, v in err.items() if k != "H_per_save"}, flips)
        assert err["saves"] > 10
        assert err["P_dphi"]["max"] <= 1e-4
        assert err["H_max"] <= 1e-9 and err["a_max"] <= 1e-9
        assert flips["off_by_fraction"] <= 1e-9   # whole dN steps only
    assert errs["split_comp"]["P_zeta"]["max"] <= 1e-4
    assert errs["split_comp"]["dphi2_max"] <= 1e-5
    assert errs["split"]["P_zeta"]["max"] <= 3e-4
    assert err["dphi2_max"] <= 1e-4
    assert err["H_max"] <= 1e-9 and err["a_max"] <= 1e-9
