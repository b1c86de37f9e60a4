"""Failure detection on the GPU without a fault: bounded device waits.

The split form's persistent step kernel (many steps per cooperative launch)
waits between steps for every CTA's arrival and for the step's scalar update;
every such wait has a poll limit, after which the kernel marks the step
IEGPU_ETIMEOUT, ends the call's stepping and returns, so the host gets a status
instead of a hung GPU.  Here the wait is made to run out on purpose through the
test hook iegpu_set_wait_limit(ctx, polls, unreachable = 1): the step barrier
then waits for an arrival count that no launch reaches (a flag nothing sets).
Nothing faults, traps or hangs: the wait gives up after 64 polls.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W = dict(L=10.0, dt=1e-3, V0=3.338e-13, ns=0.965, phi0=0.0935, dphi0=0.000796)


def _lattice(engine, N=128):
    lat = engine.Lattice(N, W["L"], W["dt"], W["V0"], W["ns"], form=engine.FORM_SPLIT)
    lat.set_shape(16, 3, 0)      # a vector-row shape: persistent launches at 128^3
    lat.set_persistent(True)
    H = lat.bunch_davies(8, W["phi0"], W["dphi0"])
    bg = engine.Bg(0.0, 1.0, H, 0.0, 1.0)
    lat.evolve_fields(0.5 * W["dt"], bg)
    return lat, bg


def test_bounded_wait_gives_up_and_context_recovers(engine):
    ref, bg_r = _lattice(engine)
    lat, bg = _lattice(engine)
    with ref, lat:
        f0, fd0 = lat.download(engine.F), lat.download(engine.FD)
        bg0 = bg.as_tuple()
        lat.set_wait_limit(64, unreachable=True)
        with pytest.raises(engine.IegpuError) as e:
            lat.leapfrog(1e30, 40, bg)
        assert e.value.code == engine.ETIMEOUT
        assert "gave up" in str(e.value)
        # the context still runs a normal call: restore the state and the
        # limits, and step as the untouched context does from the same
        # uploaded state (an upload re-splits f into its mean and FP32
        # perturbations, so both contexts take the same round trip)
        lat.set_wait_limit(0, unreachable=False)
        for x in (lat, ref):
            x.upload(engine.F, f0)
            x.upload(engine.FD, fd0)
        bg, bg_r = engine.Bg(*bg0), engine.Bg(*bg0)
        assert lat.leapfrog(1e30, 40, bg) == 40
        assert ref.leapfrog(1e30, 40, bg_r) == 40
        assert bg.as_tuple() == bg_r.as_tuple()
        assert np.array_equal(lat.download(engine.F), ref.download(engine.F))
        assert np.array_equal(lat.download(engine.FD), ref.download(engine.FD))


def test_tight_wait_limit_completes(engine):
    """A poll limit of 2^14 (about a millisecond, some 70 steps' worth at
    128^3) without the unreachable target: the waits finish and the call gives
    the same bits as the default limit."""
    ref, bg_r = _lattice(engine)
    lat, bg = _lattice(engine)
    with ref, lat:
        lat.set_wait_limit(1 << 14)
        taken = lat.leapfrog(1e30, 30, bg)
        assert taken == 30 == ref.leapfrog(1e30, 30, bg_r)
        assert np.array_equal(lat.download(engine.F), ref.download(engine.F))
