"""Size-independent properties at the workloads' full lattice sizes, where the
oracle would take too long: the FP64 form's spectrum obeys Parseval's identity
(the bins of the nonzero modes, with the corner mode where it falls past the
last bin, sum to N^3 sum (f - <f>)^2; the counts to N^3 less that mode, the
reference's weights being 2
for 0 < kz < N/2 and 1 on the kz = 0 and Nyquist planes; src/output.cpp:63-151),
and its forward + inverse FFT returns the field to rounding level."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HILL = dict(L=10.0, dt=1e-3, V0=3.338e-13, ns=0.965, phi0=0.0935, dphi0=0.000796)


@pytest.mark.parametrize("N", [256, 512])
def test_fp64_spectrum_parseval_and_round_trip(N, engine):
    w = HILL
    with engine.Lattice(N, w["L"], w["dt"], w["V0"], w["ns"], form=engine.FORM_FP64) as lat:
        H = lat.bunch_davies(8, w["phi0"], w["dphi0"])
        bg = engine.Bg(0.0, 1.0, H, 0.0, 1.0)
        lat.evolve_fields(0.5 * w["dt"], bg)
        assert lat.leapfrog(1e30, 10, bg) == 10
        f = lat.download(engine.F)
        counts, f2 = lat.spectrum(engine.F)
        g = lat.download(engine.F)
    # every mode is binned, except the corner (N/2, N/2, N/2) when its |p| =
    # sqrt(3) N/2 rounds to numbins, past the last bin (N = 256: 221.7 -> 222 of
    # 222 bins; N = 512: 443.4 -> 443 of 444), in the reference's binning too
    corner_out = int(np.floor(np.sqrt(3.0) * N / 2 + 0.5)) >= len(counts)
    assert int(counts.sum()) == N ** 3 - (1 if corner_out else 0)
    assert counts[0] == 1
    f3 = f.reshape(N, N, N)
    a = f3[:, :, 0::2].sum(axis=2) - f3[:, :, 1::2].sum(axis=2)
    b = a[:, 0::2].sum(axis=1) - a[:, 1::2].sum(axis=1)
    corner = float(b[0::2].sum() - b[1::2].sum())   # sum of f (-1)^(i+j+k)
    d = f - f.mean()
    ref = float(N) ** 3 * float(np.dot(d, d))
    assert abs(float(f2[1:].sum()) + (corner ** 2 if corner_out else 0.0) - ref) <= 1e-8 * ref
    # the zero mode is the squared sum of the field
    assert abs(f2[0] - float(f.sum()) ** 2) <= 1e-12 * f2[0]
    # the spectrum transforms f forward and back
    assert np.max(np.abs(g - f)) <= 1e-12 * np.max(np.abs(f))
