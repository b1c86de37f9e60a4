"""Generate the golden fixtures of tests/golden/ from the reference program.

Runs the unmodified reference (caravangelo/inflation-easy, built from its own
sources by oracle/build_ref.py) on small lattices and stores, per case:
  <case>/results/*.dat     the reference's own text outputs
  <case>/trace.txt         background scalars at every save(), full precision
  <case>/state.npz         final f, fd, deltaN (and h, hd) in binary
  <case>/params.txt        the params file the reference read
and, in forcing_cutoff/cut_n<N>.npz, the reference's spectraf() run once on
seeded random f and fd with the forcing cutoff on (ie_ref --spectraf), for
several (high_cutoff_index, low_cutoff_index) pairs: f and fd after the call.
A post-inflation case keeps only results/post_inflation/ (its inflation and
deltaN outputs are those of the case without the phase).  This script needs
the reference tree, so it runs only where that exists; the fixtures it writes
are committed and travel without it.

    python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "oracle"))
import build_ref  # noqa: E402

HILLTOP = dict(seed=8, dt=0.001, V0=3.338e-13, ns=0.97, initial_field=0.0935, initial_derivative=0.000796, L=10.0,
               output_freq=500, output_infrequent_freq=500, output_spectra=1, output_histogram=1, output_energy=1,
               output_box3D=0, output_box2D=0, output_bispectrum=0, screen_updates=0, nbins=256, dN=1e-7,
               Nend=0.001, use_phiref_manual=0, output_LOG=0)
USR = dict(seed=8, dt=0.001, V0=3e-9, initial_field=2.9181235049318586, initial_derivative=-0.06727651095116181,
           L=10.0, output_freq=500, output_infrequent_freq=500, output_spectra=1, output_histogram=1,
           output_energy=1, output_box3D=0, output_box2D=1, output_bispectrum=0, screen_updates=0, nbins=256,
           dN=1e-4, Nend=2.0, use_phiref_manual=0, output_LOG=0)

# name: (N, numerical, sigw, deltaN, post-inflation phase, params)
CASES = {
    "n16_hilltop": (16, 0, 0, 1, 0, HILLTOP),
    "n16_usr_sigw": (16, 1, 1, 1, 0, USR),
    "n32_hilltop": (32, 0, 0, 1, 0, HILLTOP),
    "n16_usr_sigw_post": (16, 1, 1, 1, 1, USR),
    "n16_hilltop_rk4": (16, 0, 0, 1, 0, dict(HILLTOP, inflation_integrator="rk4")),
    # a step large enough for the RK45 step control to act (rejections, h below and above dt)
    "n16_hilltop_rk45": (16, 0, 0, 1, 0, dict(HILLTOP, dt=0.05, inflation_integrator="rk45", rk45_abs_tol=1e-12,
                                              rk45_rel_tol=1e-10)),
    "n16_usr_sigw_post_rk45": (16, 1, 1, 1, 1, dict(USR, post_inflation_integrator="rk45")),
    "n16_usr_dn_rk45": (16, 1, 0, 1, 0, dict(USR, deltaN_integrator="rk45")),
    # the forcing cutoff at every infrequent save (and the initial conditions' cutoff)
    "n16_hilltop_cutoff": (16, 0, 0, 1, 0, dict(HILLTOP, high_cutoff_index=5.5, forcing_cutoff=1)),
}

# spectraf() alone: N -> (high_cutoff_index, low_cutoff_index) pairs.  |p| runs
# up to 8 sqrt(3) = 13.9 at N = 16; a low cutoff > 0 also zeroes the k = 0
# mode; high = N/2 keeps the on-axis Nyquist modes (|p| = N/2 is not > N/2).
CUT_CASES = {
    8: [(2.5, 0.0), (3.0, 1.0), (4.0, 0.0), (3.5, 1.5), (0.5, 0.0), (7.0, 0.0)],
    16: [(5.5, 0.0), (6.0, 2.5)],
}


def make_cut_fixtures() -> None:
    out = HERE / "forcing_cutoff"
    out.mkdir(exist_ok=True)
    for N, pairs in CUT_CASES.items():
        exe = build_ref.build(N, 0, 0, 1)
        rng = np.random.default_rng(1000 + N)
        f = rng.standard_normal(N ** 3)
        fd = rng.standard_normal(N ** 3)
        res = {"f_in": f, "fd_in": fd, "cuts": np.array(pairs, dtype=np.float64)}
        for q, (hi, lo) in enumerate(pairs):
            work = ROOT / "oracle" / "_ref" / f"cut_n{N}_{q}"
            if work.exists():
                shutil.rmtree(work)
            (work / "results").mkdir(parents=True)
            with open(work / "cut_in.bin", "wb") as fp:
                fp.write(f.tobytes()); fp.write(fd.tobytes()); fp.write(np.array([hi, lo]).tobytes())
            subprocess.run([str(exe), "--spectraf", str(work)], check=True, stdout=subprocess.DEVNULL)
            o = np.fromfile(work / "cut_out.bin", dtype=np.float64)
            res[f"f_{q}"], res[f"fd_{q}"] = o[:N ** 3], o[N ** 3:]
            shutil.rmtree(work)
        np.savez_compressed(out / f"cut_n{N}.npz", **res)
        print(f"forcing_cutoff/cut_n{N}", "ok")


def params_text(p: dict) -> str:
    return "".join(f"{k} = {v!r}\n" if isinstance(v, float) else f"{k} = {v}\n" for k, v in p.items())


def read_state(path: Path):
    raw = path.read_bytes()
    hdr = np.frombuffer(raw[:16], dtype=np.int32)
    N, dn, sigw, _num = (int(x) for x in hdr)
    off = 16
    scal = np.frombuffer(raw[off:off + 64], dtype=np.float64).copy()
    off += 64
    gs = N ** 3
    out = {"scalars": scal}
    out["f"] = np.frombuffer(raw[off:off + 8 * gs], dtype=np.float64).copy(); off += 8 * gs
    out["fd"] = np.frombuffer(raw[off:off + 8 * gs], dtype=np.float64).copy(); off += 8 * gs
    if dn:
        out["deltaN"] = np.frombuffer(raw[off:off + 8 * gs], dtype=np.float64).copy(); off += 8 * gs
    if sigw:
        out["h"] = np.frombuffer(raw[off:off + 24 * gs], dtype=np.float32).reshape(6, gs).copy(); off += 24 * gs
        out["hd"] = np.frombuffer(raw[off:off + 24 * gs], dtype=np.float32).reshape(6, gs).copy(); off += 24 * gs
    return out


def main() -> None:
    if not build_ref.ref_available():
        raise SystemExit("reference tree not available; fixtures are generated where it is")
    only = set(sys.argv[1:])
    if not only or "forcing_cutoff" in only:
        make_cut_fixtures()
    for name, (N, num, sigw, dn, post, p) in CASES.items():
        if only and name not in only:
            continue
        exe = build_ref.build(N, num, sigw, dn, post=post)
        work = ROOT / "oracle" / "_ref" / f"golden_{name}"
        if work.exists():
            shutil.rmtree(work)
        work.mkdir(parents=True)
        (work / "params.txt").write_text(params_text(p))
        os.symlink(HERE / "inputs", work / "inputs")
        # the RK right-hand side sums with an OpenMP reduction, whose order follows
        # the thread count: one thread gives the serial loop order
        env = dict(os.environ, OMP_NUM_THREADS="1") if any(k.endswith("_integrator") for k in p) else None
        subprocess.run([str(exe), str(work)], check=True, stdout=subprocess.DEVNULL, env=env)
        dst = HERE / name
        if dst.exists():
            shutil.rmtree(dst)
        (dst / "results").mkdir(parents=True)
        if post:
            (dst / "results" / "post_inflation").mkdir()
            for f in sorted((work / "results" / "post_inflation").iterdir()):
                shutil.copy(f, dst / "results" / "post_inflation" / f.name)
        else:
            for f in sorted((work / "results").iterdir()):
                if f.name in ("info.dat", "output.txt") or f.is_dir():
                    continue
                shutil.copy(f, dst / "results" / f.name)
        shutil.copy(work / "trace.txt", dst / "trace.txt")
        shutil.copy(work / "params.txt", dst / "params.txt")
        st = read_state(work / "state.bin")
        np.savez_compressed(dst / "state.npz", **st)
        print(name, "ok")


if __name__ == "__main__":
    main()
