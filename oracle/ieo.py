"""ctypes binding of the CPU oracle (oracle/ieo.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, never by the product.  build() compiles the
oracle from its C sources with gcc (-ffp-contract=off, OpenMP) into
oracle/_build/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libieo.so"
CLI = BUILD / "ieo_cli"
CFLAGS = ["-std=c11", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-Wall"]


def build() -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = [HERE / "ieo.c", HERE / "ieo.h"]
    newest = max(s.stat().st_mtime for s in srcs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        subprocess.check_call(["gcc", *CFLAGS, "-shared", str(HERE / "ieo.c"), "-o", str(LIB), "-lm"])
    if not CLI.exists() or CLI.stat().st_mtime < max(newest, (HERE / "ieo_cli.c").stat().st_mtime):
        subprocess.check_call(["gcc", *CFLAGS, str(HERE / "ieo.c"), str(HERE / "ieo_cli.c"), "-o", str(CLI), "-lm"])
    return LIB


class Params(C.Structure):
    _fields_ = [("N", C.c_int), ("numerical_potential", C.c_int), ("perform_deltaN", C.c_int),
                ("calculate_SIGW", C.c_int), ("criterion", C.c_int), ("seed", C.c_int),
                ("rescale_s", C.c_double), ("af", C.c_double), ("V0", C.c_double), ("rescale_B", C.c_double),
                ("ns", C.c_double), ("initial_field", C.c_double), ("initial_derivative", C.c_double),
                ("L", C.c_double), ("dt", C.c_double), ("output_freq", C.c_int),
                ("output_infrequent_freq", C.c_int), ("dN", C.c_double), ("Nend", C.c_double),
                ("use_phiref_manual", C.c_int), ("phiref_manual_value", C.c_double),
                ("high_cutoff_index", C.c_double), ("low_cutoff_index", C.c_double), ("forcing_cutoff", C.c_int),
                ("output_spectra", C.c_int), ("output_histogram", C.c_int), ("output_energy", C.c_int),
                ("output_box3D", C.c_int), ("output_box2D", C.c_int), ("screen_updates", C.c_int),
                ("nbins", C.c_int), ("int_err", C.c_int), ("int_errN", C.c_int), ("dx", C.c_double),
                ("post_inflation", C.c_int), ("af_post_given", C.c_int), ("horizon_factor", C.c_double),
                ("omega", C.c_double), ("dt_post_inflation", C.c_double), ("af_post_inflation", C.c_double),
                ("inflation_integrator", C.c_int), ("pad_", C.c_int),
                ("post_inflation_integrator", C.c_int), ("deltaN_integrator", C.c_int),
                ("rk45_abs_tol", C.c_double), ("rk45_rel_tol", C.c_double), ("rk45_min_dt", C.c_double),
                ("rk45_max_dt", C.c_double), ("rk45_safety", C.c_double),
                ("rk45_min_given", C.c_int), ("rk45_max_given", C.c_int)]


class Scalars(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("t", "a", "ad", "ad2", "astep", "Ne", "phiref", "hubble_init")]


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = C.CDLL(str(LIB))
    P, I, D = C.c_void_p, C.c_int, C.c_double
    dp, fp, ip = C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_int)
    sig = {
        "ieo_params_defaults": (None, [C.POINTER(Params), I, I]),
        "ieo_params_load": (I, [C.POINTER(Params), C.c_char_p]),
        "ieo_params_finalize": (None, [C.POINTER(Params), I, I]),
        "ieo_create": (P, [C.POINTER(Params)]),
        "ieo_destroy": (None, [P]),
        "ieo_set_threads": (None, [I]),
        "ieo_set_table": (I, [P, dp, dp, dp, I]),
        "ieo_f": (dp, [P]), "ieo_fd": (dp, [P]), "ieo_deltaN": (dp, [P]),
        "ieo_fnyquist": (dp, [P]), "ieo_fdnyquist": (dp, [P]),
        "ieo_h": (fp, [P, I]), "ieo_hd": (fp, [P, I]),
        "ieo_get_scalars": (None, [P, C.POINTER(Scalars)]),
        "ieo_set_scalars": (None, [P, C.POINTER(Scalars)]),
        "ieo_last_error": (C.c_char_p, [P]),
        "ieo_rand_uniform": (D, [P]),
        "ieo_initialize": (I, [P]), "ieo_initializef": (I, [P]), "ieo_initializeGW": (None, [P]),
        "ieo_potential": (D, [P, D]), "ieo_potential_energy": (D, [P]),
        "ieo_gradient_energy": (D, [P]), "ieo_kin_energy": (D, [P]),
        "ieo_evolve_derivs": (I, [P, D]), "ieo_evolve_fields": (None, [P, D]),
        "ieo_initialize_post_inflation": (None, [P]), "ieo_evolve_derivs_post_inflation": (None, [P, D]),
        "ieo_rk4_step_inflation": (I, [P, D]),
        "ieo_rk45_step_inflation": (I, [P, D, D, dp, ip]), "ieo_rk45_accept": (I, [P, dp, D]),
        "ieo_rk4_step_deltaN": (I, [P, D]), "ieo_rk45_step_deltaN": (I, [P, D, D, dp, ip]),
        "ieo_rk45_accept_deltaN": (I, [P, dp, D]),
        "ieo_rk45_clamp": (D, [P, D, D]), "ieo_rk45_hmax": (D, [P, D]), "ieo_set_rk_post": (None, [P, I]),
        "ieo_rescaled_step": (D, [P, D]), "ieo_leapfrog_steps": (I, [P, I]),
        "ieo_set_engine_arith": (None, [P, I]), "ieo_exact_sum": (D, [dp, C.c_size_t]),
        "ieo_set_engine_arith_default": (None, [I]),
        "ieo_exact_dot": (D, [dp, dp, C.c_size_t]),
        "ieo_fftrn_d": (None, [dp, dp, I, I]), "ieo_fftrn_f": (None, [fp, fp, I, I]),
        "ieo_numbins": (I, [I]),
        "ieo_bin_spectrum": (None, [I, dp, dp, ip, dp]),
        "ieo_spectrum_f": (None, [P, ip, dp]),
        "ieo_spectrum_f_cut": (None, [P, ip, dp, D, D]),
        "ieo_gw_spectrum": (None, [P, I, D, ip, fp, dp]),
        "ieo_initializeN": (I, [P]), "ieo_evolve_derivsN": (I, [P, D]), "ieo_evolve_fieldsN": (None, [P, D]),
        "ieo_get_phiref": (D, [P]), "ieo_deltaN_steps": (I, [P, I]), "ieo_saveN_mean": (C.c_float, [P, D]),
        "ieo_run_program": (I, [C.POINTER(Params), C.c_char_p, C.c_char_p]),
        "ieo_run_program_dump": (I, [C.POINTER(Params), C.c_char_p, C.c_char_p, C.c_char_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def default_params(N: int, numerical: bool, **kw) -> Params:
    lib = load()
    p = Params()
    lib.ieo_params_defaults(C.byref(p), N, int(numerical))
    B_given = "rescale_B" in kw
    af_given = "af" in kw
    for k, v in kw.items():
        setattr(p, k, v)
    if "af_post_inflation" in kw:
        p.af_post_given = 1
    if "rk45_min_dt" in kw:
        p.rk45_min_given = 1
    if "rk45_max_dt" in kw:
        p.rk45_max_given = 1
    lib.ieo_params_finalize(C.byref(p), int(B_given), int(af_given))
    return p


def hilltop_params(N: int, **kw) -> Params:
    """params.analytic.txt of the reference (hilltop preset)."""
    base = dict(seed=8, dt=0.001, V0=3.338e-13, ns=0.97, initial_field=0.0935, initial_derivative=0.000796,
                L=10.0, output_freq=500, output_infrequent_freq=500, dN=1e-7, Nend=0.001, nbins=256,
                screen_updates=0)
    base.update(kw)
    return default_params(N, False, **base)


def usr_params(N: int, **kw) -> Params:
    """params.numerical.txt of the reference (tabulated USR preset)."""
    base = dict(seed=8, dt=0.001, V0=3e-9, initial_field=2.9181235049318586,
                initial_derivative=-0.06727651095116181, L=10.0, output_freq=500, output_infrequent_freq=500,
                dN=1e-4, Nend=2.0, nbins=256, output_box2D=1, screen_updates=0)
    base.update(kw)
    return default_params(N, True, **base)


def exact_sum(x) -> float:
    """Correctly rounded exact sum (the oracle's long accumulator)."""
    a = np.ascontiguousarray(x, dtype=np.float64)
    return load().ieo_exact_sum(a.ctypes.data_as(C.POINTER(C.c_double)), a.size)


def exact_dot(x, y) -> float:
    """Correctly rounded exact sum of the exact products x[i] y[i]."""
    a = np.ascontiguousarray(x, dtype=np.float64)
    b = np.ascontiguousarray(y, dtype=np.float64)
    return load().ieo_exact_dot(a.ctypes.data_as(C.POINTER(C.c_double)), b.ctypes.data_as(C.POINTER(C.c_double)),
                                a.size)


def load_tables(inputs_dir: Path):
    return tuple(np.loadtxt(inputs_dir / n) for n in ("field_values.dat", "potential.dat", "potential_derivative.dat"))


class Oracle:
    """One oracle state (ieo_state)."""

    def __init__(self, params: Params, tables=None, threads: int | None = None):
        self.lib = load()
        if threads:
            self.lib.ieo_set_threads(threads)
        self.p = params
        self.N = params.N
        self.h = self.lib.ieo_create(C.byref(params))
        if not self.h:
            raise MemoryError("ieo_create failed")
        if tables is not None:
            phi, V, dV = (np.ascontiguousarray(t, dtype=np.float64) for t in tables)
            dp = C.POINTER(C.c_double)
            self.lib.ieo_set_table(self.h, phi.ctypes.data_as(dp), V.ctypes.data_as(dp), dV.ctypes.data_as(dp),
                                   len(phi))

    def set_engine_arith(self, on: bool = True) -> None:
        """The engine's lattice-sum arithmetic (exact sums, its potential sum
        and pow forms) instead of the reference's serial sums."""
        self.lib.ieo_set_engine_arith(self.h, int(on))

    def close(self):
        if self.h:
            self.lib.ieo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc:
            raise RuntimeError(self.lib.ieo_last_error(self.h).decode())

    # views
    def _view(self, ptr, n, dt):
        return np.ctypeslib.as_array(ptr, shape=(n,)).view(dt) if ptr else None

    @property
    def f(self):
        return np.ctypeslib.as_array(self.lib.ieo_f(self.h), shape=(self.N ** 3,))

    @property
    def fd(self):
        return np.ctypeslib.as_array(self.lib.ieo_fd(self.h), shape=(self.N ** 3,))

    @property
    def deltaN(self):
        return np.ctypeslib.as_array(self.lib.ieo_deltaN(self.h), shape=(self.N ** 3,))

    @property
    def fny(self):
        return np.ctypeslib.as_array(self.lib.ieo_fnyquist(self.h), shape=(2 * self.N * self.N,))

    @property
    def fdny(self):
        return np.ctypeslib.as_array(self.lib.ieo_fdnyquist(self.h), shape=(2 * self.N * self.N,))

    def h_(self, c):
        return np.ctypeslib.as_array(self.lib.ieo_h(self.h, c), shape=(self.N ** 3,))

    def hd_(self, c):
        return np.ctypeslib.as_array(self.lib.ieo_hd(self.h, c), shape=(self.N ** 3,))

    @property
    def scalars(self) -> Scalars:
        s = Scalars()
        self.lib.ieo_get_scalars(self.h, C.byref(s))
        return s

    def set_scalars(self, s: Scalars):
        self.lib.ieo_set_scalars(self.h, C.byref(s))

    # steps
    def initialize_all(self):
        """initialize() + initializef() + initializeGW() of src/initialize.cpp:40-48."""
        self._check(self.lib.ieo_initialize(self.h))
        self._check(self.lib.ieo_initializef(self.h))
        self.lib.ieo_initializeGW(self.h)

    def evolve_fields(self, d):
        self.lib.ieo_evolve_fields(self.h, d)

    def evolve_derivs(self, d):
        self._check(self.lib.ieo_evolve_derivs(self.h, d))

    def rk4_step_inflation(self, h):
        self._check(self.lib.ieo_rk4_step_inflation(self.h, h))

    def rk45_step_inflation(self, h, hmax):
        """One RK45 attempt: (accepted, h_next)."""
        hn, acc = C.c_double(h), C.c_int(0)
        self._check(self.lib.ieo_rk45_step_inflation(self.h, h, hmax, C.byref(hn), C.byref(acc)))
        return bool(acc.value), hn.value

    def rk45_accept(self, h, hmax):
        """rk45_accept_step: attempts until one is accepted; the next step's h."""
        hh = C.c_double(h)
        self._check(self.lib.ieo_rk45_accept(self.h, C.byref(hh), hmax))
        return hh.value

    def rk4_step_deltaN(self, h):
        self._check(self.lib.ieo_rk4_step_deltaN(self.h, h))

    def rk45_step_deltaN(self, h, hmax):
        hn, acc = C.c_double(h), C.c_int(0)
        self._check(self.lib.ieo_rk45_step_deltaN(self.h, h, hmax, C.byref(hn), C.byref(acc)))
        return bool(acc.value), hn.value

    def rk45_accept_deltaN(self, h, hmax):
        hh = C.c_double(h)
        self._check(self.lib.ieo_rk45_accept_deltaN(self.h, C.byref(hh), hmax))
        return hh.value

    def rk45_clamp(self, h, hmax):
        return self.lib.ieo_rk45_clamp(self.h, h, hmax)

    def rk45_hmax(self, base_step):
        return self.lib.ieo_rk45_hmax(self.h, base_step)

    def set_rk_post(self, post):
        self.lib.ieo_set_rk_post(self.h, int(bool(post)))

    def initialize_post_inflation(self):
        self.lib.ieo_initialize_post_inflation(self.h)

    def evolve_derivs_post_inflation(self, d):
        self.lib.ieo_evolve_derivs_post_inflation(self.h, d)

    def rescaled_step(self, astep):
        return self.lib.ieo_rescaled_step(self.h, astep)

    def leapfrog_steps(self, n):
        r = self.lib.ieo_leapfrog_steps(self.h, n)
        if r < 0:
            self._check(1)
        return r

    def energies(self):
        return (self.lib.ieo_kin_energy(self.h), self.lib.ieo_gradient_energy(self.h),
                self.lib.ieo_potential_energy(self.h))

    def spectrum_f(self, high_cutoff=0.0, low_cutoff=0.0):
        """spectraf(): f's spectrum; with high_cutoff > 0 the forcing cutoff
        also zeroes f's and fd's modes outside [low_cutoff, high_cutoff]."""
        nb = self.lib.ieo_numbins(self.N)
        counts = np.zeros(nb, dtype=np.int32)
        f2 = np.zeros(nb, dtype=np.float64)
        self.lib.ieo_spectrum_f_cut(self.h, counts.ctypes.data_as(C.POINTER(C.c_int)),
                                    f2.ctypes.data_as(C.POINTER(C.c_double)), high_cutoff, low_cutoff)
        return counts, f2

    def gw_spectrum(self, which, to_phys=1.0):
        nb = self.lib.ieo_numbins(self.N)
        counts = np.zeros(nb, dtype=np.int32)
        f2 = np.zeros(nb, dtype=np.float32)
        f2d = np.zeros(nb, dtype=np.float64)
        self.lib.ieo_gw_spectrum(self.h, which, to_phys, counts.ctypes.data_as(C.POINTER(C.c_int)),
                                 f2.ctypes.data_as(C.POINTER(C.c_float)), f2d.ctypes.data_as(C.POINTER(C.c_double)))
        return counts, f2, f2d

    def initializeN(self):
        self._check(self.lib.ieo_initializeN(self.h))

    def evolve_fieldsN(self, d):
        self.lib.ieo_evolve_fieldsN(self.h, d)

    def evolve_derivsN(self, d):
        self._check(self.lib.ieo_evolve_derivsN(self.h, d))

    def get_phiref(self):
        return self.lib.ieo_get_phiref(self.h)

    def deltaN_steps(self, n):
        return self.lib.ieo_deltaN_steps(self.h, n)

    def saveN_mean(self, cutoff):
        return self.lib.ieo_saveN_mean(self.h, cutoff)


def fftrn_d(f: np.ndarray, fny: np.ndarray, N: int, forward: int):
    lib = load()
    dp = C.POINTER(C.c_double)
    lib.ieo_fftrn_d(f.ctypes.data_as(dp), fny.ctypes.data_as(dp), N, forward)


def fftrn_f(f: np.ndarray, fny: np.ndarray, N: int, forward: int):
    lib = load()
    fp = C.POINTER(C.c_float)
    lib.ieo_fftrn_f(f.ctypes.data_as(fp), fny.ctypes.data_as(fp), N, forward)


def bin_spectrum(N: int, ff: np.ndarray, nyq: np.ndarray):
    lib = load()
    nb = lib.ieo_numbins(N)
    counts = np.zeros(nb, dtype=np.int32)
    f2 = np.zeros(nb, dtype=np.float64)
    dp = C.POINTER(C.c_double)
    lib.ieo_bin_spectrum(N, ff.ctypes.data_as(dp), nyq.ctypes.data_as(dp), counts.ctypes.data_as(C.POINTER(C.c_int)),
                         f2.ctypes.data_as(dp))
    return counts, f2


def run_program(params: Params, results_dir: Path, inputs_dir: Path, dump_dir: Path | None = None,
                engine_arith: bool = False) -> int:
    """The reference program's main() restated; engine_arith runs it with the
    engine's lattice-sum arithmetic (Oracle.set_engine_arith)."""
    lib = load()
    lib.ieo_set_engine_arith_default(int(engine_arith))
    try:
        return lib.ieo_run_program_dump(C.byref(params), str(results_dir).encode(), str(inputs_dir).encode(),
                                        None if dump_dir is None else str(dump_dir).encode())
    finally:
        lib.ieo_set_engine_arith_default(0)


def read_state(path: Path) -> dict:
    """Reads a state.bin written by the oracle or by oracle/ref_driver.cpp."""
    raw = Path(path).read_bytes()
    N, dn, sigw, _num = (int(x) for x in np.frombuffer(raw[:16], dtype=np.int32))
    off = 16
    out = {"scalars": np.frombuffer(raw[off:off + 64], dtype=np.float64).copy()}
    off += 64
    gs = N ** 3
    for name in ("f", "fd") + (("deltaN",) if dn else ()):
        out[name] = np.frombuffer(raw[off:off + 8 * gs], dtype=np.float64).copy()
        off += 8 * gs
    if sigw:
        out["h"] = np.frombuffer(raw[off:off + 24 * gs], dtype=np.float32).reshape(6, gs).copy()
        off += 24 * gs
        out["hd"] = np.frombuffer(raw[off:off + 24 * gs], dtype=np.float32).reshape(6, gs).copy()
    return out


def params_from_text(text: str, N: int, numerical: bool, sigw: bool, deltaN: bool = True,
                     post: bool = False) -> Params:
    """Params for a params.txt body, with the compile-time switches given."""
    kw = {}
    for line in text.splitlines():
        line = line.split("#", 1)[0].strip()
        if "=" not in line:
            continue
        k, v = (x.strip() for x in line.split("=", 1))
        if k in ("output_bispectrum", "output_LOG"):
            continue
        if k.endswith("_integrator"):
            kw[k] = {"leapfrog": 0, "lf": 0, "rk4": 1, "rk45": 2, "rkf45": 2, "dopri5": 2}.get(v.lower(), 0)
            continue
        kw[k] = float(v) if any(ch in v for ch in ".eE") else int(v)
    kw["calculate_SIGW"] = int(sigw)
    kw["perform_deltaN"] = int(deltaN)
    kw["post_inflation"] = int(post)
    return default_params(N, numerical, **kw)
