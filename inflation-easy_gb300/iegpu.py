"""ctypes binding of the C ABI in include/iegpu.h (libiegpu.so).

This is the Python face of the drop-in boundary: the same calls a C/C++ host
makes (see ie_gpu_main in host/), with numpy arrays in the reference layout
(N^3, index (i*N + j)*N + k).  There is no CPU fallback: importing this module
without a built libiegpu.so raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libiegpu.so"

OK, EINVAL, ECUDA, ERANGE, ENAN, ECOURANT, ENOMEM, ETABLE, EUNSUPPORTED, ETIMEOUT, ETOOBIG, ECONVERGE = range(12)
POT_HILLTOP, POT_TABLE = 0, 1
FORM_FP64, FORM_SPLIT, FORM_SPLIT_COMP = 0, 1, 2
CRIT_GENERIC, CRIT_MONOTONIC, CRIT_ANTIMONOTONIC = 0, 1, -1
F, FD, DELTAN = 0, 1, 2


def H(c: int) -> int:
    return 8 + c


def HD(c: int) -> int:
    return 16 + c


class Config(C.Structure):
    _fields_ = [("N", C.c_int), ("potential", C.c_int), ("sigw", C.c_int), ("form", C.c_int),
                ("criterion", C.c_int), ("L", C.c_double), ("dt", C.c_double), ("rescale_s", C.c_double),
                ("rescale_B", C.c_double), ("V0", C.c_double), ("ns", C.c_double)]


class Rk45Controls(C.Structure):
    """iegpu_rk45_controls: the reference's rk45_* keys (non-positive min/max
    steps and out-of-range values take the reference's defaults)."""
    _fields_ = [("abs_tol", C.c_double), ("rel_tol", C.c_double), ("min_dt", C.c_double),
                ("max_dt", C.c_double), ("safety", C.c_double)]

    def __init__(self, abs_tol=1e-8, rel_tol=1e-6, min_dt=-1.0, max_dt=-1.0, safety=0.9):
        super().__init__(abs_tol, rel_tol, min_dt, max_dt, safety)


class Bg(C.Structure):
    _fields_ = [("t", C.c_double), ("a", C.c_double), ("ad", C.c_double), ("ad2", C.c_double),
                ("astep", C.c_double)]

    def as_tuple(self):
        return (self.t, self.a, self.ad, self.ad2, self.astep)


class IegpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"iegpu error {code}: {msg}")
        self.code = code


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise FileNotFoundError(f"{LIB_PATH} is not built; run __graft_entry__.build()")
    lib = C.CDLL(str(LIB_PATH))
    P, I, D = C.c_void_p, C.c_int, C.c_double
    dp, ip, fp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_float)
    sig = {
        "iegpu_version": (I, []),
        "iegpu_strerror": (C.c_char_p, [I]),
        "iegpu_create": (I, [C.POINTER(Config), C.POINTER(P)]),
        "iegpu_destroy": (I, [P]),
        "iegpu_last_error": (C.c_char_p, [P]),
        "iegpu_stream": (P, [P]),
        "iegpu_launch_count": (C.c_longlong, [P]),
        "iegpu_set_table": (I, [P, dp, dp, dp, I]),
        "iegpu_upload": (I, [P, I, P, P]),
        "iegpu_download": (I, [P, I, P, P]),
        "iegpu_add": (I, [P, I, D]),
        "iegpu_evolve_fields": (I, [P, D, C.POINTER(Bg)]),
        "iegpu_evolve_derivs": (I, [P, D, C.POINTER(Bg)]),
        "iegpu_leapfrog": (I, [P, D, I, C.POINTER(Bg), ip, dp]),
        "iegpu_rk4_step_inflation": (I, [P, D, C.POINTER(Bg)]),
        "iegpu_rk4": (I, [P, D, I, C.POINTER(Bg), ip, dp]),
        "iegpu_rk45_effective": (I, [C.POINTER(Rk45Controls), D, C.POINTER(Rk45Controls)]),
        "iegpu_rk45_step_inflation": (I, [P, C.POINTER(Rk45Controls), D, D, dp, ip, C.POINTER(Bg)]),
        "iegpu_rk45": (I, [P, C.POINTER(Rk45Controls), D, I, dp, C.POINTER(Bg), ip, dp]),
        "iegpu_deltaN_rk4_steps": (I, [P, D, I, D, C.POINTER(Bg)]),
        "iegpu_deltaN_rk45": (I, [P, C.POINTER(Rk45Controls), D, D, I, D, dp, dp, C.POINTER(Bg), ip, dp]),
        "iegpu_post_inflation_rk4": (I, [P, D, D, D, I, C.POINTER(Bg), ip, dp]),
        "iegpu_post_inflation_rk45": (I, [P, C.POINTER(Rk45Controls), D, D, D, I, dp, C.POINTER(Bg), ip, dp]),
        "iegpu_energies": (I, [P, C.POINTER(Bg), dp]),
        "iegpu_means": (I, [P, dp]),
        "iegpu_bunch_davies": (I, [P, I, D, D, D, D, dp]),
        "iegpu_autotune": (I, [P, C.POINTER(Bg), ip, ip, ip]),
        "iegpu_timer_start": (I, [P]),
        "iegpu_timer_stop": (I, [P, C.POINTER(C.c_float)]),
        "iegpu_profile_leapfrog": (I, [P, D, I, C.POINTER(Bg), dp, I]),
        "iegpu_histogram": (I, [P, I, I, dp, dp, dp]),
        "iegpu_fft": (I, [P, I, I]),
        "iegpu_numbins": (I, [I]),
        "iegpu_spectrum": (I, [P, I, ip, dp, I]),
        "iegpu_spectrum_cutoff": (I, [P, ip, dp, I, D, D]),
        "iegpu_gw_spectrum": (I, [P, I, D, ip, dp, I]),
        "iegpu_gw_spectrum_ref": (I, [P, I, D, ip, C.POINTER(C.c_float), dp, I]),
        "iegpu_initializeN": (I, [P, D]),
        "iegpu_get_phiref": (I, [P, dp]),
        "iegpu_evolve_fieldsN": (I, [P, D, D]),
        "iegpu_evolve_derivsN": (I, [P, D]),
        "iegpu_deltaN_steps": (I, [P, D, I, D]),
        "iegpu_saveN_mean": (I, [P, D, fp]),
        "iegpu_shift": (I, [P, I, D]),
        "iegpu_zero_above": (I, [P, I, D]),
        "iegpu_sum": (I, [P, I, dp]),
        "iegpu_shell_spectrum_noalloc": (I, [P, P, I, P, P, P]),
        "iegpu_set_shape": (I, [P, I, I, I]),
        "iegpu_set_persistent": (I, [P, I]),
        "iegpu_set_wait_limit": (I, [P, C.c_uint, I]),
        "iegpu_measure_fp64_rate": (I, [I, dp]),
        "iegpu_initialize_post_inflation": (I, [P, D, D, I, C.POINTER(Bg)]),
        "iegpu_evolve_derivs_post_inflation": (I, [P, D, D, C.POINTER(Bg)]),
        "iegpu_post_inflation_leapfrog": (I, [P, D, D, D, I, C.POINTER(Bg), C.POINTER(I), dp]),
        "iegpu_ens_create": (I, [C.POINTER(Config), ip, I, C.POINTER(P)]),
        "iegpu_ens_destroy": (I, [P]),
        "iegpu_ens_last_error": (C.c_char_p, [P]),
        "iegpu_ens_launch_count": (C.c_longlong, [P]),
        "iegpu_ens_stream": (P, [P]),
        "iegpu_ens_set_table": (I, [P, dp, dp, dp, I]),
        "iegpu_ens_bunch_davies": (I, [P, ip, D, D, D, D, dp]),
        "iegpu_ens_evolve_fields": (I, [P, dp, P]),
        "iegpu_ens_leapfrog": (I, [P, dp, I, P, ip]),
        "iegpu_ens_profile": (I, [P, I, P, dp, dp]),
        "iegpu_ens_autotune": (I, [P, P, ip, ip, ip]),
        "iegpu_ens_shapes": (I, [P, ip, ip, ip]),
        "iegpu_ens_set_shape": (I, [P, I, I, I, I]),
        "iegpu_ens_set_persistent": (I, [P, I]),
        "iegpu_ens_timer_start": (I, [P]),
        "iegpu_ens_timer_stop": (I, [P, C.POINTER(C.c_float)]),
        "iegpu_ens_download": (I, [P, I, I, dp]),
        "iegpu_ens_deltaN": (I, [P, P, D, D, I, D, dp, fp]),
        "iegpu_ens_zeta_spectra": (I, [P, ip, dp]),
        "iegpu_ens_zeta_histogram": (I, [P, I, I, D, dp, dp, dp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _ptr(a: np.ndarray, dtype) -> C.c_void_p:
    assert a.dtype == dtype and a.flags["C_CONTIGUOUS"], (a.dtype, dtype)
    return C.c_void_p(a.ctypes.data)


class Lattice:
    """One device lattice (an iegpu context)."""

    def __init__(self, N: int, L: float, dt: float, V0: float, ns: float = 0.97, rescale_B: float | None = None,
                 rescale_s: float = 0.0, potential: int = POT_HILLTOP, sigw: bool = False, form: int = FORM_FP64,
                 criterion: int | None = None):
        self.lib = load()
        if rescale_B is None:
            rescale_B = float(np.sqrt(V0))
        if criterion is None:
            criterion = CRIT_MONOTONIC if potential == POT_TABLE else CRIT_ANTIMONOTONIC
        self.cfg = Config(N, potential, int(bool(sigw)), form, criterion, L, dt, rescale_s, rescale_B, V0, ns)
        self.N = N
        self.sigw = bool(sigw)
        h = C.c_void_p()
        rc = self.lib.iegpu_create(C.byref(self.cfg), C.byref(h))
        if rc != OK:
            raise IegpuError(rc, self.lib.iegpu_strerror(rc).decode())
        self.h = h

    # -- plumbing ---------------------------------------------------------
    def _check(self, rc: int) -> None:
        if rc != OK:
            raise IegpuError(rc, self.lib.iegpu_last_error(self.h).decode())

    def close(self) -> None:
        if self.h:
            self.lib.iegpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def stream(self) -> int:
        return self.lib.iegpu_stream(self.h) or 0

    @property
    def launches(self) -> int:
        return self.lib.iegpu_launch_count(self.h)

    # -- state ------------------------------------------------------------
    def set_table(self, phi: np.ndarray, V: np.ndarray, dV: np.ndarray) -> None:
        phi, V, dV = (np.ascontiguousarray(x, dtype=np.float64) for x in (phi, V, dV))
        dp = C.POINTER(C.c_double)
        self._check(self.lib.iegpu_set_table(self.h, phi.ctypes.data_as(dp), V.ctypes.data_as(dp),
                                             dV.ctypes.data_as(dp), len(phi)))

    def upload(self, field: int, host: np.ndarray, nyquist: np.ndarray | None = None) -> None:
        dt = np.float64 if field in (F, FD, DELTAN) else np.float32
        host = np.ascontiguousarray(host, dtype=dt)
        ny = None if nyquist is None else np.ascontiguousarray(nyquist, dtype=dt)
        self._check(self.lib.iegpu_upload(self.h, field, _ptr(host, dt), None if ny is None else _ptr(ny, dt)))

    def download(self, field: int, nyquist: bool = False, out: np.ndarray | None = None):
        """The field as a host array; `out` (contiguous, N^3 elements of the
        field's type) is filled and returned instead of a new array."""
        dt = np.float64 if field in (F, FD, DELTAN) else np.float32
        if out is None:
            out = np.empty(self.N ** 3, dtype=dt)
        elif out.dtype != dt or out.size != self.N ** 3 or not out.flags["C_CONTIGUOUS"]:
            raise ValueError(f"out must be a contiguous {dt.__name__} array of {self.N ** 3} elements")
        ny = np.empty(2 * self.N * self.N, dtype=dt) if nyquist else None
        self._check(self.lib.iegpu_download(self.h, field, _ptr(out, dt), None if ny is None else _ptr(ny, dt)))
        return (out, ny) if nyquist else out

    def add(self, field: int, value: float) -> None:
        self._check(self.lib.iegpu_add(self.h, field, value))

    # -- initial conditions -----------------------------------------------
    def bunch_davies(self, seed: int, phi0: float, dphi0: float, high_cut: float = 0.0, low_cut: float = 0.0) -> float:
        h = C.c_double()
        self._check(self.lib.iegpu_bunch_davies(self.h, seed, phi0, dphi0, high_cut, low_cut, C.byref(h)))
        return h.value

    # -- leapfrog ---------------------------------------------------------
    def evolve_fields(self, d: float, bg: Bg) -> None:
        self._check(self.lib.iegpu_evolve_fields(self.h, d, C.byref(bg)))

    def evolve_derivs(self, d: float, bg: Bg) -> None:
        self._check(self.lib.iegpu_evolve_derivs(self.h, d, C.byref(bg)))

    def leapfrog(self, af: float, max_steps: int, bg: Bg, trace: bool = False):
        steps = C.c_int(0)
        tr = np.zeros(max(1, max_steps), dtype=np.float64) if trace else None
        self._check(self.lib.iegpu_leapfrog(self.h, af, max_steps, C.byref(bg), C.byref(steps),
                                            None if tr is None else tr.ctypes.data_as(C.POINTER(C.c_double))))
        return (steps.value, tr[:steps.value]) if trace else steps.value

    def rk4_step_inflation(self, h: float, bg: Bg) -> None:
        self._check(self.lib.iegpu_rk4_step_inflation(self.h, h, C.byref(bg)))

    def rk4(self, af: float, max_steps: int, bg: Bg, trace: bool = False):
        steps = C.c_int(0)
        tr = np.zeros(max(1, max_steps), dtype=np.float64) if trace else None
        self._check(self.lib.iegpu_rk4(self.h, af, max_steps, C.byref(bg), C.byref(steps),
                                       None if tr is None else tr.ctypes.data_as(C.POINTER(C.c_double))))
        return (steps.value, tr[:steps.value]) if trace else steps.value

    def rk45_step_inflation(self, h: float, hmax: float, bg: Bg, controls: "Rk45Controls | None" = None):
        """One RK45 attempt: (accepted, h_next)."""
        hn, acc = C.c_double(h), C.c_int(0)
        self._check(self.lib.iegpu_rk45_step_inflation(self.h, C.byref(controls or Rk45Controls()), h, hmax,
                                                       C.byref(hn), C.byref(acc), C.byref(bg)))
        return bool(acc.value), hn.value

    def rk45(self, af: float, max_steps: int, bg: Bg, h: float, controls: "Rk45Controls | None" = None,
             trace: bool = False):
        """RK45 steps while a <= af: (steps, h carried to the next call[, a trace])."""
        steps, hh = C.c_int(0), C.c_double(h)
        tr = np.zeros(max(1, max_steps), dtype=np.float64) if trace else None
        self._check(self.lib.iegpu_rk45(self.h, C.byref(controls or Rk45Controls()), af, max_steps, C.byref(hh),
                                        C.byref(bg), C.byref(steps),
                                        None if tr is None else tr.ctypes.data_as(C.POINTER(C.c_double))))
        return (steps.value, hh.value, tr[:steps.value]) if trace else (steps.value, hh.value)

    def energies(self, bg: Bg):
        out = (C.c_double * 3)()
        self._check(self.lib.iegpu_energies(self.h, C.byref(bg), out))
        return tuple(out)

    # -- measurement ------------------------------------------------------
    def set_shape(self, rows: int, prefetch: int, chunks: int) -> None:
        self._check(self.lib.iegpu_set_shape(self.h, rows, prefetch, chunks))

    # -- post-inflation phase (plain FP64 form, SIGW on) ------------------
    def initialize_post_inflation(self, bg: Bg, horizon_factor: float = 1.0, omega: float = 1.0 / 3.0,
                                  from_deltaN: bool = True) -> None:
        self._check(self.lib.iegpu_initialize_post_inflation(self.h, horizon_factor, omega, int(from_deltaN),
                                                             C.byref(bg)))

    def evolve_derivs_post_inflation(self, d: float, bg: Bg, omega: float = 1.0 / 3.0) -> None:
        self._check(self.lib.iegpu_evolve_derivs_post_inflation(self.h, d, omega, C.byref(bg)))

    def post_inflation_leapfrog(self, af_post: float, dt_post: float, max_steps: int, bg: Bg,
                                omega: float = 1.0 / 3.0, trace: bool = False):
        steps = C.c_int(0)
        tr = np.zeros(max(1, max_steps), dtype=np.float64) if trace else None
        self._check(self.lib.iegpu_post_inflation_leapfrog(self.h, af_post, dt_post, omega, max_steps, C.byref(bg),
                                                           C.byref(steps),
                                                           None if tr is None else tr.ctypes.data_as(C.POINTER(C.c_double))))
        return (steps.value, tr[:steps.value]) if trace else steps.value

    def post_inflation_rk4(self, af_post: float, dt_post: float, max_steps: int, bg: Bg,
                           omega: float = 1.0 / 3.0) -> int:
        steps = C.c_int(0)
        self._check(self.lib.iegpu_post_inflation_rk4(self.h, af_post, dt_post, omega, max_steps, C.byref(bg),
                                                      C.byref(steps), None))
        return steps.value

    def post_inflation_rk45(self, af_post: float, dt_post: float, max_steps: int, bg: Bg, h: float,
                            omega: float = 1.0 / 3.0, controls: "Rk45Controls | None" = None):
        """(steps, h carried to the next call)."""
        steps, hh = C.c_int(0), C.c_double(h)
        self._check(self.lib.iegpu_post_inflation_rk45(self.h, C.byref(controls or Rk45Controls()), af_post, dt_post,
                                                       omega, max_steps, C.byref(hh), C.byref(bg), C.byref(steps),
                                                       None))
        return steps.value, hh.value

    def set_persistent(self, on: bool) -> None:
        self._check(self.lib.iegpu_set_persistent(self.h, int(bool(on))))

    def set_wait_limit(self, polls: int, unreachable: bool = False) -> None:
        """Poll limit of the split form's bounded device waits (0: default);
        unreachable makes the persistent step barrier give up (tests)."""
        self._check(self.lib.iegpu_set_wait_limit(self.h, polls, int(unreachable)))

    def autotune(self, bg: Bg):
        r, p, ch = C.c_int(), C.c_int(), C.c_int()
        self._check(self.lib.iegpu_autotune(self.h, C.byref(bg), C.byref(r), C.byref(p), C.byref(ch)))
        return {"rows": r.value, "prefetch": p.value, "chunks": ch.value}

    def timer_start(self) -> None:
        self._check(self.lib.iegpu_timer_start(self.h))

    def timer_stop(self) -> float:
        ms = C.c_float()
        self._check(self.lib.iegpu_timer_stop(self.h, C.byref(ms)))
        return ms.value

    def profile_leapfrog(self, af: float, nsteps: int, bg: Bg):
        ms = (C.c_double * 2)()
        self._check(self.lib.iegpu_profile_leapfrog(self.h, af, nsteps, C.byref(bg), ms, 2))
        return tuple(ms)

    # -- diagnostics ------------------------------------------------------
    def means(self):
        out = (C.c_double * 3)()
        self._check(self.lib.iegpu_means(self.h, out))
        return tuple(out)

    def histogram(self, field: int, nbins: int):
        bmin, df = C.c_double(), C.c_double()
        freq = np.zeros(nbins, dtype=np.float64)
        self._check(self.lib.iegpu_histogram(self.h, field, nbins, C.byref(bmin), C.byref(df),
                                             freq.ctypes.data_as(C.POINTER(C.c_double))))
        return bmin.value, df.value, freq

    def fft(self, field: int, forward: int) -> None:
        self._check(self.lib.iegpu_fft(self.h, field, forward))

    def numbins(self) -> int:
        return self.lib.iegpu_numbins(self.N)

    def spectrum(self, field: int):
        nb = self.numbins()
        counts = np.zeros(nb, dtype=np.int32)
        f2 = np.zeros(nb, dtype=np.float64)
        self._check(self.lib.iegpu_spectrum(self.h, field, counts.ctypes.data_as(C.POINTER(C.c_int)),
                                            f2.ctypes.data_as(C.POINTER(C.c_double)), nb))
        return counts, f2

    def spectrum_cutoff(self, high_cutoff: float, low_cutoff: float = 0.0):
        """spectraf() with the forcing cutoff: f's spectrum, then f's and fd's
        modes outside [low_cutoff, high_cutoff] zeroed (high_cutoff > 0)."""
        nb = self.numbins()
        counts = np.zeros(nb, dtype=np.int32)
        f2 = np.zeros(nb, dtype=np.float64)
        self._check(self.lib.iegpu_spectrum_cutoff(self.h, counts.ctypes.data_as(C.POINTER(C.c_int)),
                                                   f2.ctypes.data_as(C.POINTER(C.c_double)), nb, high_cutoff,
                                                   low_cutoff))
        return counts, f2

    def gw_spectrum(self, which: int, to_phys: float = 1.0):
        nb = self.numbins()
        counts = np.zeros(nb, dtype=np.int32)
        f2 = np.zeros(nb, dtype=np.float64)
        self._check(self.lib.iegpu_gw_spectrum(self.h, which, to_phys, counts.ctypes.data_as(C.POINTER(C.c_int)),
                                               f2.ctypes.data_as(C.POINTER(C.c_double)), nb))
        return counts, f2

    def gw_spectrum_ref(self, which: int, to_phys: float = 1.0):
        """(counts, f2 float32, f2 float64): the reference's float accumulators
        (its loop order) and the same values summed in double (another order)."""
        nb = self.numbins()
        counts = np.zeros(nb, dtype=np.int32)
        f2 = np.zeros(nb, dtype=np.float32)
        f2d = np.zeros(nb, dtype=np.float64)
        self._check(self.lib.iegpu_gw_spectrum_ref(self.h, which, to_phys, counts.ctypes.data_as(C.POINTER(C.c_int)),
                                                   f2.ctypes.data_as(C.POINTER(C.c_float)),
                                                   f2d.ctypes.data_as(C.POINTER(C.c_double)), nb))
        return counts, f2, f2d

    # -- deltaN -----------------------------------------------------------
    def initializeN(self, a: float) -> None:
        self._check(self.lib.iegpu_initializeN(self.h, a))

    def get_phiref(self) -> float:
        v = C.c_double()
        self._check(self.lib.iegpu_get_phiref(self.h, C.byref(v)))
        return v.value

    def evolve_fieldsN(self, d: float, phiref: float) -> None:
        self._check(self.lib.iegpu_evolve_fieldsN(self.h, d, phiref))

    def evolve_derivsN(self, d: float) -> None:
        self._check(self.lib.iegpu_evolve_derivsN(self.h, d))

    def deltaN_rk4_steps(self, dN: float, nsteps: int, phiref: float, bg: Bg) -> None:
        """nsteps of rk4_step_deltaN; bg.a and bg.t advance, Ne is the caller's."""
        self._check(self.lib.iegpu_deltaN_rk4_steps(self.h, dN, nsteps, phiref, C.byref(bg)))

    def deltaN_rk45(self, dN: float, Nend: float, max_steps: int, phiref: float, h: float, Ne: float, bg: Bg,
                    controls: "Rk45Controls | None" = None):
        """The RK45 deltaN loop: (steps, h carried, Ne)."""
        hh, ne, steps = C.c_double(h), C.c_double(Ne), C.c_int(0)
        self._check(self.lib.iegpu_deltaN_rk45(self.h, C.byref(controls or Rk45Controls()), dN, Nend, max_steps,
                                               phiref, C.byref(hh), C.byref(ne), C.byref(bg), C.byref(steps), None))
        return steps.value, hh.value, ne.value

    def deltaN_steps(self, dN: float, nsteps: int, phiref: float) -> None:
        self._check(self.lib.iegpu_deltaN_steps(self.h, dN, nsteps, phiref))

    def saveN_mean(self, cutoff: float) -> float:
        v = C.c_float()
        self._check(self.lib.iegpu_saveN_mean(self.h, cutoff, C.byref(v)))
        return v.value

    def shift(self, field: int, value: float) -> None:
        self._check(self.lib.iegpu_shift(self.h, field, value))

    def zero_above(self, field: int, thr: float) -> None:
        self._check(self.lib.iegpu_zero_above(self.h, field, thr))

    def sum(self, field: int) -> float:
        v = C.c_double()
        self._check(self.lib.iegpu_sum(self.h, field, C.byref(v)))
        return v.value


def measure_fp64_rate(op: int) -> float:
    """FP64 thread instructions per second of the current device (op 0: DFMA,
    1: DADD, 2: DMUL)."""
    out = C.c_double()
    rc = load().iegpu_measure_fp64_rate(op, C.byref(out))
    if rc:
        raise IegpuError(rc, "FP64 rate probe failed")
    return out.value


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class Ensemble:
    """Many independent lattices evolved together in the split form (an
    iegpu_ens).  `Ns` gives each lattice's size; per-lattice values (seeds,
    af, background scalars) are arrays indexed by lattice."""

    def __init__(self, Ns, L: float, dt: float, V0: float, ns: float = 0.97, rescale_B: float | None = None,
                 rescale_s: float = 0.0, potential: int = POT_HILLTOP, criterion: int | None = None):
        self.lib = load()
        if rescale_B is None:
            rescale_B = float(np.sqrt(V0))
        if criterion is None:
            criterion = CRIT_MONOTONIC if potential == POT_TABLE else CRIT_ANTIMONOTONIC
        self.cfg = Config(0, potential, 0, FORM_SPLIT, criterion, L, dt, rescale_s, rescale_B, V0, ns)
        self.Ns = np.ascontiguousarray(Ns, dtype=np.int32)
        self.count = len(self.Ns)
        h = C.c_void_p()
        rc = self.lib.iegpu_ens_create(C.byref(self.cfg), _ip(self.Ns), self.count, C.byref(h))
        if rc != OK:
            raise IegpuError(rc, self.lib.iegpu_strerror(rc).decode())
        self.h = h

    def _check(self, rc: int) -> None:
        if rc != OK:
            raise IegpuError(rc, self.lib.iegpu_ens_last_error(self.h).decode())

    def close(self) -> None:
        if self.h:
            self.lib.iegpu_ens_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def launches(self) -> int:
        return self.lib.iegpu_ens_launch_count(self.h)

    def bgs(self, hubble) -> C.Array:
        """Background scalars of every lattice at the start: t = 0, a = 1, ad = H."""
        b = (Bg * self.count)()
        for q, hq in enumerate(hubble):
            b[q] = Bg(0.0, 1.0, float(hq), 0.0, 1.0)
        return b

    def set_table(self, phi, V, dV) -> None:
        phi, V, dV = (np.ascontiguousarray(x, dtype=np.float64) for x in (phi, V, dV))
        self._check(self.lib.iegpu_ens_set_table(self.h, _dp(phi), _dp(V), _dp(dV), len(phi)))

    def bunch_davies(self, seeds, phi0: float, dphi0: float, high_cut: float = 0.0, low_cut: float = 0.0):
        seeds = np.ascontiguousarray(seeds, dtype=np.int32)
        hub = np.zeros(self.count)
        self._check(self.lib.iegpu_ens_bunch_davies(self.h, _ip(seeds), phi0, dphi0, high_cut, low_cut, _dp(hub)))
        return hub

    def evolve_fields(self, d, bg) -> None:
        d = np.ascontiguousarray(np.broadcast_to(d, (self.count,)), dtype=np.float64)
        self._check(self.lib.iegpu_ens_evolve_fields(self.h, _dp(d), bg))

    def leapfrog(self, af, max_steps: int, bg):
        af = np.ascontiguousarray(np.broadcast_to(af, (self.count,)), dtype=np.float64)
        steps = np.zeros(self.count, dtype=np.int32)
        self._check(self.lib.iegpu_ens_leapfrog(self.h, _dp(af), max_steps, bg, _ip(steps)))
        return steps

    def profile(self, nsteps: int, bg):
        a, b = C.c_double(), C.c_double()
        self._check(self.lib.iegpu_ens_profile(self.h, nsteps, bg, C.byref(a), C.byref(b)))
        return a.value, b.value

    def autotune(self, bg):
        """Per lattice: rows per tile (N: whole planes), planes prefetched, plane chunks."""
        r, p, ch = (np.zeros(self.count, dtype=np.int32) for _ in range(3))
        self._check(self.lib.iegpu_ens_autotune(self.h, bg, _ip(r), _ip(p), _ip(ch)))
        return {"rows": r, "prefetch": p, "chunks": ch}

    def shapes(self):
        """The current launch shape of each lattice's size class, as autotune() returns it."""
        r, p, ch = (np.zeros(self.count, dtype=np.int32) for _ in range(3))
        self._check(self.lib.iegpu_ens_shapes(self.h, _ip(r), _ip(p), _ip(ch)))
        return {"rows": r, "prefetch": p, "chunks": ch}

    def set_shape(self, N: int, rows: int, prefetch: int, chunks: int) -> None:
        self._check(self.lib.iegpu_ens_set_shape(self.h, N, rows, prefetch, chunks))

    def set_persistent(self, on: bool) -> None:
        """One cooperative launch of up to 64 steps over a queue of every
        lattice's tiles (on), or one kernel per size and step (off)."""
        self._check(self.lib.iegpu_ens_set_persistent(self.h, 1 if on else 0))

    def timer_start(self) -> None:
        self._check(self.lib.iegpu_ens_timer_start(self.h))

    def timer_stop(self) -> float:
        ms = C.c_float()
        self._check(self.lib.iegpu_ens_timer_stop(self.h, C.byref(ms)))
        return ms.value

    def download(self, lattice: int, field: int) -> np.ndarray:
        out = np.empty(int(self.Ns[lattice]) ** 3, dtype=np.float64)
        self._check(self.lib.iegpu_ens_download(self.h, lattice, field, _dp(out)))
        return out

    def deltaN(self, bg, dN: float, Nend: float, phiref_manual: float | None = None):
        phiref = np.zeros(self.count)
        nmean = np.zeros(self.count, dtype=np.float32)
        self._check(self.lib.iegpu_ens_deltaN(self.h, bg, dN, Nend, int(phiref_manual is not None),
                                              0.0 if phiref_manual is None else phiref_manual, _dp(phiref),
                                              nmean.ctypes.data_as(C.POINTER(C.c_float))))
        return phiref, nmean

    def zeta_spectra(self):
        """[(counts, f2)] per lattice, as iegpu_spectrum of that lattice's zeta (spectraN)."""
        nbs = [self.lib.iegpu_numbins(int(n)) for n in self.Ns]
        tot = int(sum(nbs))
        counts = np.zeros(tot, dtype=np.int32)
        f2 = np.zeros(tot)
        self._check(self.lib.iegpu_ens_zeta_spectra(self.h, _ip(counts), _dp(f2)))
        out, at = [], 0
        for nb in nbs:
            out.append((counts[at:at + nb], f2[at:at + nb]))
            at += nb
        return out

    def zeta_histogram(self, N: int = 0, nbins: int = 200, nsigma: float = 10.0):
        sigma, lo, width = C.c_double(), C.c_double(), C.c_double()
        counts = np.zeros(nbins, dtype=np.int64)
        outside = np.zeros(2, dtype=np.int64)
        ll = C.POINTER(C.c_longlong)
        self._check(self.lib.iegpu_ens_zeta_histogram(self.h, N, nbins, nsigma, C.byref(sigma), C.byref(lo),
                                                      C.byref(width), counts.ctypes.data_as(ll),
                                                      outside.ctypes.data_as(ll)))
        return {"sigma": sigma.value, "lo": lo.value, "width": width.value, "counts": counts, "outside": outside}
