"""Build recipe of the GB300 engine: libiegpu.so (CUDA, sm_103a) and the host
program ie_gpu_main.  Everything is built in-tree into inflation-easy_gb300/_build/.

The translation units that must reproduce the reference's per-site arithmetic
bit for bit are compiled with -fmad=false; host code everywhere gets
-ffp-contract=off so that the host-side scalar arithmetic (twiddle tables,
background scalars) does not fuse multiply-adds on the Arm host either.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
BUILD = PKG / "_build"
LIB = BUILD / "libiegpu.so"
MAIN = BUILD / "ie_gpu_main"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                 f"-I{ROOT / 'include'}", f"-I{CSRC}"]

# translation unit -> extra flags
UNITS = {
    "ctx.cu": ["-fmad=false"],
    "leapfrog_fp64.cu": ["-fmad=false"],
    "fft.cu": ["-fmad=false"],
    "spectra.cu": ["-fmad=false"],
    "deltaN.cu": ["-fmad=false"],
    "reduce_ops.cu": ["-fmad=false"],
    "ic.cu": ["-fmad=false"],
    "split_fp32.cu": [],
    "split_rows4_128.cu": [],
    "split_rows4_256.cu": [],
    "split_rows4_512.cu": [],
    "ensemble.cu": [],
    "ensemble_dn.cu": ["-fmad=false"],
    "measure.cu": [],
}


def nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = Path("/usr/local/cuda/bin/nvcc")
    if cand.exists():
        return str(cand)
    raise FileNotFoundError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [ROOT / "include" / "iegpu.h", Path(__file__)]
    nv = nvcc()
    jobs = []
    objs = []
    for unit, extra in UNITS.items():
        src = CSRC / unit
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, [src, *headers]):
            jobs.append([nv, *COMMON, *extra, "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    if jobs or _stale(LIB, objs):
        _run([nv, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)])
    host_srcs = sorted(HOST.glob("*.cpp")) if HOST.exists() else []
    if host_srcs and (_stale(MAIN, host_srcs + [LIB, ROOT / "include" / "iegpu.h"])):
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{ROOT / 'include'}", *map(str, host_srcs),
              "-o", str(MAIN), f"-L{BUILD}", "-liegpu", f"-Wl,-rpath,{BUILD}", "-lm"])
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
