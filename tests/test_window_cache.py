"""The split step's table-window lookups on the CPU: the bracket search over
the window (walk and branch-free forms) and the register caches of the
background's bracket with one or two neighbours either side
(inflation-easy_gb300/csrc/split_window.cuh), against a search over the whole
window, bit for bit (tests/native/window_cache_check.cu, built with nvcc)."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

HERE = Path(__file__).resolve().parent
CSRC = ROOT / "inflation-easy_gb300" / "csrc"


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    exe = tmp_path_factory.mktemp("window") / "window_cache_check"
    subprocess.check_call([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off", f"-I{CSRC}",
                           f"-I{ROOT / 'include'}", str(HERE / "native" / "window_cache_check.cu"), "-o", str(exe)])
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_window_lookups_match_a_full_search(checker, seed):
    out = subprocess.run([str(checker), str(seed), "3000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    words = out.stdout.split()
    assert int(words[1]) > 1_000_000, out.stdout
    assert words[-1] == "0", out.stdout
