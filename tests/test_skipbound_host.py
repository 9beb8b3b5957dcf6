"""Host-side bounds of the TF/SF skip test (dgtd_gb300/csrc/skipbound.hpp), checked on the CPU
against the exact sum the reference evaluates (GlobalEvolution.cpp:587-598) for random node
clouds, plane waves and stage times: every decision the bounds make must agree with it."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_skip_bound_decisions_agree_with_exact_sum(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cuda_inc = Path("/usr/local/cuda/include")
    if not (cuda_inc / "cuda_runtime.h").exists():
        pytest.skip("no CUDA headers")
    exe = tmp_path / "skipbound_check"
    cmd = [cxx, "-O2", "-std=c++17", "-I", str(ROOT / "dgtd_gb300" / "csrc"), "-I", str(cuda_inc),
           str(ROOT / "tests" / "host" / "skipbound_check.cpp"), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    decided, undecided, wrong = (int(v) for v in out.stdout.split()[1::2])
    assert wrong == 0 and decided > 10 * undecided, out.stdout
