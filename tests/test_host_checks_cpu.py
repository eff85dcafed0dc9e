"""Host-side checks of the library's C++ code that need no GPU: compiled here with the
system C++ compiler against the library's internal header and run."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "cdlmotif.jl_gb300", "csrc")
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


def _build_and_run(src, tmp_path):
    cxx = shutil.which("g++")
    if cxx is None or not os.path.isfile(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers are missing")
    exe = str(tmp_path / "check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", CSRC, "-I", os.path.join(ROOT, "include"),
                    "-I", CUDA_INC, src, "-o", exe], check=True, capture_output=True, text=True)
    return subprocess.run([exe], capture_output=True, text=True, timeout=60)


def test_position_checks_match_per_entry_conditions(tmp_path):
    r = _build_and_run(os.path.join(ROOT, "tests", "host", "position_checks.cpp"), tmp_path)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
