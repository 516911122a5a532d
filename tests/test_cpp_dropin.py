"""The C++ drop-in header compiles against the reference's own headers, wins overload
resolution for CUDA memory views, and maps argument errors to std::invalid_argument.

Needs the reference checkout (its headers), so it runs where that checkout exists and is
skipped elsewhere."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import pytest

from oracle import build as oracle_build

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.skipif(oracle_build.reference_root() is None, reason="reference headers not present")
def test_dropin_compiles_and_dispatches(tmp_path):
    from iane_gb300 import build as lib_build

    lib = lib_build.build()
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "dropin_check"
    cmd = [nvcc, "-std=c++20", "--expt-extended-lambda", "--expt-relaxed-constexpr",
           "-gencode", "arch=compute_103a,code=sm_103a", "-I", str(oracle_build.reference_root() / "include"),
           "-I", str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "dropin_check.cu"), "-o", str(exe),
           "-L", str(lib.parent), "-liane_gb300", f"-Xlinker=-rpath={lib.parent}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-4000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, env=dict(os.environ), timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "ok   even kernel extent" in run.stdout and "ok   mismatched extents" in run.stdout
