"""Build ``iane_gb300/libiane_gb300.so`` from ``csrc/*.cu`` for sm_103a with nvcc.

Each translation unit is compiled in parallel into ``iane_gb300/_build/``; the shared
library is linked in-tree next to this file. Only out-of-date objects are rebuilt.

Run as ``python -m iane_gb300.build`` (add ``--force`` to rebuild everything).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libiane_gb300.so"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                     "--expt-relaxed-constexpr", "-I", str(INCLUDE)]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(path).exists():
        raise RuntimeError("nvcc not found")
    return path


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.rglob("*.h"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path, force: bool, verbose: bool) -> Path:
    obj = BUILD / (src.stem + ".o")
    if force or _stale(obj, [src] + _headers()):
        cmd = [nvcc()] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
        if verbose:
            (BUILD / (src.stem + ".ptxas.txt")).write_text(res.stderr)
    return obj


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    # the translation units with many kernel instantiations first, so the pool ends together
    heavy = ("conv_f32_k", "rl_pass", "rl_batch_k")
    sources = sorted(CSRC.glob("*.cu"), key=lambda p: (not p.stem.startswith(heavy), p.name))
    jobs = jobs or max(1, min(len(sources), os.cpu_count() or 4))
    with ThreadPoolExecutor(max_workers=jobs) as pool:
        objects = list(pool.map(lambda s: _compile(s, force, verbose), sources))
    if force or _stale(LIB, objects):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc()] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objects] + ["-lcufft"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
