"""Build recipe for the CPU oracle (test infrastructure only).

* ``oracle/liboracle.so`` -- the C restatement in ``iane_oracle.c`` (gcc, pthreads) and the
  deterministic input generator in ``det_synth.c``. Built everywhere, including the GPU host.
* ``oracle/_ref/libiane_ref.so`` -- ``ref_shim.cpp`` compiled against the reference's own
  headers, read in place from the reference checkout (``IANE_REFERENCE`` or
  ``/root/reference``). Built only where that checkout exists; never copied.
* ``oracle/_ref/ref_conv_f32_3d.cubin`` and ``.json`` -- the reference's own CUDA convolution
  kernel (``ref_gpu.cu``) and its argument layout, also from the headers in place. A cubin is
  device code, so unlike the host library it runs on a GPU host of another CPU architecture.

Run as ``python oracle/build.py``.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
ORACLE_LIB = HERE / "liboracle.so"
REF_LIB = REF_DIR / "libiane_ref.so"


def reference_root() -> Path | None:
    root = Path(os.environ.get("IANE_REFERENCE", "/root/reference"))
    return root if (root / "include" / "iane" / "algorithms" / "convolution.hpp").is_file() else None


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    mtime = target.stat().st_mtime
    return any(s.stat().st_mtime > mtime for s in sources)


def build_oracle(force: bool = False) -> Path:
    sources = [HERE / "iane_oracle.c", HERE / "det_synth.c"]
    header = HERE.parent / "include" / "iane_gb" / "capi.h"
    if force or _stale(ORACLE_LIB, sources + [header]):
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        subprocess.check_call([
            "gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
            *[str(s) for s in sources], "-o", str(tmp), "-lm",
        ])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_reference(force: bool = False) -> Path | None:
    root = reference_root()
    if root is None:
        return None
    src = HERE / "ref_shim.cpp"
    header = HERE.parent / "include" / "iane_gb" / "capi.h"
    if force or _stale(REF_LIB, [src, header]):
        REF_DIR.mkdir(exist_ok=True)
        tmp = REF_LIB.with_suffix(".so.tmp")
        subprocess.check_call([
            "g++", "-O2", "-std=c++20", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
            "-I", str(root / "include"), str(src), "-o", str(tmp),
        ])
        os.replace(tmp, REF_LIB)
    return REF_LIB


REF_CUBIN = REF_DIR / "ref_conv_f32_3d.cubin"
REF_LAYOUT = REF_DIR / "ref_conv_f32_3d.json"


def build_reference_gpu(force: bool = False) -> Path | None:
    """The reference's own CUDA convolution kernel for f32 3-D views (``ref_gpu.cu``) as a cubin
    for sm_103a, and the byte layout of its functor argument (``ref_gpu_layout.cpp``, run here)
    as JSON, both into ``_ref``. Built only where the reference checkout exists; the cubin is
    device code, so it also serves a GPU host of another CPU architecture."""
    root = reference_root()
    if root is None:
        return None
    sources = [HERE / "ref_gpu.cu", HERE / "ref_gpu_types.hpp", HERE / "ref_gpu_layout.cpp"]
    if force or _stale(REF_CUBIN, sources) or _stale(REF_LAYOUT, sources):
        REF_DIR.mkdir(exist_ok=True)
        inc = ["-I", str(root / "include")]
        tmp = REF_CUBIN.with_suffix(".cubin.tmp")
        subprocess.check_call(["nvcc", "-cubin", "-std=c++20", "--expt-relaxed-constexpr", "--expt-extended-lambda",
                               "-gencode", "arch=compute_103a,code=sm_103a", "-O3", *inc,
                               str(HERE / "ref_gpu.cu"), "-o", str(tmp)])
        os.replace(tmp, REF_CUBIN)
        probe = REF_DIR / "ref_gpu_layout"
        subprocess.check_call(["g++", "-std=c++20", "-O0", *inc, str(HERE / "ref_gpu_layout.cpp"), "-o", str(probe)])
        layout = subprocess.run([str(probe)], check=True, capture_output=True, text=True).stdout
        REF_LAYOUT.write_text(layout)
        probe.unlink()
    return REF_CUBIN


def main() -> int:
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv) or "reference checkout absent: oracle/_ref not built")
    print(build_reference_gpu(force="--force" in sys.argv) or "reference checkout absent: no reference cubin")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
