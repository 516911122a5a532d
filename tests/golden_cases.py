"""Access to the golden vectors (tests/golden/golden.npz, made by make_golden.py)."""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden.npz"
_data = None


def data():
    global _data
    if _data is None:
        _data = dict(np.load(GOLDEN))
    return _data


def conv_cases():
    d = data()
    names = sorted({k.split("__")[0] for k in d if k.endswith("__border") and not k.startswith("morph_")})
    return [(n, d[f"{n}__src"], d[f"{n}__kernel"], d[f"{n}__out"], str(d[f"{n}__border"])) for n in names]


def rgb8_cases():
    """Packed rgb8 images (h, w, 3) convolved by the reference with a per-channel pixel type;
    the border is the name's suffix."""
    d = data()
    names = sorted({k.split("__")[0] for k in d if k.startswith("rgb8_") and k.endswith("__src")})
    return [(n, d[f"{n}__src"], d[f"{n}__kernel"], d[f"{n}__out"], n.rsplit("_", 1)[1]) for n in names]


def morph_cases():
    """Erosion / dilation outputs of the reference: (name, src, radius, op, border, mask or None, out)."""
    d = data()
    names = sorted({k.split("__")[0] for k in d if k.startswith("morph_") and k.endswith("__src")})
    out = []
    for n in names:
        mask = d[f"{n}__mask"]
        out.append((n, d[f"{n}__src"], tuple(int(v) for v in d[f"{n}__radius"]), str(d[f"{n}__op"]),
                    str(d[f"{n}__border"]), mask.astype(bool) if mask.size else None, d[f"{n}__out"]))
    return out


def mirror_cases():
    d = data()
    return [(n, d[f"{n}__src"], d[f"{n}__kernel"], d[f"{n}__out"]) for n in ("mirror_2d", "mirror_3d")]


def rl_cases():
    d = data()
    out = []
    for name, init, iters in (("rl_3d_init0", 0, 8), ("rl_3d_init1", 1, 8), ("rl_2d", 0, 12)):
        out.append((name, d[f"{name}__obs"], d[f"{name}__psf"], d[f"{name}__out"], init, iters))
    return out


def bench_pattern(width, height):
    """The reference benchmark's image and kernel (benchmarks/convolution.cu:88-96)."""
    i = np.arange(width * height, dtype=np.int64)
    image = (((i * 19) ^ (i // width)) & 0xFF).astype(np.uint8).reshape(height, width)
    k = np.arange(81, dtype=np.int64)
    kernel = (((k * 3) % 7 - 2) / 64.0).astype(np.float32).reshape(9, 9)
    return image, kernel


def bench_sha256() -> str:
    return str(data()["bench_u8_2560x1920__sha256"])


CONFIGS = Path(__file__).resolve().parent / "golden" / "configs.npz"
_configs = None


def configs():
    """The benchmark configurations run by the reference (tests/golden/make_config_fixtures.py)."""
    global _configs
    if _configs is None:
        _configs = dict(np.load(CONFIGS))
    return _configs
