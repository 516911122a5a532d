"""Generate the golden vectors in tests/golden/ from the reference itself.

Run where the reference checkout is present (it builds oracle/_ref/libiane_ref.so from the
reference's headers): ``python tests/golden/make_golden.py``. Every array comes from the
reference's own ``iane::convolve`` or from RL restated on the reference's own views and
algorithms; mirror-border cases use the reference convolution on an explicitly
mirror-padded image, cropped. The inputs are seeded and stored with the outputs.
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from oracle import build as oracle_build  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden.npz"


def gaussian(shape, sigma):
    grids = np.meshgrid(*[np.arange(n) - n // 2 for n in shape], indexing="ij")
    g = np.exp(-sum((x / s) ** 2 for x, s in zip(grids, sigma)) / 2.0)
    return (g / g.sum()).astype(np.float32)


def bench_pattern(width, height):
    """The reference benchmark's image and kernel (benchmarks/convolution.cu:88-96)."""
    i = np.arange(width * height, dtype=np.int64)
    image = (((i * 19) ^ (i // width)) & 0xFF).astype(np.uint8).reshape(height, width)
    k = np.arange(81, dtype=np.int64)
    kernel = (((k * 3) % 7 - 2) / 64.0).astype(np.float32).reshape(9, 9)
    return image, kernel


def ref_conv(src, kernel, out_dtype, border):
    out = np.zeros(src.shape, dtype=out_dtype)
    oracle.convolve(src, kernel, out, border, use_reference=True)
    return out


def main() -> int:
    if oracle_build.build_reference() is None:
        print("reference checkout not found", file=sys.stderr)
        return 1
    rng = np.random.default_rng(20261203)
    g = {}

    def case(name, src, kernel, out_dtype, border):
        g[f"{name}__src"] = src
        g[f"{name}__kernel"] = kernel
        g[f"{name}__out"] = ref_conv(src, kernel, out_dtype, border)
        g[f"{name}__border"] = np.array(border)

    case("f32_2d_clamp", rng.random((17, 23), dtype=np.float32), rng.standard_normal((5, 7)).astype(np.float32),
         np.float32, "clamp")
    case("f32_3d_zero", rng.random((6, 9, 11), dtype=np.float32), rng.random((3, 5, 3), dtype=np.float32),
         np.float32, "zero")
    case("f32_1d_clamp", rng.random(37, dtype=np.float32), rng.standard_normal(9).astype(np.float32),
         np.float32, "clamp")
    case("f32_3d_clamp_bigkernel", rng.random((4, 5, 6), dtype=np.float32), rng.random((5, 7, 9), dtype=np.float32),
         np.float32, "clamp")
    case("u8_2d_f32k_clamp", *bench_pattern(45, 31), np.uint8, "clamp")
    case("u8_2d_f32k_zero", *bench_pattern(45, 31), np.uint8, "zero")
    case("i32_3d_zero", rng.integers(-1000, 1000, (5, 7, 8), dtype=np.int32),
         rng.integers(-9, 10, (3, 3, 5), dtype=np.int32), np.int32, "zero")
    case("u16_2d_i32k_clamp", rng.integers(0, 65535, (12, 19), dtype=np.uint16),
         rng.integers(-3, 4, (3, 5), dtype=np.int32), np.uint16, "clamp")
    case("i16_2d_i32k_zero", rng.integers(-30000, 30000, (9, 14), dtype=np.int16),
         rng.integers(-2, 3, (5, 3), dtype=np.int32), np.int16, "zero")
    case("u8_2d_i32k_clamp", rng.integers(0, 255, (11, 13), dtype=np.uint8),
         rng.integers(-1, 3, (3, 3), dtype=np.int32), np.uint8, "clamp")
    case("f32_2d_f32k_to_u8", rng.random((10, 12), dtype=np.float32) * 300.0 - 20.0,
         rng.random((3, 3), dtype=np.float32), np.uint8, "clamp")
    case("f32_2d_f32k_to_i32", (rng.standard_normal((8, 9)) * 1e9).astype(np.float32),
         rng.standard_normal((3, 3)).astype(np.float32), np.int32, "zero")
    case("f64_3d_zero", rng.random((5, 6, 7)), rng.random((3, 3, 3)), np.float64, "clamp")

    # Mirror border (not in the reference): reference convolution of the mirror-padded
    # image with any border, cropped back to the original extent.
    src = rng.random((13, 10), dtype=np.float32)
    k = gaussian((7, 7), (1.5, 1.5))
    padded = oracle.mirror_pad(src, (3, 3))
    full = ref_conv(padded, k, np.float32, "clamp")
    g["mirror_2d__src"], g["mirror_2d__kernel"] = src, k
    g["mirror_2d__out"] = np.ascontiguousarray(full[3:-3, 3:-3])
    src3 = rng.random((4, 6, 5), dtype=np.float32)
    k3 = rng.random((3, 5, 7), dtype=np.float32)
    padded3 = oracle.mirror_pad(src3, (1, 2, 3))
    full3 = ref_conv(padded3, k3, np.float32, "zero")
    g["mirror_3d__src"], g["mirror_3d__kernel"] = src3, k3
    g["mirror_3d__out"] = np.ascontiguousarray(full3[1:-1, 2:-2, 3:-3])

    # Richardson-Lucy, restated on the reference's convolve/zip_view/copy.
    obs3 = (rng.poisson(rng.random((10, 14, 16)) * 200.0 + 10.0)).astype(np.float32)
    psf3 = gaussian((3, 5, 5), (1.0, 1.5, 1.5))
    for init in (0, 1):
        est = oracle.rl(obs3, psf3, 8, 1e-6, init=init, use_reference=True)
        g[f"rl_3d_init{init}__obs"], g[f"rl_3d_init{init}__psf"] = obs3, psf3
        g[f"rl_3d_init{init}__out"] = est.copy()
    obs2 = rng.integers(0, 255, (21, 26)).astype(np.float32)
    psf2 = gaussian((5, 7), (1.2, 1.8))
    est = oracle.rl(obs2, psf2, 12, 1e-6, init=0, use_reference=True)
    g["rl_2d__obs"], g["rl_2d__psf"], g["rl_2d__out"] = obs2, psf2, est.copy()

    # The reference benchmark at full size (benchmarks/convolution.cu:84-118): keep the
    # SHA-256 of the reference output (clamp) instead of the 4.9 MB image.
    image, kernel = bench_pattern(2560, 1920)
    bench_out = ref_conv(image, kernel, np.uint8, "clamp")
    g["bench_u8_2560x1920__sha256"] = np.array(hashlib.sha256(bench_out.tobytes()).hexdigest())

    # Element types added later, from their own seed so that the arrays above stay as they
    # were: i8 and u32 scalars, and packed rgb8 pixels (the custom element of
    # examples/convolution/main.cu:20-56) through the reference's convolve with a pixel type
    # of those semantics (oracle/ref_shim.cpp).
    rng2 = np.random.default_rng(20261204)
    case("i8_2d_f32k_clamp", rng2.integers(-128, 128, (13, 17), dtype=np.int8),
         rng2.standard_normal((5, 3)).astype(np.float32), np.int8, "clamp")
    case("i8_3d_i32k_zero", rng2.integers(-128, 128, (4, 7, 9), dtype=np.int8),
         rng2.integers(-3, 4, (3, 3, 3), dtype=np.int32), np.int8, "zero")
    case("u32_2d_f32k_zero", rng2.integers(0, 2 ** 32, (9, 11), dtype=np.uint32),
         rng2.random((3, 5), dtype=np.float32), np.uint32, "zero")
    case("u32_1d_i32k_clamp", rng2.integers(0, 2 ** 31, 29, dtype=np.uint32),
         rng2.integers(-2, 5, 7, dtype=np.int32), np.uint32, "clamp")
    for border in ("clamp", "zero"):
        rgb = rng2.integers(0, 256, (19, 23, 3), dtype=np.uint8)
        k = (rng2.standard_normal((5, 7)) / 4.0).astype(np.float32)
        out = np.zeros_like(rgb)
        oracle.convolve_rgb8(rgb, k, out, border, use_reference=True)
        g[f"rgb8_2d_{border}__src"], g[f"rgb8_2d_{border}__kernel"], g[f"rgb8_2d_{border}__out"] = rgb, k, out
    rgb, k = bench_pattern(64, 48)
    rgb = np.stack([rgb, rgb[::-1], 255 - rgb], axis=-1).copy()
    out = np.zeros_like(rgb)
    oracle.convolve_rgb8(rgb, k, out, "clamp", use_reference=True)
    g["rgb8_bench_clamp__src"], g["rgb8_bench_clamp__kernel"], g["rgb8_bench_clamp__out"] = rgb, k, out

    # Flat morphology through the reference's own erode / dilate (box footprints and mask
    # predicates), own seed: float data with NaNs and signed zeros exercise the update rule.
    rng3 = np.random.default_rng(20261205)

    def morph(name, src, radius, op, border, mask=None):
        out = np.zeros_like(src)
        oracle.morphology(src, out, radius, op, border, mask, use_reference=True)
        g[f"morph_{name}__src"], g[f"morph_{name}__out"] = src, out
        g[f"morph_{name}__radius"] = np.array(radius, np.int32)
        g[f"morph_{name}__op"], g[f"morph_{name}__border"] = np.array(op), np.array(border)
        g[f"morph_{name}__mask"] = np.zeros(0, np.uint8) if mask is None else mask.astype(np.uint8)

    morph("u8_2d_box_erode_clamp", rng3.integers(0, 256, (23, 31), dtype=np.uint8), (1, 2), "erode", "clamp")
    morph("u8_2d_box_dilate_zero", rng3.integers(0, 256, (23, 31), dtype=np.uint8), (2, 1), "dilate", "zero")
    fl = rng3.standard_normal((5, 9, 13)).astype(np.float32)
    fl[fl > 1.5] = np.nan
    fl[np.abs(fl) < 0.2] = 0.0
    fl[(np.abs(fl) < 0.4) & (fl < 0)] = -0.0
    morph("f32_3d_box_erode_zero", fl, (1, 1, 2), "erode", "zero")
    morph("f32_3d_box_dilate_clamp", fl, (1, 2, 1), "dilate", "clamp")
    cross = np.zeros((5, 3), bool)
    cross[2, :] = True
    cross[:, 1] = True
    morph("i16_2d_mask_dilate_clamp", rng3.integers(-30000, 30000, (17, 19), dtype=np.int16), (2, 1), "dilate",
          "clamp", cross)
    ring = np.ones((3, 3, 3), bool)
    ring[1, 1, 1] = False
    morph("f64_3d_mask_erode_zero", rng3.standard_normal((6, 7, 8)), (1, 1, 1), "erode", "zero", ring)
    morph("u32_1d_box_dilate_zero", rng3.integers(0, 2 ** 32, 40, dtype=np.uint32), (3,), "dilate", "zero")

    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(g)} arrays)")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
