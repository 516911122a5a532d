"""The row-strip direct kernel (direct_rows.cu), which iane_gb_convolve takes for 2-D f32 images
(or stacks of 2-D planes under a kernel one plane deep) of at least 4 M pixels with f32 kernels
of odd extents up to 7 (square, non-square and line filters).

Against the oracle within the FP32 bar |gpu - ref| <= 1e-5 * conv(|src|, |k|) for the three
borders, every kernel size, ragged image sizes and non-symmetric taps; bit for bit against the
tiled kernel over the whole image, borders included (a copy of the source one float off a
16-byte boundary is not TMA-addressable, so it takes the tiled kernel's element staging, whose
sums are added in the same order); a pitched source and a cropped, unaligned destination; and
the sizes just outside what the kernel takes."""
from __future__ import annotations

import numpy as np
import pytest

import iane_gb300
import oracle
from conftest import rel_err_bound
from gpu_helpers import empty_like_np, gaussian, magnitude, to_gpu, to_host, torch

pytestmark = pytest.mark.gpu

# kernel extents k: an int for square kernels, else (ky, kx)
CASES = [((2048, 2080), 7, "mirror"), ((2111, 2049), 5, "clamp"), ((2100, 2200), 3, "zero"),
         ((1030, 4096), 7, "clamp"), ((2049, 2177), 7, "zero"), ((4100, 1025), 3, "mirror"),
         # one strip that is both the first and the last; a last strip one column wide; the
         # least height taken (four steps) in one chunk per strip
         ((32769, 128), 7, "mirror"), ((16400, 257), 5, "clamp"), ((128, 32800), 3, "mirror"),
         # stacks of planes, each filtered on its own
         ((3, 1400, 1500), 7, "mirror"), ((5, 1000, 900), 5, "clamp"), ((2, 2048, 2048), 3, "zero"),
         # non-square kernels and line filters
         ((2050, 2100), (1, 7), "mirror"), ((2100, 2050), (7, 1), "clamp"), ((2049, 2111), (3, 7), "zero"),
         ((2111, 2049), (5, 3), "mirror"), ((2048, 2080), (7, 5), "clamp"), ((3, 1400, 1500), (1, 5), "mirror")]


def random_taps(k, seed, planes=False):
    rng = np.random.default_rng(seed)
    shape = (k, k) if isinstance(k, int) else k
    taps = (rng.random(shape, dtype=np.float32) - 0.3).astype(np.float32)
    return taps[None] if planes else taps


@pytest.mark.parametrize("shape,k,border", CASES, ids=[f"{s}-{k}-{b}".replace(" ", "") for s, k, b in CASES])
def test_against_oracle(cuda, shape, k, border):
    kseed = k if isinstance(k, int) else 10 * k[0] + k[1]
    rng = np.random.default_rng(sum(shape) + kseed)
    src = rng.random(shape, dtype=np.float32) * 4.0 - 1.0
    taps = random_taps(k, kseed + 11, planes=len(shape) == 3)
    ref = np.zeros(shape, np.float32)
    oracle.convolve(src, taps, ref, border)
    out = empty_like_np(shape, np.float32)
    iane_gb300.convolve(to_gpu(src), to_gpu(taps), out, border)
    assert rel_err_bound(to_host(out), ref, magnitude(src, taps, border)) <= 1e-5
    iane_gb300.device_status()


def misaligned_copy(src):
    """The same image in a buffer whose rows start 4 bytes past a 16-byte boundary."""
    t = torch()
    n = src.size
    flat = t.zeros(n + 4, dtype=t.float32, device="cuda")
    view = flat[1:1 + n].view(*src.shape)
    view.copy_(to_gpu(src))
    assert view.data_ptr() % 16 == 4
    return view


@pytest.mark.parametrize("k,border", [(7, "mirror"), (7, "clamp"), (5, "zero"), (3, "mirror"), ((1, 7), "mirror"),
                                      ((7, 3), "clamp"), ((5, 1), "mirror")])
def test_whole_image_equals_the_tiled_kernel_bit_for_bit(cuda, k, border):
    rng = np.random.default_rng(40 + (k if isinstance(k, int) else 10 * k[0] + k[1]))
    shape = (2085, 2100)
    src = rng.random(shape, dtype=np.float32)
    taps = gaussian((k, k), (k / 4.0, k / 3.0)) if k in (5, 7) else random_taps(k, 3)
    g = to_gpu(taps)
    rows = empty_like_np(shape, np.float32)
    iane_gb300.convolve(to_gpu(src), g, rows, border)           # row-strip kernel
    tiled = empty_like_np(shape, np.float32)
    iane_gb300.convolve(misaligned_copy(src), g, tiled, border)  # tiled kernel, element staging
    assert np.array_equal(to_host(rows), to_host(tiled))


def test_pitched_source_and_cropped_destination(cuda):
    t = torch()
    rng = np.random.default_rng(81)
    shape = (2050, 2100)
    big = rng.random((shape[0], 2112), dtype=np.float32)  # rows padded to 2112 floats
    src = np.ascontiguousarray(big[:, :shape[1]])
    taps = random_taps(7, 5)
    ref = np.zeros(shape, np.float32)
    oracle.convolve(src, taps, ref, "mirror")
    dst_big = t.zeros((shape[0] + 3, shape[1] + 41), dtype=t.float32, device="cuda")
    dst = dst_big[1:1 + shape[0], 3:3 + shape[1]]  # rows not 16-byte aligned: scalar stores
    iane_gb300.convolve(to_gpu(big)[:, :shape[1]], to_gpu(taps), dst, "mirror")
    assert rel_err_bound(to_host(dst), ref, magnitude(src, taps, "mirror")) <= 1e-5
    outside = dst_big.clone()
    outside[1:1 + shape[0], 3:3 + shape[1]] = 0
    assert float(outside.abs().max()) == 0.0


@pytest.mark.parametrize("shape,kshape", [((2047, 2048), (7, 7)), ((2048, 2048), (9, 5)), ((2048, 2048), (9, 9)),
                                          ((2, 2048, 2048), (3, 7, 7)), ((2, 1024, 2047), (1, 7, 7))])
def test_neighbouring_cases_take_the_other_kernels(cuda, shape, kshape):
    # just under 4 M pixels (one plane or a stack), 9 rows, 9 x 9 and a kernel three planes
    # deep: the tiled kernel, same bar
    rng = np.random.default_rng(sum(shape))
    src = rng.random(shape, dtype=np.float32)
    taps = (rng.random(kshape, dtype=np.float32) - 0.3).astype(np.float32)
    ref = np.zeros(src.shape, np.float32)
    oracle.convolve(src, taps, ref, "mirror")
    out = empty_like_np(src.shape, np.float32)
    iane_gb300.convolve(to_gpu(src), to_gpu(taps), out, "mirror")
    assert rel_err_bound(to_host(out), ref, magnitude(src, taps, "mirror")) <= 1e-5


def test_non_finite_pixels_match_the_tiled_kernel_bit_for_bit(cuda):
    # NaN and +-Inf samples (near the image's corners, edges and interior) propagate through
    # the same FMAs in the same order in both kernels: the outputs' bit patterns are equal
    rng = np.random.default_rng(90)
    shape = (2085, 2100)
    src = rng.random(shape, dtype=np.float32)
    for (y, x), v in {(0, 0): np.nan, (1, 2098): np.inf, (2084, 5): -np.inf, (1000, 1000): np.nan,
                      (1500, 64): np.inf, (31, 127): -np.inf, (2083, 2099): np.nan}.items():
        src[y, x] = v
    taps = random_taps(7, 9)
    g = to_gpu(taps)
    for border in ("mirror", "zero"):
        rows = empty_like_np(shape, np.float32)
        iane_gb300.convolve(to_gpu(src), g, rows, border)
        tiled = empty_like_np(shape, np.float32)
        iane_gb300.convolve(misaligned_copy(src), g, tiled, border)
        a, b = to_host(rows), to_host(tiled)
        assert np.isnan(a).any() and np.isinf(a).any()
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_stack_equals_the_tiled_kernel_bit_for_bit(cuda):
    rng = np.random.default_rng(91)
    src = rng.random((3, 1200, 1300), dtype=np.float32)
    taps = gaussian((1, 7, 7), (1.0, 1.7, 2.1))
    g = to_gpu(taps)
    for border in ("mirror", "clamp"):
        rows = empty_like_np(src.shape, np.float32)
        iane_gb300.convolve(to_gpu(src), g, rows, border)
        tiled = empty_like_np(src.shape, np.float32)
        iane_gb300.convolve(misaligned_copy(src), g, tiled, border)
        assert np.array_equal(to_host(rows), to_host(tiled))
