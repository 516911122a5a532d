"""The row-strip separable kernel for large 2-D images (separable_rows.cu), which takes
iane_gb_convolve_separable for f32 images of at least 4 M pixels.

Against the oracle (successive 1-D convolutions, the reference's convolve with unit-extent
kernels) within the FP32 bar |gpu - ref| <= 1e-5 * conv(|src|, |k|), for all three borders,
radii 1..7 per axis (different on the two axes), a pitched source and a cropped destination;
and bit for bit against the tiled separable kernel, which smaller images take: interior pixels
of a large image equal the same pixels of a 1024 x 1024 crop."""
from __future__ import annotations

import numpy as np
import pytest

import iane_gb300
import oracle
from conftest import rel_err_bound
from gpu_helpers import empty_like_np, gaussian, magnitude, to_gpu, to_host, torch

pytestmark = pytest.mark.gpu


def taps(n, sigma):
    return gaussian((n,), (sigma,))


CASES = [((2048, 2080), 7, 7, "mirror"), ((2111, 2049), 3, 15, "clamp"), ((2100, 2200), 15, 5, "zero"),
         ((2048, 2304), 1, 9, "mirror"), ((4096, 1030), 11, 13, "clamp")]


@pytest.mark.parametrize("shape,kx,ky,border", CASES, ids=[f"{s}-{x}-{y}-{b}" for s, x, y, b in CASES])
def test_large_2d_against_oracle(cuda, shape, kx, ky, border):
    rng = np.random.default_rng(sum(shape) + kx * 31 + ky)
    src = rng.random(shape, dtype=np.float32) * 4.0 - 1.0
    tx, ty = taps(kx, max(0.6, kx / 4)), taps(ky, max(0.6, ky / 5))
    ref = np.zeros_like(src)
    oracle.convolve_separable(src, [tx, ty], ref, border)
    out = empty_like_np(shape, np.float32)
    iane_gb300.convolve_separable(to_gpu(src), [to_gpu(tx), to_gpu(ty)], out, border)
    outer = np.outer(ty, tx).astype(np.float32)
    assert rel_err_bound(to_host(out), ref, magnitude(src, outer, border)) <= 1e-5
    iane_gb300.device_status()


def test_pitched_source_and_strided_destination(cuda):
    t = torch()
    rng = np.random.default_rng(77)
    shape = (2050, 2100)
    big = rng.random((shape[0], 2112), dtype=np.float32)  # rows padded to 2112 floats (16-byte pitch)
    src = big[:, :shape[1]]
    tx, ty = taps(7, 1.5), taps(9, 2.0)
    ref = np.zeros(shape, np.float32)
    oracle.convolve_separable(np.ascontiguousarray(src), [tx, ty], ref, "mirror")
    g_big = to_gpu(big)
    dst_big = t.zeros((shape[0] + 3, shape[1] + 40), dtype=t.float32, device="cuda")
    dst = dst_big[1:1 + shape[0], 4:4 + shape[1]]  # a crop of a larger, row-pitched buffer
    iane_gb300.convolve_separable(g_big[:, :shape[1]], [to_gpu(tx), to_gpu(ty)], dst, "mirror")
    outer = np.outer(ty, tx).astype(np.float32)
    assert rel_err_bound(to_host(dst), ref, magnitude(np.ascontiguousarray(src), outer, "mirror")) <= 1e-5
    outside = dst_big.clone()
    outside[1:1 + shape[0], 4:4 + shape[1]] = 0
    assert float(outside.abs().max()) == 0.0  # nothing written outside the view


def test_interior_equals_the_tiled_kernel_bit_for_bit(cuda):
    rng = np.random.default_rng(78)
    src = rng.random((2304, 2048), dtype=np.float32)
    tx, ty = taps(7, 1.4), taps(13, 2.6)
    g = to_gpu(src)
    big = empty_like_np(src.shape, np.float32)
    iane_gb300.convolve_separable(g, [to_gpu(tx), to_gpu(ty)], big, "zero")  # row-strip kernel
    y0, x0, n = 700, 500, 1024
    crop = empty_like_np((n, n), np.float32)
    iane_gb300.convolve_separable(g[y0:y0 + n, x0:x0 + n], [to_gpu(tx), to_gpu(ty)], crop, "zero")  # tiled
    r = 8  # beyond both radii from the crop's edges, the two see the same inputs
    got = to_host(big)[y0 + r:y0 + n - r, x0 + r:x0 + n - r]
    want = to_host(crop)[r:n - r, r:n - r]
    assert np.array_equal(got, want)
