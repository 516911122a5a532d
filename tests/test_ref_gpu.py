"""The reference's own CUDA convolution kernel, built from its headers into a cubin
(oracle/ref_gpu.cu) and launched through the driver API (oracle/ref_gpu.py), on the GPU.

Its results are the reference's: bit-identical to the CPU oracle (which is pinned to the
reference) and to this library's exact mode, for both of the reference's borders. This pins the
GPU baseline that bench.py's reference arm times. Skipped where the cubin was not built (it is
built only where the reference's headers are)."""
from __future__ import annotations

import numpy as np
import pytest

import iane_gb300
import oracle
from gpu_helpers import empty_like_np, to_gpu, to_host
from oracle import ref_gpu

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_gpu.available(), reason="reference cubin not built here")]


@pytest.mark.parametrize("border", ["clamp", "zero"])
@pytest.mark.parametrize("shape,kshape", [((12, 40, 36), (3, 7, 5)), ((5, 9, 70), (7, 3, 9)), ((1, 1, 1), (1, 1, 1))])
def test_reference_kernel_is_the_reference_result(cuda, shape, kshape, border):
    rng = np.random.default_rng(sum(shape) + sum(kshape))
    src = rng.random(shape, dtype=np.float32)
    kernel = rng.standard_normal(kshape).astype(np.float32)
    want = np.zeros_like(src)
    oracle.convolve(src, kernel, want, border)
    ref = ref_gpu.ReferenceConvolution()
    got = empty_like_np(shape, np.float32)
    ref.convolve(to_gpu(src), to_gpu(kernel), got, border)
    ours = empty_like_np(shape, np.float32)
    iane_gb300.convolve(to_gpu(src), to_gpu(kernel), ours, border, exact=True)
    assert np.array_equal(to_host(got), want)
    assert np.array_equal(to_host(ours), want)
    ref.close()


def test_reference_kernel_on_a_strided_crop(cuda):
    rng = np.random.default_rng(5)
    big = rng.random((10, 30, 50), dtype=np.float32)
    kernel = rng.random((3, 5, 5), dtype=np.float32)
    src = big[2:8, 3:27, 4:44]  # a crop: its extent is the sampling boundary
    want = np.zeros(src.shape, np.float32)
    oracle.convolve(np.ascontiguousarray(src), kernel, want, "clamp")
    g_big = to_gpu(big)
    ref = ref_gpu.ReferenceConvolution()
    got = empty_like_np(src.shape, np.float32)
    ref.convolve(g_big[2:8, 3:27, 4:44], to_gpu(kernel), got, "clamp")
    assert np.array_equal(to_host(got), want)
    ref.close()
