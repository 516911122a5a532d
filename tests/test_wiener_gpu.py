"""Wiener deconvolution on the GPU against the oracle (examples/wiener/main.cu:44-83 of the
reference, restated with float64 DFTs).

Bars: the FP32 result is within 5e-4 of the image maximum of the oracle's float64 result
(FP32 transforms, amplified by the filter's gain of at most 1 / (2 sqrt(noise))); u8 results
differ from the oracle's by at most one level, where the FP32 value lies that close to a
rounding boundary."""
from __future__ import annotations

import zlib

import numpy as np
import pytest

import iane_gb300
import oracle
from gpu_helpers import empty_like_np, gaussian, to_gpu, to_host, torch

pytestmark = pytest.mark.gpu


def blurred(rng, shape, psf, noise_level=2.0):
    """A random scene blurred periodically by the PSF, plus noise, as u8."""
    scene = rng.random(shape) * 200 + 20
    h = np.fft.fftn(oracle.wiener_pad_psf(psf.astype(np.float64), shape))
    img = np.fft.ifftn(np.fft.fftn(scene) * h).real + rng.standard_normal(shape) * noise_level
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


CASES = [((300,), (9,)), ((128, 96), (7, 9)), ((97, 61), (5, 5)), ((64, 64), (4, 6)), ((16, 24, 20), (5, 5, 3)),
         ((512, 512), (15, 15))]


@pytest.mark.parametrize("shape,pshape", CASES, ids=[f"{s}-{p}" for s, p in CASES])
@pytest.mark.parametrize("noise", [0.002, 0.05])
def test_wiener_parity(cuda, shape, pshape, noise):
    rng = np.random.default_rng(zlib.crc32(repr((shape, pshape, noise)).encode()))
    psf = gaussian(pshape, [max(0.7, n / 4) for n in pshape])
    obs = blurred(rng, shape, psf)
    w = iane_gb300.Wiener(to_gpu(psf), shape, noise)
    out = empty_like_np(shape, np.float32)
    w.run(to_gpu(obs), out)
    ref = oracle.wiener(obs, psf, noise, np.float64)
    assert float(np.max(np.abs(to_host(out) - ref))) <= 5e-4 * float(obs.max())
    out8 = empty_like_np(shape, np.uint8)
    w.run(to_gpu(obs), out8)
    diff = np.abs(to_host(out8).astype(np.int32) - oracle.wiener(obs, psf, noise).astype(np.int32))
    assert int(diff.max()) <= 1 and float(np.mean(diff)) < 0.01
    w.close()


def test_wiener_delta_psf_known_answer(cuda):
    # a centred delta: H = 1 and the result is observed / (1 + noise)
    rng = np.random.default_rng(5)
    obs = rng.integers(0, 256, (40, 50)).astype(np.uint8)
    delta = np.zeros((3, 3), np.float32)
    delta[1, 1] = 1.0
    w = iane_gb300.Wiener(to_gpu(delta), obs.shape, 0.25)
    out = empty_like_np(obs.shape, np.float32)
    w.run(to_gpu(obs), out)
    assert np.allclose(to_host(out), obs / 1.25, rtol=1e-5, atol=1e-3)
    w.close()


def test_wiener_strided_views_and_types(cuda):
    t = torch()
    rng = np.random.default_rng(9)
    psf = gaussian((5, 7), (1.2, 1.6))
    big = blurred(rng, (70, 90), psf)
    src_np = np.ascontiguousarray(big[3:67, 5:85])
    ref = oracle.wiener(src_np, psf, 0.01, np.float64)
    w = iane_gb300.Wiener(to_gpu(psf), src_np.shape, 0.01)
    dst_big = t.zeros((70, 200), device="cuda")
    dst = dst_big[3:67, 10:170:2]
    w.run(to_gpu(big)[3:67, 5:85], dst)
    assert float(np.max(np.abs(to_host(dst) - ref))) <= 5e-4 * 255
    # u16 and f32 observed images give the same result as the u8 one
    for dtype in (np.uint16, np.float32):
        out = empty_like_np(src_np.shape, np.float32)
        w.run(to_gpu(src_np.astype(dtype)), out)
        assert float(np.max(np.abs(to_host(out) - ref))) <= 5e-4 * 255
    w.close()


def test_wiener_errors(cuda):
    psf = to_gpu(gaussian((5, 5), (1.0, 1.0)))
    for noise in (0.0, -1.0, float("nan"), float("inf")):
        with pytest.raises(iane_gb300.IaneInvalidArgument):
            iane_gb300.Wiener(psf, (32, 32), noise)
    with pytest.raises(iane_gb300.IaneInvalidArgument):
        iane_gb300.Wiener(psf, (4, 32), 0.01)  # PSF must fit inside the image
    w = iane_gb300.Wiener(psf, (32, 32), 0.01)
    obs = to_gpu(np.zeros((32, 32), np.uint8))
    with pytest.raises(iane_gb300.IaneInvalidArgument):
        w.run(to_gpu(np.zeros((32, 31), np.uint8)), empty_like_np((32, 31), np.uint8))
    with pytest.raises(iane_gb300.IaneLengthError):
        w.run(obs, empty_like_np((32, 32), np.uint8), scratch=torch().empty(16, dtype=torch().uint8, device="cuda"))
    w.close()
