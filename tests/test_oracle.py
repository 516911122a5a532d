"""The CPU oracle is pinned: it reproduces the reference's known answers, the golden
vectors made by the reference, and (where the reference is built here) the live reference
on random inputs, bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from golden_cases import bench_pattern, conv_cases, mirror_cases, morph_cases, rgb8_cases, rl_cases


def test_known_answer_1d_flip_zero_border():
    # test/unit/algorithms/test_convolution.cpp:10-23 of the reference
    out = np.zeros(3, np.int32)
    oracle.convolve(np.array([1, 2, 3], np.int32), np.array([1, 0, 0], np.int32), out, "zero")
    assert out.tolist() == [2, 3, 0]


@pytest.mark.parametrize("border,expected", [("clamp", [20, 20, 120, 120]), ("zero", [20, 0, 120, 0])])
def test_known_answer_crop_boundary(border, expected):
    # test/unit/algorithms/test_convolution.cpp:25-51: the crop's extent is the boundary
    source = np.array([[10 * x + 100 * y for x in range(4)] for y in range(2)], np.uint8)
    crop = source[:, 1:3]
    out = np.zeros((2, 2), np.uint8)
    oracle.convolve(crop, np.array([[1, 0, 0]], np.float32), out, border)
    assert out.ravel().tolist() == expected


@pytest.mark.parametrize("dim", [2, 3])
def test_known_answer_nd_last_axis(dim):
    # test/unit/algorithms/convolution_cases.hpp:12-34 (channel 0 of its pixel element):
    # 3^N image of i+1, kernel {2,-1,0} along the last axis, zero border.
    shape = (3,) * dim
    src = (np.arange(3 ** dim, dtype=np.int32) + 1).reshape(shape)
    kshape = (3,) + (1,) * (dim - 1)
    kernel = np.array([2, -1, 0], np.int32).reshape(kshape)
    out = np.zeros(shape, np.int32)
    oracle.convolve(src, kernel, out, "zero")
    plane = 3 ** (dim - 1)
    flat = src.ravel()
    layer = np.arange(flat.size) // plane
    nxt = np.where(layer == 2, 0, flat + plane)
    assert np.array_equal(out.ravel(), 2 * nxt - flat)


@pytest.mark.parametrize("case", conv_cases(), ids=lambda c: c[0])
def test_oracle_matches_golden_convolution(case):
    name, src, kernel, expected, border = case
    out = np.zeros(expected.shape, expected.dtype)
    oracle.convolve(src, kernel, out, border)
    assert np.array_equal(out, expected), name


@pytest.mark.parametrize("case", rgb8_cases(), ids=lambda c: c[0])
def test_oracle_rgb8_matches_golden(case):
    name, src, kernel, expected, border = case
    out = np.zeros_like(src)
    oracle.convolve_rgb8(src, kernel, out, border)
    assert np.array_equal(out, expected), name


def test_oracle_rgb8_is_three_u8_channels():
    rng = np.random.default_rng(5)
    rgb = rng.integers(0, 256, (9, 14, 3), dtype=np.uint8)
    k = rng.standard_normal((3, 5)).astype(np.float32)
    out = np.zeros_like(rgb)
    oracle.convolve_rgb8(rgb, k, out, "mirror")
    for c in range(3):
        ch = np.zeros((9, 14), np.uint8)
        oracle.convolve(np.ascontiguousarray(rgb[..., c]), k, ch, "mirror")
        assert np.array_equal(out[..., c], ch)


@pytest.mark.parametrize("case", mirror_cases(), ids=lambda c: c[0])
def test_oracle_mirror_matches_padded_reference(case):
    name, src, kernel, expected = case
    out = np.zeros(expected.shape, np.float32)
    oracle.convolve(src, kernel, out, "mirror")
    assert np.array_equal(out, expected), name


@pytest.mark.parametrize("case", rl_cases(), ids=lambda c: c[0])
def test_oracle_matches_golden_rl(case):
    name, obs, psf, expected, init, iters = case
    est = oracle.rl(obs, psf, iters, 1e-6, init=init)
    assert np.array_equal(est, expected), name


def test_separable_oracle_equals_sequential_unit_kernels():
    rng = np.random.default_rng(5)
    src = rng.random((5, 8, 9), dtype=np.float32)
    taps = [rng.random(n, dtype=np.float32) for n in (5, 3, 3)]
    out = np.zeros_like(src)
    oracle.convolve_separable(src, taps, out, "mirror")
    a = src
    for axis, t in enumerate(taps):
        shape = [1, 1, 1]
        shape[2 - axis] = t.size
        nxt = np.zeros_like(src)
        oracle.convolve(a, t.reshape(shape), nxt, "mirror")
        a = nxt
    assert np.array_equal(out, a)


def test_benchmark_pattern_small_exact_in_fp32_accumulation():
    # The benchmark kernel is k/64: every partial sum is exact in FP32 as well as FP64,
    # which is why GPU FP32 accumulation reproduces the reference's bytes bit-exactly.
    image, kernel = bench_pattern(64, 48)
    out = np.zeros(image.shape, np.uint8)
    oracle.convolve(image, kernel, out, "clamp")
    assert out.dtype == np.uint8 and out.shape == (48, 64)


def test_sensitivity_interior_is_kernel_sum():
    psf = np.random.default_rng(1).random((3, 5, 7), dtype=np.float32)
    s = oracle.sensitivity(psf, (9, 10, 11))
    assert abs(float(s[4, 5, 5]) - float(psf.astype(np.float64).sum())) < 1e-5
    assert float(s[0, 0, 0]) < float(s[4, 5, 5])


reference = pytest.mark.skipif(not oracle.reference_available(), reason="reference checkout not built here")


@reference
@pytest.mark.parametrize("border", ["clamp", "zero"])
@pytest.mark.parametrize("shape,kshape", [((31,), (7,)), ((12, 17), (5, 3)), ((6, 7, 9), (3, 5, 7)), ((3, 4, 5), (7, 9, 11))])
def test_oracle_matches_live_reference_f32(border, shape, kshape):
    rng = np.random.default_rng(sum(shape) + len(border))
    src = rng.standard_normal(shape).astype(np.float32)
    kernel = rng.standard_normal(kshape).astype(np.float32)
    a, b = np.zeros_like(src), np.zeros_like(src)
    oracle.convolve(src, kernel, a, border)
    oracle.convolve(src, kernel, b, border, use_reference=True)
    assert np.array_equal(a, b)


@reference
def test_oracle_matches_live_reference_strided_views():
    rng = np.random.default_rng(3)
    big = rng.random((9, 20, 24), dtype=np.float32)
    src = big[1:8, 2:17:2, 3:21]
    kernel = rng.random((3, 3, 5), dtype=np.float32)
    a = np.zeros((7, 8, 18), np.float32)
    b = np.zeros((7, 8, 40), np.float32)[:, :, ::2][:, :, :18]
    oracle.convolve(src, kernel, a, "clamp")
    oracle.convolve(src, kernel, b, "clamp", use_reference=True)
    assert np.array_equal(a, b)


@reference
@pytest.mark.parametrize("border", ["clamp", "zero"])
def test_oracle_rgb8_matches_live_reference(border):
    rng = np.random.default_rng(17 + len(border))
    rgb = rng.integers(0, 256, (3, 11, 8, 3), dtype=np.uint8)
    k = rng.standard_normal((3, 3, 5)).astype(np.float32)
    a, b = np.zeros_like(rgb), np.zeros_like(rgb)
    oracle.convolve_rgb8(rgb, k, a, border)
    oracle.convolve_rgb8(rgb, k, b, border, use_reference=True)
    assert np.array_equal(a, b)


@reference
@pytest.mark.parametrize("dtypes", [(np.int8, np.float32, np.int8), (np.uint32, np.int32, np.uint32),
                                    (np.float32, np.float32, np.int8), (np.float32, np.float32, np.uint32)])
def test_oracle_new_scalar_types_match_live_reference(dtypes):
    sd, kd, dd = dtypes
    rng = np.random.default_rng(23)
    if sd == np.float32:
        src = (rng.standard_normal((6, 10, 7)) * 3e9).astype(np.float32)
    else:
        info = np.iinfo(sd)
        src = rng.integers(info.min, info.max, (6, 10, 7), dtype=sd, endpoint=True)
    k = rng.integers(-3, 4, (3, 5, 3)).astype(kd) if kd == np.int32 else rng.standard_normal((3, 5, 3)).astype(kd)
    a, b = np.zeros(src.shape, dd), np.zeros(src.shape, dd)
    oracle.convolve(src, k, a, "zero")
    oracle.convolve(src, k, b, "zero", use_reference=True)
    assert np.array_equal(a, b)


@reference
def test_oracle_rl_matches_live_reference_with_u8_like_data():
    rng = np.random.default_rng(11)
    obs = rng.integers(0, 256, (7, 9, 12)).astype(np.float32)
    psf = rng.random((3, 3, 5), dtype=np.float32)
    psf /= psf.sum()
    for init in (0, 1):
        a = oracle.rl(obs, psf, 6, 1e-6, init=init)
        b = oracle.rl(obs, psf, 6, 1e-6, init=init, use_reference=True)
        assert np.array_equal(a, b)


# --- Wiener (numpy restatement) -------------------------------------------------------------

def test_wiener_oracle_dft_matches_direct_definition():
    # the reference's FFT test computes each bin as sum x * exp(-2 pi i k x / n) in double
    # (test/unit/prepared/real_fft_cases.hpp:47-75); the oracle's transform is that sum
    size = (5, 7)
    img = ((np.arange(35) * 7) % 11 - 4).astype(np.float64).reshape(size)
    spec = np.fft.fftn(img)
    ky, kx = np.meshgrid(np.arange(size[0]), np.arange(size[1]), indexing="ij")
    for v in range(size[0]):
        for u in range(size[1]):
            phase = -2 * np.pi * (u * kx / size[1] + v * ky / size[0])
            direct = np.sum(img * np.cos(phase)) + 1j * np.sum(img * np.sin(phase))
            assert abs(spec[v, u] - direct) < 3e-5


def test_wiener_oracle_known_answers():
    rng = np.random.default_rng(2)
    obs = rng.integers(0, 256, (12, 20)).astype(np.uint8)
    # a centred delta: H = 1, so the result is observed / (1 + noise)
    delta = np.zeros((3, 5), np.float32)
    delta[1, 2] = 1.0
    out = oracle.wiener(obs, delta, 0.25, np.float64)
    assert np.allclose(out, obs / 1.25, atol=1e-9)
    assert np.array_equal(oracle.wiener(obs, delta, 0.25), oracle.to_gray8(obs / 1.25))
    # the PSF centre goes to the origin: an off-centre delta shifts the image back
    shifted = np.zeros((3, 5), np.float32)
    shifted[1, 3] = 1.0  # one column right of the centre: convolution shifts by +1 in x
    out = oracle.wiener(obs, shifted, 1e-9, np.float64)
    assert np.allclose(out, np.roll(obs, -1, axis=1), atol=1e-6)
    # the wrapped PSF: tap x lands at (x - e // 2) mod n
    pad = oracle.wiener_pad_psf(np.arange(15, dtype=np.float32).reshape(3, 5), (4, 6))
    assert pad[0, 0] == 7 and pad[0, 5] == 6 and pad[3, 4] == 0 and pad[3, 0] == 2 and pad[1, 2] == 14


def test_to_gray8_rule():
    v = np.array([-1.0, 0.0, 0.49, 0.5, 1.5, 2.4999, 254.5, 255.0, 300.0, np.nan], np.float32)
    assert oracle.to_gray8(v).tolist() == [0, 0, 0, 1, 2, 2, 255, 255, 255, 0]


# --- flat morphology --------------------------------------------------------------------------

def test_morphology_known_answers():
    # test/unit/algorithms/color_morphology_cases.hpp:87-117: values {99, 3, 1, 5, 2, 99},
    # crop [1, 5); a 1-radius box with clamp, and the offset-+1-only footprint with zero
    src = np.array([99, 3, 1, 5, 2, 99], np.int32)[1:5]
    out = np.zeros(4, np.int32)
    assert oracle.morphology(src, out, (1,), "erode").tolist() == [1, 1, 1, 2]
    assert oracle.morphology(src, out, (1,), "dilate").tolist() == [3, 5, 5, 5]
    forward = np.array([False, False, True])
    assert oracle.morphology(src, out, (1,), "erode", "zero", forward).tolist() == [1, 5, 2, 0]
    assert oracle.morphology(src, out, (1,), "dilate", "zero", forward).tolist() == [0, 3, 1, 5]


def test_morphology_compound_known_answer():
    # color_morphology_cases.hpp:119-166 in 3-D: a two-plane slab plus an impulse; opening
    # removes the impulse and keeps the slab, closing the complement does the same
    for close in (False, True):
        img = np.zeros((3, 3, 4), np.int32)
        img[:, :, :2] = 1
        img[1, 1, 3] = 1
        if close:
            img = 1 - img
        out = np.zeros_like(img)
        oracle.morphology(img, out, (1, 1, 1), "closing" if close else "opening")
        want = np.zeros_like(img)
        want[:, :, :2] = 1
        assert np.array_equal(out, 1 - want if close else want)


@pytest.mark.parametrize("case", morph_cases(), ids=lambda c: c[0])
def test_oracle_morphology_matches_golden(case):
    name, src, radius, op, border, mask, expected = case
    out = np.zeros_like(src)
    oracle.morphology(src, out, radius, op, border, mask)
    assert out.tobytes() == expected.tobytes(), name  # bitwise: NaN and signed zeros included


@reference
@pytest.mark.parametrize("dtype", [np.uint8, np.int16, np.float32])
@pytest.mark.parametrize("border", ["clamp", "zero"])
def test_oracle_morphology_matches_live_reference(dtype, border):
    rng = np.random.default_rng(31)
    src = (rng.standard_normal((4, 9, 11)) * 50).astype(dtype) if dtype == np.float32 else \
        rng.integers(np.iinfo(dtype).min, np.iinfo(dtype).max, (4, 9, 11), dtype=dtype)
    mask = rng.random((3, 5, 3)) < 0.5
    for op in ("erode", "dilate"):
        for m in (None, mask):
            a, b = np.zeros_like(src), np.zeros_like(src)
            oracle.morphology(src, a, (1, 2, 1), op, border, m)
            oracle.morphology(src, b, (1, 2, 1), op, border, m, use_reference=True)
            assert a.tobytes() == b.tobytes()
