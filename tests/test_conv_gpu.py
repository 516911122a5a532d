"""GPU convolution parity against the oracle and the reference's golden vectors.

Bars: integer images with integer kernels, and every result in exact mode, are
bit-identical to the reference; FP32 results (FP32 accumulation) are within 1e-5 of the
reference relative to conv(|src|, |kernel|) element by element."""
from __future__ import annotations

import hashlib
import zlib

import numpy as np
import pytest

import iane_gb300
import oracle
from golden_cases import bench_pattern, bench_sha256, conv_cases, mirror_cases
from gpu_helpers import empty_like_np, gaussian, magnitude, to_gpu, to_host, torch
from conftest import rel_err_bound

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5


def run_gpu(src, kernel, out_dtype, border, exact=False):
    s, k = to_gpu(src), to_gpu(kernel)
    d = empty_like_np(src.shape, out_dtype)
    iane_gb300.convolve(s, k, d, border, exact=exact)
    return to_host(d)


def run_oracle(src, kernel, out_dtype, border):
    out = np.zeros(src.shape, out_dtype)
    oracle.convolve(src, kernel, out, border)
    return out


def check_fp32(gpu, ref, src, kernel, border):
    assert gpu.shape == ref.shape
    err = rel_err_bound(gpu, ref, magnitude(src, kernel, border))
    assert err <= FP32_TOL, err


def test_known_answer_1d(cuda):
    out = run_gpu(np.array([1, 2, 3], np.int32), np.array([1, 0, 0], np.int32), np.int32, "zero")
    assert out.tolist() == [2, 3, 0]


@pytest.mark.parametrize("border,expected", [("clamp", [20, 20, 120, 120]), ("zero", [20, 0, 120, 0])])
def test_known_answer_crop(cuda, border, expected):
    t = torch()
    source = to_gpu(np.array([[10 * x + 100 * y for x in range(4)] for y in range(2)], np.uint8))
    crop = source[:, 1:3]
    out = t.zeros((2, 2), dtype=t.uint8, device="cuda")
    iane_gb300.convolve(crop, to_gpu(np.array([[1, 0, 0]], np.float32)), out, border)
    assert to_host(out).ravel().tolist() == expected


@pytest.mark.parametrize("dim", [2, 3])
def test_known_answer_nd_last_axis(cuda, dim):
    shape = (3,) * dim
    src = (np.arange(3 ** dim, dtype=np.int32) + 1).reshape(shape)
    kernel = np.array([2, -1, 0], np.int32).reshape((3,) + (1,) * (dim - 1))
    out = run_gpu(src, kernel, np.int32, "zero")
    plane = 3 ** (dim - 1)
    flat = src.ravel()
    nxt = np.where(np.arange(flat.size) // plane == 2, 0, flat + plane)
    assert np.array_equal(out.ravel(), 2 * nxt - flat)


@pytest.mark.parametrize("case", conv_cases(), ids=lambda c: c[0])
def test_golden_exact_mode_is_bit_identical(cuda, case):
    name, src, kernel, expected, border = case
    assert np.array_equal(run_gpu(src, kernel, expected.dtype, border, exact=True), expected), name


@pytest.mark.parametrize("case", conv_cases(), ids=lambda c: c[0])
def test_golden_fast_mode(cuda, case):
    name, src, kernel, expected, border = case
    out = run_gpu(src, kernel, expected.dtype, border)
    integer_pair = np.issubdtype(src.dtype, np.integer) and np.issubdtype(kernel.dtype, np.integer)
    bench_like = name.startswith("u8_2d_f32k")  # k/64 taps: FP32 sums are exact
    if integer_pair or bench_like:
        assert np.array_equal(out, expected), name
    elif expected.dtype in (np.float32, np.float64):
        check_fp32(out, expected, src, kernel, border)
    else:
        # float data into an integer destination: the FP32 sum may differ by its rounding
        # error and then round across a boundary of the cast, so allow one unit beyond the
        # FP32 bound; exact mode is bit-identical (above)
        slack = 1.0 + FP32_TOL * magnitude(src, kernel, border)
        assert np.all(np.abs(out.astype(np.float64) - expected.astype(np.float64)) <= slack), name


@pytest.mark.parametrize("case", mirror_cases(), ids=lambda c: c[0])
def test_golden_mirror(cuda, case):
    name, src, kernel, expected = case
    assert np.array_equal(run_gpu(src, kernel, np.float32, "mirror", exact=True), expected), name
    check_fp32(run_gpu(src, kernel, np.float32, "mirror"), expected, src, kernel, "mirror")


SHAPES = [
    ((1,), (1,)), ((37,), (9,)), ((5,), (11,)),
    ((1, 1), (3, 3)), ((17, 29), (5, 7)), ((64, 64), (7, 7)), ((70, 131), (15, 31)), ((3, 200), (9, 1)),
    ((1, 1, 1), (3, 3, 3)), ((9, 10, 11), (3, 5, 7)), ((7, 33, 65), (7, 15, 15)), ((4, 5, 6), (9, 9, 9)),
    ((19, 40, 72), (5, 3, 13)), ((2, 96, 100), (3, 11, 21)),
    # 16-byte aligned rows: TMA staging, clamp/mirror edges fixed up in shared memory
    ((9, 8), (15, 15)), ((16, 24), (13, 31)), ((5, 12, 20), (7, 9, 5)), ((3, 130, 260), (3, 7, 7)),
    # 29791 taps on the tiled path (one kernel plane's taps in shared memory at a time)
    ((20, 40, 36), (31, 31, 31)),
]


@pytest.mark.parametrize("border", ["clamp", "zero", "mirror"])
@pytest.mark.parametrize("shape,kshape", SHAPES, ids=[f"{s}-{k}" for s, k in SHAPES])
def test_random_f32_parity(cuda, shape, kshape, border):
    rng = np.random.default_rng(zlib.crc32(repr((shape, kshape, border)).encode()))
    src = rng.standard_normal(shape).astype(np.float32)
    kernel = rng.standard_normal(kshape).astype(np.float32)
    ref = run_oracle(src, kernel, np.float32, border)
    check_fp32(run_gpu(src, kernel, np.float32, border), ref, src, kernel, border)
    if kernel.size * 8 > 200 * 1024:
        # the exact (FP64) mode keeps all taps in shared memory and refuses larger kernels
        with pytest.raises(iane_gb300.IaneError) as err:
            run_gpu(src, kernel, np.float32, border, exact=True)
        assert err.value.status == iane_gb300.abi.UNSUPPORTED
        return
    assert np.array_equal(run_gpu(src, kernel, np.float32, border, exact=True), ref)


@pytest.mark.parametrize("border", ["clamp", "zero", "mirror"])
@pytest.mark.parametrize("dtypes", [(np.uint8, np.int32, np.uint8), (np.uint16, np.int32, np.uint16),
                                    (np.int16, np.int32, np.int16), (np.int32, np.int32, np.int32)])
def test_random_integer_bit_exact(cuda, dtypes, border):
    sd, kd, dd = dtypes
    rng = np.random.default_rng(7)
    info = np.iinfo(sd)
    src = rng.integers(max(info.min, -50000), min(info.max, 50000), (6, 21, 34)).astype(sd)
    kernel = rng.integers(-4, 5, (3, 5, 3)).astype(kd)
    ref = run_oracle(src, kernel, dd, border)
    assert np.array_equal(run_gpu(src, kernel, dd, border), ref)


def test_strided_and_cropped_views(cuda):
    t = torch()
    rng = np.random.default_rng(9)
    big = rng.random((11, 40, 50), dtype=np.float32)
    kernel = rng.random((3, 5, 7), dtype=np.float32)
    src_np = big[2:9, 3:37:2, 5:46]
    g = to_gpu(big)[2:9, 3:37:2, 5:46]
    dst_big = t.zeros((9, 20, 90), device="cuda")
    dst = dst_big[1:8, 1:18, 3:85:2][:, :, : src_np.shape[2]]
    assert tuple(dst.shape) == src_np.shape
    for border in ("clamp", "zero", "mirror"):
        ref = run_oracle(np.ascontiguousarray(src_np), kernel, np.float32, border)
        iane_gb300.convolve(g, to_gpu(kernel), dst, border)
        check_fp32(to_host(dst), ref, src_np, kernel, border)
        iane_gb300.convolve(g, to_gpu(kernel), dst, border, exact=True)
        assert np.array_equal(to_host(dst), ref)
    # untouched padding around the destination crop
    mask = t.ones_like(dst_big, dtype=t.bool)
    mask[1:8, 1:18, 3:85:2] = False
    assert float(dst_big[mask].abs().max()) == 0.0


def test_reference_benchmark_bit_exact(cuda):
    # benchmarks/convolution.cu:84-118: 2560x1920 u8, 9x9 float kernel, clamp; the
    # reference checks its CUDA output byte-for-byte against its serial CPU output.
    image, kernel = bench_pattern(2560, 1920)
    out = run_gpu(image, kernel, np.uint8, "clamp")
    assert hashlib.sha256(out.tobytes()).hexdigest() == bench_sha256()


def test_rl_volume_convolution_slabs(cuda):
    # The 3-D RL volume (256x256x64) and PSF (15x15x7) at full size: the GPU result on
    # every plane of a few z-slabs equals the oracle on that slab (a slab that holds the
    # kernel's whole z support gives the full-volume answer for its centre plane).
    rng = np.random.default_rng(2)
    vol = (rng.random((64, 256, 256), dtype=np.float32) * 100).astype(np.float32)
    psf = gaussian((7, 15, 15), (1.0, 2.0, 2.0))
    out = run_gpu(vol, psf, np.float32, "zero")
    for z0 in (0, 2, 31, 62, 63):
        lo, hi = max(0, z0 - 3), min(64, z0 + 4)
        slab = np.ascontiguousarray(vol[lo:hi])
        ref = run_oracle(slab, psf, np.float32, "zero")[z0 - lo]
        mag = magnitude(slab, psf, "zero")[z0 - lo]
        assert rel_err_bound(out[z0], ref, mag) <= FP32_TOL


@pytest.mark.parametrize("border", ["clamp", "zero", "mirror"])
@pytest.mark.parametrize("shape,taps", [((40,), (7,)), ((33, 70), (7, 7)), ((512, 512), (7, 7)), ((9, 30, 75), (5, 3, 7)),
                                       ((20, 20, 20), (9, 9, 9)), ((3, 5, 4), (7, 9, 11)), ((70, 90), (21, 3)),
                                       ((37, 41, 130), (15, 15, 15)), ((1, 1, 1), (3, 3, 3)), ((17, 1, 200), (3, 5, 1)),
                                       ((64, 64, 64), (3, 3, 3)), ((50, 70, 150), (7, 7, 7)), ((33, 17, 16), (9, 1, 5)),
                                       ((130, 40, 66), (3, 7, 9)), ((12, 16, 16), (5, 5, 5))])
def test_separable_parity(cuda, shape, taps, border):
    rng = np.random.default_rng(len(shape) * 100 + taps[0])
    src = rng.random(shape, dtype=np.float32)
    tap_list = [gaussian((n,), (max(0.5, n / 5),)) for n in taps]
    ref = np.zeros_like(src)
    oracle.convolve_separable(src, tap_list, ref, border)
    d = empty_like_np(shape, np.float32)
    iane_gb300.convolve_separable(to_gpu(src), [to_gpu(t) for t in tap_list], d, border)
    out = to_host(d)
    # each 1-D pass accumulates in FP32; positive data and taps
    assert float(np.max(np.abs(out - ref) / np.maximum(np.abs(ref), 1e-30))) <= FP32_TOL


def test_separable_strided_views(cuda):
    t = torch()
    rng = np.random.default_rng(8)
    big = rng.random((30, 70, 90), dtype=np.float32)
    src_np = np.ascontiguousarray(big[3:27, 5:65:2, 1:88])
    g = to_gpu(big)[3:27, 5:65:2, 1:88]
    taps = [gaussian((n,), (1.2,)) for n in (5, 7, 3)]
    for border in ("clamp", "zero", "mirror"):
        ref = np.zeros_like(src_np)
        oracle.convolve_separable(src_np, taps, ref, border)
        dst_big = t.zeros((24, 30, 200), device="cuda")
        dst = dst_big[:, :, 3:3 + 2 * src_np.shape[2]:2]
        iane_gb300.convolve_separable(g, [to_gpu(x) for x in taps], dst, border)
        out = to_host(dst)
        assert float(np.max(np.abs(out - ref) / np.maximum(np.abs(ref), 1e-30))) <= FP32_TOL


def test_separable_equals_direct_outer_product(cuda):
    rng = np.random.default_rng(4)
    src = rng.random((512, 512), dtype=np.float32)
    g = gaussian((7,), (1.5,))
    direct = run_gpu(src, np.outer(g, g).astype(np.float32), np.float32, "mirror")
    d = empty_like_np(src.shape, np.float32)
    iane_gb300.convolve_separable(to_gpu(src), [to_gpu(g), to_gpu(g)], d, "mirror")
    assert float(np.max(np.abs(to_host(d) - direct) / direct)) <= 2e-6


def test_errors_raise_before_launch(cuda):
    a = to_gpu(np.zeros((8, 8), np.float32))
    with pytest.raises(iane_gb300.IaneInvalidArgument):
        iane_gb300.convolve(a, to_gpu(np.zeros((2, 3), np.float32)), a.clone())
    with pytest.raises(iane_gb300.IaneInvalidArgument):
        iane_gb300.convolve(a, to_gpu(np.zeros((3, 3), np.float32)), to_gpu(np.zeros((8, 9), np.float32)))
    empty = to_gpu(np.zeros((0, 8), np.float32))
    iane_gb300.convolve(empty, to_gpu(np.ones((3, 3), np.float32)), empty.clone())
    iane_gb300.device_status()


# --- spectral (FFT) convolution ---------------------------------------------------------

@pytest.mark.parametrize("border", ["clamp", "zero", "mirror"])
@pytest.mark.parametrize("shape,kshape", [((300,), (61,)), ((40, 70), (31, 21)), ((12, 30, 50), (9, 15, 21)),
                                          ((3, 5, 4), (7, 9, 11)), ((1, 33, 17), (1, 5, 3))])
def test_fft_convolution_parity(cuda, shape, kshape, border):
    """The spectral path against the FP64 oracle, with the direct FP32 path's per-element bar."""
    rng = np.random.default_rng(zlib.crc32(repr(("fft", shape, kshape, border)).encode()))
    src = rng.standard_normal(shape).astype(np.float32)
    kernel = rng.standard_normal(kshape).astype(np.float32)
    ref = run_oracle(src, kernel, np.float32, border)
    d = empty_like_np(shape, np.float32)
    iane_gb300.convolve(to_gpu(src), to_gpu(kernel), d, border, method="fft")
    check_fp32(to_host(d), ref, src, kernel, border)
    # f64 destination: FP64 transforms, far inside the bar
    d64 = empty_like_np(shape, np.float64)
    iane_gb300.convolve(to_gpu(src), to_gpu(kernel), d64, border, method="fft")
    ref64 = run_oracle(src, kernel, np.float64, border)
    assert rel_err_bound(to_host(d64), ref64, magnitude(src, kernel, border)) <= 1e-9


def test_fft_strided_and_cropped_views(cuda):
    """Strided source and destination crops go through the pad and crop kernels' view
    addressing; the padding around the destination crop stays untouched."""
    t = torch()
    rng = np.random.default_rng(31)
    big = rng.random((11, 40, 50), dtype=np.float32)
    kernel = rng.random((5, 9, 7), dtype=np.float32)
    src_np = big[2:9, 3:37:2, 5:46]
    g = to_gpu(big)[2:9, 3:37:2, 5:46]
    dst_big = t.zeros((9, 20, 90), device="cuda")
    dst = dst_big[1:8, 1:18, 3:85:2][:, :, : src_np.shape[2]]
    for border in ("clamp", "zero", "mirror"):
        ref = run_oracle(np.ascontiguousarray(src_np), kernel, np.float32, border)
        iane_gb300.convolve(g, to_gpu(kernel), dst, border, method="fft")
        check_fp32(to_host(dst), ref, src_np, kernel, border)
    mask = t.ones_like(dst_big, dtype=t.bool)
    mask[1:8, 1:18, 3:85:2] = False
    assert float(dst_big[mask].abs().max()) == 0.0


def test_fft_auto_picks_one_of_the_two_paths(cuda):
    """`auto` returns bit-for-bit the direct or the spectral result; for a 31^3 kernel on a
    64x128x128 volume the cost model picks the spectral path."""
    rng = np.random.default_rng(21)
    src = to_gpu(rng.random((64, 128, 128), dtype=np.float32))
    kernel = to_gpu((rng.random((31, 31, 31), dtype=np.float32) / 31 ** 3).astype(np.float32))
    outs = {}
    for method in ("direct", "fft", "auto"):
        d = empty_like_np((64, 128, 128), np.float32)
        iane_gb300.convolve(src, kernel, d, "zero", method=method)
        outs[method] = to_host(d)
    assert np.array_equal(outs["auto"], outs["fft"])
    # the direct path sums 29791 taps in FP32 (about 1e-5 of the maximum); the spectral one
    # carries FP64 transforms, so the difference is the direct path's rounding
    assert float(np.max(np.abs(outs["fft"] - outs["direct"]) / np.abs(outs["direct"]).max())) < 3e-5
    small = to_gpu(rng.random((3, 3, 3), dtype=np.float32))
    d1, d2 = empty_like_np((64, 128, 128), np.float32), empty_like_np((64, 128, 128), np.float32)
    iane_gb300.convolve(src, small, d1, "zero", method="auto")
    iane_gb300.convolve(src, small, d2, "zero", method="direct")
    assert np.array_equal(to_host(d1), to_host(d2))


def test_fft_rejects_integer_types_and_exact_mode(cuda):
    a = to_gpu(np.zeros((16, 16), np.uint8))
    k = to_gpu(np.ones((3, 3), np.int32))
    with pytest.raises(iane_gb300.IaneError) as info:
        iane_gb300.convolve(a, k, a.clone(), "zero", method="fft")
    assert info.value.status == iane_gb300.abi.UNSUPPORTED
    f = to_gpu(np.zeros((16, 16), np.float32))
    kf = to_gpu(np.ones((3, 3), np.float32))
    with pytest.raises(iane_gb300.IaneInvalidArgument):
        iane_gb300.convolve(f, kf, f.clone(), "zero", exact=True, method="fft")
