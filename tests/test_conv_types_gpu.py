"""GPU parity for element types beyond f32 on the tiled FP32 path, packed rgb8 pixels and
texture sources, against the oracle and the reference's golden vectors.

Bars: exact mode is bit-identical to the reference; fast mode (FP32 sums) is within 1e-5 of
the reference relative to conv(|src|, |kernel|), plus one unit where an integer destination's
rounding can cross a boundary."""
from __future__ import annotations

import ctypes
import zlib

import numpy as np
import pytest

import iane_gb300
import oracle
from golden_cases import bench_pattern, rgb8_cases
from gpu_helpers import empty_like_np, magnitude, to_gpu, to_host, torch

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5


def random_of(rng, dtype, shape):
    if np.issubdtype(dtype, np.floating):
        return (rng.standard_normal(shape) * 50).astype(dtype)
    info = np.iinfo(dtype)
    return rng.integers(info.min, info.max, shape, dtype=dtype, endpoint=True)


def oracle_conv(src, kernel, out_dtype, border):
    out = np.zeros(src.shape, out_dtype)
    oracle.convolve(np.ascontiguousarray(src), kernel, out, border)
    return out


def assert_fast_close(out, ref, src, kernel, border):
    mag = magnitude(np.ascontiguousarray(src), kernel, border)
    diff = np.abs(out.astype(np.float64) - ref.astype(np.float64))
    slack = FP32_TOL * mag + (1.0 if np.issubdtype(ref.dtype, np.integer) else 0.0)
    assert np.all(diff <= slack), float(np.max(diff - slack))


# --- the tiled FP32 path for every scalar source type ---------------------------------------

TYPE_PAIRS = [(np.uint8, np.uint8), (np.uint8, np.float32), (np.int8, np.int8), (np.uint16, np.uint16),
              (np.int16, np.float32), (np.int32, np.int32), (np.uint32, np.uint32), (np.uint16, np.float64),
              (np.float32, np.int8)]


@pytest.mark.parametrize("border", ["clamp", "zero", "mirror"])
@pytest.mark.parametrize("types", TYPE_PAIRS, ids=lambda t: f"{np.dtype(t[0]).name}-{np.dtype(t[1]).name}")
@pytest.mark.parametrize("shape,kshape", [((70, 131), (9, 9)), ((5, 40, 72), (3, 7, 5)), ((300,), (11,))])
def test_tiled_fast_path_types(cuda, types, shape, kshape, border):
    sd, dd = types
    rng = np.random.default_rng(zlib.crc32(repr((types, shape, border)).encode()))
    src = random_of(rng, sd, shape)
    kernel = (rng.standard_normal(kshape) / np.prod(kshape)).astype(np.float32)
    ref = oracle_conv(src, kernel, dd, border)
    out = empty_like_np(shape, dd)
    iane_gb300.convolve(to_gpu(src), to_gpu(kernel), out, border)
    assert_fast_close(to_host(out), ref, src, kernel, border)
    iane_gb300.convolve(to_gpu(src), to_gpu(kernel), out, border, exact=True)
    assert np.array_equal(to_host(out), ref)


def test_reference_benchmark_tiled_u8_is_bit_exact(cuda):
    # k/64 taps on bytes: every FP32 partial sum is exact, so the fast path equals the
    # reference's double sums whatever the summation order (benchmarks/convolution.cu:84-118)
    image, kernel = bench_pattern(640, 480)
    out = empty_like_np(image.shape, np.uint8)
    iane_gb300.convolve(to_gpu(image), to_gpu(kernel), out, "clamp")
    assert np.array_equal(to_host(out), oracle_conv(image, kernel, np.uint8, "clamp"))


# --- packed rgb8 pixels ----------------------------------------------------------------------

@pytest.mark.parametrize("case", rgb8_cases(), ids=lambda c: c[0])
def test_rgb8_golden(cuda, case):
    name, src, kernel, expected, border = case
    out = torch().zeros(src.shape, dtype=torch().uint8, device="cuda")
    iane_gb300.convolve_rgb8(to_gpu(src), to_gpu(kernel), out, border, exact=True)
    assert np.array_equal(to_host(out), expected), name
    iane_gb300.convolve_rgb8(to_gpu(src), to_gpu(kernel), out, border)
    fast = to_host(out).astype(np.int32)
    if name.startswith("rgb8_bench"):
        assert np.array_equal(fast, expected), name  # k/64 taps: exact FP32 sums
    else:
        assert int(np.max(np.abs(fast - expected.astype(np.int32)))) <= 1, name


@pytest.mark.parametrize("border", ["clamp", "zero", "mirror"])
def test_rgb8_strided_3d(cuda, border):
    t = torch()
    rng = np.random.default_rng(41)
    big = rng.integers(0, 256, (6, 24, 40, 3), dtype=np.uint8)
    src_np = np.ascontiguousarray(big[1:5, 2:22, 3:36])
    kernel = (rng.standard_normal((3, 5, 7)) / 20).astype(np.float32)
    ref = np.zeros_like(src_np)
    oracle.convolve_rgb8(src_np, kernel, ref, border)
    g = to_gpu(big)[1:5, 2:22, 3:36]
    dst_big = t.zeros((6, 24, 80, 3), dtype=t.uint8, device="cuda")
    dst = dst_big[1:5, 2:22, 3:69:2]
    iane_gb300.convolve_rgb8(g, to_gpu(kernel), dst, border, exact=True)
    assert np.array_equal(to_host(dst), ref)
    iane_gb300.convolve_rgb8(g, to_gpu(kernel), dst, border)
    assert int(np.max(np.abs(to_host(dst).astype(np.int32) - ref.astype(np.int32)))) <= 1
    mask = t.ones(dst_big.shape[:3], dtype=t.bool, device="cuda")
    mask[1:5, 2:22, 3:69:2] = False
    assert int(dst_big[mask].max()) == 0


def test_rgb8_refuses_mixed_types(cuda):
    t = torch()
    rgb = t.zeros((8, 8, 3), dtype=t.uint8, device="cuda")
    k = to_gpu(np.ones((3, 3), np.float32))
    ki = to_gpu(np.ones((3, 3), np.int32))
    with pytest.raises(iane_gb300.IaneError) as info:
        iane_gb300.convolve_rgb8(rgb, ki, rgb.clone())
    assert info.value.status == iane_gb300.abi.UNSUPPORTED
    s = iane_gb300.abi.rgb8_view(rgb.data_ptr(), tuple(rgb.shape), tuple(rgb.stride()))
    plain = t.zeros((8, 8), dtype=t.uint8, device="cuda")
    d = iane_gb300.abi.torch_view(plain)
    kv = iane_gb300.abi.torch_view(k)
    status = iane_gb300.lib().iane_gb_convolve(ctypes.byref(s), ctypes.byref(kv), ctypes.byref(d), 0, 0, None)
    assert status == iane_gb300.abi.UNSUPPORTED


# --- texture sources -------------------------------------------------------------------------

def test_texture_convolution_matches_cpu_for_both_borders(cuda):
    # test/unit/algorithms/test_convolution_cuda.cu:53-86: a 5x4 float texture, a 3x3 crop
    # at (1, 1) and a 3x3 kernel; the texture result equals the CPU convolution of the crop
    source = (np.arange(20, dtype=np.float32) - 6).reshape(4, 5)
    kernel = ((np.arange(9, dtype=np.float32) - 3) / 8).reshape(3, 3)
    tex = iane_gb300.Texture(source.shape, source.dtype).upload(source)
    view = tex.view().subview((1, 1), (3, 3))
    for border in ("clamp", "zero"):
        expected = oracle_conv(source[1:4, 1:4], kernel, np.float32, border)
        for exact in (False, True):
            out = empty_like_np((3, 3), np.float32)
            iane_gb300.convolve(view, to_gpu(kernel), out, border, exact=exact)
            assert np.array_equal(to_host(out), expected), (border, exact)
    tex.close()


TEXEL_TYPES = [np.uint8, np.int8, np.uint16, np.int16, np.int32, np.uint32, np.float32]


@pytest.mark.parametrize("rank", [1, 2, 3])
@pytest.mark.parametrize("dtype", TEXEL_TYPES, ids=lambda d: np.dtype(d).name)
def test_texture_source_parity(cuda, dtype, rank):
    rng = np.random.default_rng(zlib.crc32(repr((np.dtype(dtype).name, rank)).encode()))
    full_shape = {1: (150,), 2: (37, 90), 3: (9, 30, 44)}[rank]
    origin = {1: (7,), 2: (3, 11), 3: (1, 4, 6)}[rank]
    shape = {1: (120,), 2: (30, 70), 3: (7, 22, 35)}[rank]
    kshape = {1: (9,), 2: (5, 7), 3: (3, 5, 3)}[rank]
    data = random_of(rng, dtype, full_shape)
    # device upload for even ranks, host upload for odd ones: both of the reference's paths
    tex = iane_gb300.Texture(full_shape, np.dtype(dtype).name)
    tex.upload(to_gpu(data) if rank % 2 == 0 else data)
    view = tex.view().subview(origin, shape)
    crop = np.ascontiguousarray(data[tuple(slice(o, o + n) for o, n in zip(origin, shape))])
    kernel = (rng.standard_normal(kshape) / np.prod(kshape)).astype(np.float32)
    out_dtype = np.float32 if dtype == np.float32 else dtype
    for border in ("clamp", "zero", "mirror"):
        ref = oracle_conv(crop, kernel, out_dtype, border)
        out = empty_like_np(shape, out_dtype)
        iane_gb300.convolve(view, to_gpu(kernel), out, border, exact=True)
        assert np.array_equal(to_host(out), ref), border
        iane_gb300.convolve(view, to_gpu(kernel), out, border)
        assert_fast_close(to_host(out), ref, crop, kernel, border)
    if dtype != np.float32:
        ki = rng.integers(-3, 4, kshape).astype(np.int32)
        ref = oracle_conv(crop, ki, out_dtype, "zero")
        out = empty_like_np(shape, out_dtype)
        iane_gb300.convolve(view, to_gpu(ki), out, "zero")
        assert np.array_equal(to_host(out), ref)
    tex.close()


def test_texture_upload_from_padded_rows(cuda):
    t = torch()
    rng = np.random.default_rng(12)
    big = rng.random((5, 20, 64), dtype=np.float32)
    dev = to_gpu(big)[:, 2:18, 0:50]  # contiguous rows, padded rows and planes
    tex = iane_gb300.Texture((5, 16, 50), "float32").upload(dev)
    out = t.zeros((5, 16, 50), device="cuda")
    iane_gb300.convolve(tex.view(), to_gpu(np.ones((1, 1, 1), np.float32)), out, "zero", exact=True)
    assert np.array_equal(to_host(out), big[:, 2:18, 0:50])
    tex.close()


def test_texture_errors(cuda):
    tex = iane_gb300.Texture((4, 6), "float32").upload(np.zeros((4, 6), np.float32))
    k = to_gpu(np.ones((3, 3), np.float32))
    out = empty_like_np((3, 3), np.float32)
    outside = iane_gb300.TextureView(tex, (2, 4), (3, 3))
    with pytest.raises(iane_gb300.IaneInvalidArgument):
        iane_gb300.convolve(outside, k, out)
    with pytest.raises(iane_gb300.IaneError) as info:
        iane_gb300.convolve(tex.view().subview((0, 0), (3, 3)), k, out, method="fft")
    assert info.value.status == iane_gb300.abi.UNSUPPORTED
    with pytest.raises(iane_gb300.IaneInvalidArgument):
        tex.upload(np.zeros((4, 5), np.float32))
    with pytest.raises(iane_gb300.IaneInvalidArgument):
        tex.upload(np.zeros((4, 6), np.int32))
    with pytest.raises(TypeError):
        iane_gb300.Texture((4, 4), "float64")
    tex.close()
    # an empty texture allocates nothing; convolving its empty view does nothing
    empty = iane_gb300.Texture((0, 3), "float32")
    assert empty.handle == 0
    iane_gb300.convolve(empty.view(), k, empty_like_np((0, 3), np.float32))
    empty.close()


# --- single-plane kernels on large images (at least 2 x SMs 64x64 tiles) --------------------

@pytest.mark.parametrize("border", ["clamp", "zero", "mirror"])
@pytest.mark.parametrize("case", ["f32_tma", "f32_strided", "u8_narrow", "u16_narrow", "i32_copy", "texture_u8",
                                  "f32_3d_plane_kernel"])
def test_large_single_plane_parity(cuda, case, border):
    """Large 2-D images (and a 3-D volume with a one-plane kernel) take the single-plane
    64x64-tile kernels (direct summation): every staging mode against the oracle."""
    t = torch()
    rng = np.random.default_rng(zlib.crc32(repr((case, border)).encode()))
    shape = (8, 640, 700) if case == "f32_3d_plane_kernel" else (1100, 1500)
    kshape = (1, 9, 7) if case == "f32_3d_plane_kernel" else (7, 13)
    kernel = (rng.standard_normal(kshape) / np.prod(kshape)).astype(np.float32)
    dtype = {"u8_narrow": np.uint8, "texture_u8": np.uint8, "u16_narrow": np.uint16, "i32_copy": np.int32}.get(case,
                                                                                                        np.float32)
    src = random_of(rng, dtype, shape)
    out_dtype = np.float32
    ref = oracle_conv(src, kernel, out_dtype, border)
    out = empty_like_np(shape, out_dtype)
    if case == "texture_u8":
        tex = iane_gb300.Texture(shape, "uint8").upload(src)
        source = tex.view()
    elif case == "f32_strided":
        big = to_gpu(np.zeros((shape[0], shape[1] + 40), np.float32))
        big[:, 13:13 + shape[1]] = to_gpu(src)
        source = big[:, 13:13 + shape[1]]
    else:
        source = to_gpu(src)
    iane_gb300.convolve(source, to_gpu(kernel), out, border)
    assert_fast_close(to_host(out), ref, src, kernel, border)
    if case == "texture_u8":
        tex.close()
    del t
