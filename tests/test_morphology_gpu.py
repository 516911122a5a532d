"""Flat morphology on the GPU: bit-identical (NaN and signed zeros included) to the reference's
erode / dilate, through its golden vectors and the oracle."""
from __future__ import annotations

import zlib

import numpy as np
import pytest

import iane_gb300
import oracle
from golden_cases import morph_cases
from gpu_helpers import empty_like_np, to_gpu, to_host, torch

pytestmark = pytest.mark.gpu


def run_gpu(src, radius, op, border, mask=None):
    out = empty_like_np(src.shape, src.dtype)
    fp = None if mask is None else to_gpu(mask.astype(np.uint8))
    iane_gb300.morphology(to_gpu(src), out, radius, op, border, fp)
    return to_host(out)


def test_known_answers(cuda):
    # test/unit/algorithms/color_morphology_cases.hpp:87-117 (a crop of a 6-element image)
    t = torch()
    src = to_gpu(np.array([99, 3, 1, 5, 2, 99], np.int32))[1:5]
    out = t.zeros(4, dtype=t.int32, device="cuda")
    forward = to_gpu(np.array([0, 0, 1], np.uint8))
    for op, fp, border, want in (("erode", None, "clamp", [1, 1, 1, 2]), ("dilate", None, "clamp", [3, 5, 5, 5]),
                                 ("erode", forward, "zero", [1, 5, 2, 0]), ("dilate", forward, "zero", [0, 3, 1, 5])):
        iane_gb300.morphology(src, out, (1,), op, border, fp)
        assert to_host(out).tolist() == want, (op, border)


@pytest.mark.parametrize("case", morph_cases(), ids=lambda c: c[0])
def test_golden(cuda, case):
    name, src, radius, op, border, mask, expected = case
    assert run_gpu(src, radius, op, border, mask).tobytes() == expected.tobytes(), name


TYPES = [np.uint8, np.int8, np.uint16, np.int16, np.int32, np.uint32, np.float32, np.float64]


@pytest.mark.parametrize("dtype", TYPES, ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("shape,radius", [((200,), (5,)), ((37, 70), (2, 3)), ((9, 40, 45), (1, 2, 3)),
                                          ((3, 5, 4), (2, 0, 4)), ((64, 300), (40, 1))])
def test_box_parity(cuda, dtype, shape, radius):
    rng = np.random.default_rng(zlib.crc32(repr((np.dtype(dtype).name, shape)).encode()))
    if np.issubdtype(dtype, np.floating):
        src = rng.standard_normal(shape).astype(dtype)
        src[rng.random(shape) < 0.05] = np.nan
        src[rng.random(shape) < 0.05] = 0.0
        src[rng.random(shape) < 0.05] = -0.0
    else:
        info = np.iinfo(dtype)
        src = rng.integers(info.min, info.max, shape, dtype=dtype, endpoint=True)
    for op in ("erode", "dilate"):
        for border in ("clamp", "zero", "mirror"):
            ref = np.zeros_like(src)
            oracle.morphology(src, ref, radius, op, border)
            assert run_gpu(src, radius, op, border).tobytes() == ref.tobytes(), (op, border)


@pytest.mark.parametrize("shape,radius", [((30, 41), (2, 3)), ((7, 12, 15), (1, 2, 1))])
def test_masked_footprints(cuda, shape, radius):
    rng = np.random.default_rng(len(shape))
    src = rng.integers(0, 1000, shape).astype(np.int32)
    mask = rng.random(tuple(2 * r + 1 for r in radius)) < 0.4
    for op in ("erode", "dilate"):
        for border in ("clamp", "zero", "mirror"):
            ref = np.zeros_like(src)
            oracle.morphology(src, ref, radius, op, border, mask)
            assert np.array_equal(run_gpu(src, radius, op, border, mask), ref), (op, border)


@pytest.mark.parametrize("op", ["opening", "closing"])
def test_compound_in_place_and_strided(cuda, op):
    t = torch()
    rng = np.random.default_rng(3)
    big = rng.integers(0, 256, (10, 40, 60), dtype=np.uint8)
    src_np = np.ascontiguousarray(big[1:9, 3:37, 5:55])
    ref = np.zeros_like(src_np)
    oracle.morphology(src_np, ref, (1, 2, 2), op, "clamp")
    g = to_gpu(big)
    view = g[1:9, 3:37, 5:55]
    iane_gb300.morphology(view, view, (1, 2, 2), op, "clamp")  # in place on a strided crop
    assert np.array_equal(to_host(view), ref)
    assert np.array_equal(to_host(g)[0], big[0])  # outside the crop untouched
    # the reference's 4-D slab-and-impulse case, in 3-D
    img = np.zeros((3, 3, 4), np.int32)
    img[:, :, :2] = 1
    img[1, 1, 3] = 1
    close = op == "closing"
    if close:
        img = 1 - img
    out = empty_like_np(img.shape, np.int32)
    iane_gb300.morphology(to_gpu(img), out, (1, 1, 1), op)
    want = np.zeros_like(img)
    want[:, :, :2] = 1
    assert np.array_equal(to_host(out), 1 - want if close else want)
    del t


def test_errors(cuda):
    a = to_gpu(np.zeros((8, 8), np.float32))
    with pytest.raises(iane_gb300.IaneInvalidArgument):
        iane_gb300.morphology(a, a.clone(), (-1, 1))
    with pytest.raises(iane_gb300.IaneInvalidArgument):
        iane_gb300.morphology(a, to_gpu(np.zeros((8, 8), np.float64)), (1, 1))
    with pytest.raises(iane_gb300.IaneError) as info:
        iane_gb300.morphology(a, a.clone(), (600, 600), footprint=None)  # direct-kernel work bound
    assert info.value.status == iane_gb300.abi.UNSUPPORTED
    with pytest.raises(iane_gb300.IaneError):
        iane_gb300.morphology(to_gpu(np.zeros((8, 8), np.float32)).bfloat16(), a.clone().bfloat16(), (1, 1))


@pytest.mark.parametrize("radius", [1, 2, 3])
@pytest.mark.parametrize("dtype", [np.uint8, np.int16, np.uint32, np.float32, np.float64], ids=lambda d: np.dtype(d).name)
def test_cube_footprints(cuda, dtype, radius):
    """Equal radii on all three axes take the unrolled kernel with the z window in registers;
    several z chunks (the volume is deeper than one chunk), NaN and signed zeros included."""
    rng = np.random.default_rng(zlib.crc32(repr((np.dtype(dtype).name, radius)).encode()))
    shape = (45, 37, 70)
    if np.issubdtype(dtype, np.floating):
        src = rng.standard_normal(shape).astype(dtype)
        src[rng.random(shape) < 0.05] = np.nan
        src[rng.random(shape) < 0.05] = 0.0
        src[rng.random(shape) < 0.05] = -0.0
    else:
        info = np.iinfo(dtype)
        src = rng.integers(info.min, info.max, shape, dtype=dtype, endpoint=True)
    r = (radius,) * 3
    for op in ("erode", "dilate"):
        for border in ("clamp", "zero", "mirror"):
            ref = np.zeros_like(src)
            oracle.morphology(src, ref, r, op, border)
            assert run_gpu(src, r, op, border).tobytes() == ref.tobytes(), (op, border)


@pytest.mark.parametrize("radius", [1, 2, 3])
def test_cube_footprints_on_strided_views(cuda, radius):
    """The cube kernel's per-block staging offsets on a cropped view with an x stride of two
    elements, all three borders."""
    t = torch()
    rng = np.random.default_rng(100 + radius)
    big = rng.standard_normal((44, 33, 140)).astype(np.float32)
    big[rng.random(big.shape) < 0.03] = np.nan
    crop = (slice(2, 40), slice(3, 30), slice(1, 130, 2))
    src = np.ascontiguousarray(big[crop])
    g = to_gpu(big)
    r = (radius,) * 3
    for op in ("erode", "dilate"):
        for border in ("clamp", "zero", "mirror"):
            ref = np.zeros_like(src)
            oracle.morphology(src, ref, r, op, border)
            out = t.zeros((44, 33, 140), dtype=t.float32, device="cuda")
            iane_gb300.morphology(g[crop], out[crop], r, op, border)
            assert to_host(out[crop]).tobytes() == ref.tobytes(), (op, border)


def test_cube_footprint_with_a_plane_beyond_31_bit_offsets(cuda):
    """A view whose plane spans more than 2^31 bytes (two rows 2^31 + 4 KiB apart) takes the
    general fused 3-D kernel; the result is the same."""
    t = torch()
    row = (1 << 29) + 1024  # elements between the two rows: 2^31 + 4 KiB
    buf = t.zeros(row + 3 * 64 + 64, dtype=t.float32, device="cuda")
    rng = np.random.default_rng(7)
    vals = rng.standard_normal((3, 2, 64)).astype(np.float32)
    view = buf.as_strided((3, 2, 64), (64, row, 1))
    view.copy_(t.from_numpy(vals).cuda())
    out = t.zeros((3, 2, 64), dtype=t.float32, device="cuda")
    for op in ("erode", "dilate"):
        ref = np.zeros_like(vals)
        oracle.morphology(vals, ref, (1, 1, 1), op, "clamp")
        iane_gb300.morphology(view, out, (1, 1, 1), op, "clamp")
        assert to_host(out).tobytes() == ref.tobytes(), op
    del buf
