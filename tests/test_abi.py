"""The C-ABI library loads and exports every entry point include/iane_gb/capi.h declares,
and rejects bad arguments on the host before touching a GPU."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import iane_gb300
from iane_gb300 import _lib, abi


def test_library_exports_every_declared_symbol():
    lib = _lib.lib()
    declared = _lib.header_functions()
    assert len(declared) >= 10
    missing = [name for name in declared if not hasattr(lib, name)]
    assert not missing, missing


def test_abi_version():
    assert _lib.lib().iane_gb_abi_version() == abi.ABI_VERSION


def _host_view(arr):
    # Host pointers are fine here: every case fails validation before any CUDA call.
    return abi.numpy_view(arr)


def _call_convolve(src, kernel, dst, border=abi.BORDER_CLAMP, flags=0):
    s, k, d = _host_view(src), _host_view(kernel), _host_view(dst)
    return _lib.lib().iane_gb_convolve(ctypes.byref(s), ctypes.byref(k), ctypes.byref(d), border, flags, None)


def test_even_kernel_is_invalid_argument():
    a = np.zeros((4, 4), np.float32)
    status = _call_convolve(a, np.zeros((2, 3), np.float32), a.copy())
    assert status == abi.INVALID_ARGUMENT
    assert "odd" in _lib.last_error()


def test_mismatched_extents_are_invalid_argument():
    status = _call_convolve(np.zeros((4, 4), np.float32), np.zeros((3, 3), np.float32), np.zeros((4, 5), np.float32))
    assert status == abi.INVALID_ARGUMENT
    assert "matching" in _lib.last_error()


def test_rank_mismatch_and_bad_border_and_flags():
    a = np.zeros((4, 4), np.float32)
    assert _call_convolve(a, np.zeros((3,), np.float32), a.copy()) == abi.INVALID_ARGUMENT
    assert _call_convolve(a, np.zeros((3, 3), np.float32), a.copy(), border=7) == abi.INVALID_ARGUMENT
    assert _call_convolve(a, np.zeros((3, 3), np.float32), a.copy(), flags=8) == abi.INVALID_ARGUMENT


def test_unsupported_kernel_type():
    a = np.zeros((4, 4), np.float32)
    assert _call_convolve(a, np.zeros((3, 3), np.uint8), a.copy()) == abi.UNSUPPORTED


def test_empty_image_is_a_no_op():
    a = np.zeros((0, 5), np.float32)
    assert _call_convolve(a, np.zeros((3, 3), np.float32), a.copy()) == abi.OK


def test_null_view_and_rank_four():
    lib = _lib.lib()
    k = _host_view(np.zeros((3,), np.float32))
    assert lib.iane_gb_convolve(None, ctypes.byref(k), ctypes.byref(k), 0, 0, None) == abi.INVALID_ARGUMENT
    v = abi.View()
    v.rank = 4
    v.dtype = abi.F32
    assert lib.iane_gb_convolve(ctypes.byref(v), ctypes.byref(v), ctypes.byref(v), 0, 0, None) == abi.UNSUPPORTED


def test_python_layer_raises_typed_errors():
    with pytest.raises(iane_gb300.IaneInvalidArgument):
        _lib.check(abi.INVALID_ARGUMENT)
    with pytest.raises(iane_gb300.IaneLengthError):
        _lib.check(abi.LENGTH_ERROR)


def test_rl_prepare_rejects_even_psf_without_gpu():
    lib = _lib.lib()
    psf = _host_view(np.zeros((4, 3), np.float32))
    ext = (ctypes.c_int32 * 3)(8, 8, 1)
    handle = ctypes.c_void_p()
    assert lib.iane_gb_rl_prepare(ctypes.byref(psf), 2, ext, None, ctypes.byref(handle)) == abi.INVALID_ARGUMENT
    assert not handle.value


def test_wait_probe_checks_its_limit_and_kind_before_any_launch():
    lib = iane_gb300.lib()
    for bad in (0, 10000001):
        assert lib.iane_gb_wait_probe(bad, 0, None) == iane_gb300.abi.INVALID_ARGUMENT
    for kind in (-1, 3):
        assert lib.iane_gb_wait_probe(1000, kind, None) == iane_gb300.abi.INVALID_ARGUMENT


def test_rgb8_and_texture_argument_checks():
    lib = _lib.lib()
    rgb = np.zeros((4, 5, 3), np.uint8)
    s = abi.rgb8_view(rgb.ctypes.data, rgb.shape, rgb.strides)
    plain = np.zeros((4, 5), np.uint8)
    k = _host_view(np.ones((3, 3), np.float32))
    d = _host_view(plain)
    # rgb8 needs an rgb8 destination
    assert lib.iane_gb_convolve(ctypes.byref(s), ctypes.byref(k), ctypes.byref(d), 0, 0, None) == abi.UNSUPPORTED
    # texture creation: texel types and ranks; an empty texture needs no device
    handle = ctypes.c_uint64(7)
    ext = (ctypes.c_int32 * 3)(4, 4, 1)
    assert lib.iane_gb_texture_create(abi.F64, 2, ext, ctypes.byref(handle)) == abi.UNSUPPORTED
    assert lib.iane_gb_texture_create(abi.F32, 4, ext, ctypes.byref(handle)) == abi.UNSUPPORTED
    neg = (ctypes.c_int32 * 3)(4, -1, 1)
    assert lib.iane_gb_texture_create(abi.F32, 2, neg, ctypes.byref(handle)) == abi.INVALID_ARGUMENT
    empty = (ctypes.c_int32 * 3)(0, 4, 1)
    assert lib.iane_gb_texture_create(abi.U8, 2, empty, ctypes.byref(handle)) == abi.OK
    assert handle.value == 0
    assert lib.iane_gb_texture_destroy(0) == abi.OK
    assert lib.iane_gb_convolve_texture(None, ctypes.byref(k), ctypes.byref(d), 0, 0, None) == abi.INVALID_ARGUMENT
    assert lib.iane_gb_texture_upload(12345, ctypes.byref(d), None) == abi.INVALID_ARGUMENT


def test_morphology_argument_checks():
    lib = _lib.lib()
    a = np.zeros((6, 7), np.float32)
    s, d = _host_view(a), _host_view(a.copy())
    bad = (ctypes.c_int32 * 3)(-1, 1, 0)
    assert lib.iane_gb_morphology(ctypes.byref(s), ctypes.byref(d), bad, None, abi.ERODE, 0, None) == abi.INVALID_ARGUMENT
    ok = (ctypes.c_int32 * 3)(1, 1, 0)
    assert lib.iane_gb_morphology(ctypes.byref(s), ctypes.byref(d), ok, None, 7, 0, None) == abi.INVALID_ARGUMENT
    assert lib.iane_gb_morphology(ctypes.byref(s), ctypes.byref(d), ok, None, abi.OPENING, 0, None) == \
        abi.INVALID_ARGUMENT
    other = _host_view(np.zeros((6, 7), np.float64))
    assert lib.iane_gb_morphology(ctypes.byref(s), ctypes.byref(other), ok, None, abi.ERODE, 0, None) == \
        abi.INVALID_ARGUMENT
    ext = (ctypes.c_int32 * 3)(7, 6, 1)
    assert lib.iane_gb_morphology_scratch_bytes(abi.F32, 2, ext) == 2 * ((7 * 6 * 4 + 255) // 256 * 256)


def test_wiener_argument_checks():
    lib = _lib.lib()
    psf = _host_view(np.ones((3, 3), np.float32))
    ext = (ctypes.c_int32 * 3)(16, 16, 1)
    plan = ctypes.c_void_p()
    for noise in (0.0, -1.0, float("nan"), float("inf")):
        assert lib.iane_gb_wiener_prepare(ctypes.byref(psf), 2, ext, noise, None, ctypes.byref(plan)) == \
            abi.INVALID_ARGUMENT
        assert "Noise must be finite and positive" in _lib.last_error()
    small = (ctypes.c_int32 * 3)(2, 16, 1)
    assert lib.iane_gb_wiener_prepare(ctypes.byref(psf), 2, small, 0.01, None, ctypes.byref(plan)) == \
        abi.INVALID_ARGUMENT
    assert "PSF must fit inside the input image" in _lib.last_error()
    assert lib.iane_gb_wiener_run(None, None, None, None, 0, None) == abi.INVALID_ARGUMENT
