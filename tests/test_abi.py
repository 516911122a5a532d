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


def test_wait_probe_checks_its_limit_before_any_launch():
    lib = iane_gb300.lib()
    for bad in (0, 10000001):
        assert lib.iane_gb_wait_probe(bad, None) == iane_gb300.abi.INVALID_ARGUMENT
