"""Loader for ``libiane_gb300.so`` (the C ABI in ``include/iane_gb/capi.h``).

There is no fallback: if the library is missing or fails to load, every entry point
raises. Build it with ``python -m iane_gb300.build``.
"""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

from . import abi

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libiane_gb300.so"
HEADER = HERE.parent / "include" / "iane_gb" / "capi.h"

_VIEW_P = ctypes.POINTER(abi.View)
_lib = None


class IaneError(RuntimeError):
    """A negative status from the C ABI; ``status`` holds the code."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status}: {abi.STATUS_NAMES.get(status, 'unknown')})")
        self.status = status


class IaneInvalidArgument(IaneError, ValueError):
    """The reference throws std::invalid_argument for these."""


class IaneLengthError(IaneError, ValueError):
    """The reference throws std::length_error for an undersized scratch reservation."""


def header_functions() -> list[str]:
    """Names of the functions ``capi.h`` declares."""
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|size_t)\s+(iane_gb_\w+)\s*\(", text, flags=re.M)))


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m iane_gb300.build`")
    l = ctypes.CDLL(str(LIB_PATH))
    vp, cvp, i32p = ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)
    l.iane_gb_abi_version.argtypes = []
    l.iane_gb_abi_version.restype = ctypes.c_int
    l.iane_gb_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    l.iane_gb_last_error.restype = ctypes.c_size_t
    l.iane_gb_device_status.argtypes = [vp]
    l.iane_gb_device_status.restype = ctypes.c_int
    l.iane_gb_wait_probe.argtypes = [ctypes.c_uint, ctypes.c_int, vp]
    l.iane_gb_wait_probe.restype = ctypes.c_int
    l.iane_gb_fp32_peak_probe.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double), vp]
    l.iane_gb_fp32_peak_probe.restype = ctypes.c_int
    l.iane_gb_convolve.argtypes = [_VIEW_P, _VIEW_P, _VIEW_P, ctypes.c_int, ctypes.c_uint, vp]
    l.iane_gb_convolve.restype = ctypes.c_int
    l.iane_gb_convolve_separable.argtypes = [_VIEW_P, ctypes.POINTER(_VIEW_P), _VIEW_P, ctypes.c_int, vp]
    l.iane_gb_convolve_separable.restype = ctypes.c_int
    l.iane_gb_rl_prepare.argtypes = [_VIEW_P, ctypes.c_int, i32p, vp, ctypes.POINTER(vp)]
    l.iane_gb_rl_prepare.restype = ctypes.c_int
    l.iane_gb_rl_prepare_ex.argtypes = [_VIEW_P, ctypes.c_int, i32p, ctypes.c_uint, vp, ctypes.POINTER(vp)]
    l.iane_gb_rl_prepare_ex.restype = ctypes.c_int
    l.iane_gb_rl_scratch_bytes.argtypes = [cvp]
    l.iane_gb_rl_scratch_bytes.restype = ctypes.c_size_t
    l.iane_gb_rl_run.argtypes = [vp, _VIEW_P, _VIEW_P, ctypes.c_int, ctypes.c_float, ctypes.c_int, vp,
                                 ctypes.c_size_t, vp, vp]
    l.iane_gb_rl_run.restype = ctypes.c_int
    l.iane_gb_rl_host_scratch_bytes.argtypes = [cvp, ctypes.c_int]
    l.iane_gb_rl_host_scratch_bytes.restype = ctypes.c_size_t
    l.iane_gb_rl_run_host.argtypes = [vp, vp, ctypes.c_int, vp, ctypes.c_int, ctypes.c_float, ctypes.c_int, vp,
                                      ctypes.c_size_t, vp]
    l.iane_gb_rl_run_host.restype = ctypes.c_int
    l.iane_gb_rl_run_noalloc.argtypes = [_VIEW_P, _VIEW_P, _VIEW_P, ctypes.c_int, ctypes.c_float, ctypes.c_int, vp]
    l.iane_gb_rl_run_noalloc.restype = ctypes.c_int
    l.iane_gb_rl_batch_prepare.argtypes = [_VIEW_P, ctypes.c_int, i32p, ctypes.c_uint, vp, ctypes.POINTER(vp)]
    l.iane_gb_rl_batch_prepare.restype = ctypes.c_int
    l.iane_gb_rl_batch_scratch_bytes.argtypes = [cvp]
    l.iane_gb_rl_batch_scratch_bytes.restype = ctypes.c_size_t
    l.iane_gb_rl_batch_tiles.argtypes = [cvp, i32p]
    l.iane_gb_rl_batch_tiles.restype = ctypes.c_int
    l.iane_gb_rl_batch_config.argtypes = [cvp, i32p, i32p, i32p]
    l.iane_gb_rl_batch_config.restype = ctypes.c_int
    l.iane_gb_rl_batch_configure.argtypes = [cvp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    l.iane_gb_rl_batch_configure.restype = ctypes.c_int
    l.iane_gb_rl_batch_run.argtypes = [vp, _VIEW_P, _VIEW_P, ctypes.c_int, ctypes.c_float, ctypes.c_int, vp,
                                       ctypes.c_size_t, vp]
    l.iane_gb_rl_batch_run.restype = ctypes.c_int
    l.iane_gb_rl_batch_destroy.argtypes = [vp]
    l.iane_gb_rl_batch_destroy.restype = ctypes.c_int
    sz, ll, f, i = ctypes.c_size_t, ctypes.c_longlong, ctypes.c_float, ctypes.c_int
    l.iane_gb_cnn_conv3.argtypes = [vp, i, vp, i, i, i, i, vp, vp, i, vp, vp, vp, i, vp, vp]
    l.iane_gb_cnn_wgrad_scratch_bytes.argtypes = [i, i, i, i, i, i]
    l.iane_gb_cnn_wgrad_scratch_bytes.restype = sz
    l.iane_gb_cnn_conv3_wgrad.argtypes = [vp, i, vp, i, i, i, i, vp, i, vp, vp, vp, sz, vp]
    l.iane_gb_cnn_flip.argtypes = [vp, i, i, vp, vp]
    l.iane_gb_cnn_pool2.argtypes = [vp, i, i, i, i, vp, vp]
    l.iane_gb_cnn_pool2_grad.argtypes = [vp, i, i, i, i, vp, vp, i, vp]
    l.iane_gb_cnn_up2.argtypes = [vp, i, i, i, i, vp, vp]
    l.iane_gb_cnn_up2_grad.argtypes = [vp, i, i, i, i, vp, vp, vp]
    l.iane_gb_cnn_mse.argtypes = [vp, vp, ll, vp, vp, vp]
    l.iane_gb_cnn_adam.argtypes = [vp, vp, vp, vp, vp, ll, f, f, f, f, i, f, vp]
    l.iane_gb_cnn_tc_packed_bytes.argtypes = [i, i, i]
    l.iane_gb_cnn_tc_packed_bytes.restype = sz
    l.iane_gb_cnn_tc_pack.argtypes = [vp, i, i, i, vp, vp]
    l.iane_gb_cnn_conv3_tc.argtypes = [vp, i, vp, i, i, i, i, vp, vp, i, vp, vp, vp, i, vp]
    for name in ("conv3", "conv3_wgrad", "flip", "pool2", "pool2_grad", "up2", "up2_grad", "mse", "adam", "tc_pack",
                 "conv3_tc"):
        getattr(l, "iane_gb_cnn_" + name).restype = ctypes.c_int
    l.iane_gb_rl_destroy.argtypes = [vp]
    l.iane_gb_rl_destroy.restype = ctypes.c_int
    u64 = ctypes.c_uint64
    l.iane_gb_texture_create.argtypes = [i, i, i32p, ctypes.POINTER(u64)]
    l.iane_gb_texture_upload.argtypes = [u64, _VIEW_P, vp]
    l.iane_gb_texture_destroy.argtypes = [u64]
    l.iane_gb_convolve_texture.argtypes = [ctypes.POINTER(abi.TextureView), _VIEW_P, _VIEW_P, i, ctypes.c_uint, vp]
    u8p = ctypes.c_void_p
    l.iane_gb_morphology.argtypes = [_VIEW_P, _VIEW_P, i32p, u8p, i, i, vp]
    l.iane_gb_morphology.restype = ctypes.c_int
    l.iane_gb_morphology_scratch_bytes.argtypes = [i, i, i32p]
    l.iane_gb_morphology_scratch_bytes.restype = sz
    l.iane_gb_morphology_compound.argtypes = [_VIEW_P, _VIEW_P, i32p, u8p, i, i, vp, sz, vp]
    l.iane_gb_morphology_compound.restype = ctypes.c_int
    l.iane_gb_wiener_prepare.argtypes = [_VIEW_P, i, i32p, f, vp, ctypes.POINTER(vp)]
    l.iane_gb_wiener_scratch_bytes.argtypes = [cvp]
    l.iane_gb_wiener_scratch_bytes.restype = sz
    l.iane_gb_wiener_run.argtypes = [vp, _VIEW_P, _VIEW_P, vp, sz, vp]
    l.iane_gb_wiener_destroy.argtypes = [vp]
    for name in ("wiener_prepare", "wiener_run", "wiener_destroy"):
        getattr(l, "iane_gb_" + name).restype = ctypes.c_int
    for name in ("texture_create", "texture_upload", "texture_destroy", "convolve_texture"):
        getattr(l, "iane_gb_" + name).restype = ctypes.c_int
    if l.iane_gb_abi_version() != abi.ABI_VERSION:
        raise RuntimeError("libiane_gb300.so ABI version mismatch; rebuild it")
    _lib = l
    return l


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    lib().iane_gb_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int) -> None:
    if status == abi.OK:
        return
    message = last_error()
    if status == abi.INVALID_ARGUMENT:
        raise IaneInvalidArgument(status, message)
    if status == abi.LENGTH_ERROR:
        raise IaneLengthError(status, message)
    raise IaneError(status, message)
