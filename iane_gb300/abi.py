"""ctypes mirror of ``include/iane_gb/capi.h``: the view descriptor, codes and constants.

Pure data definitions; loading the CUDA library happens in ``iane_gb300._lib``.

Axis order: IANE views put axis 0 fastest (reference include/iane/resource/packed_layout.hpp:10-34).
A C-ordered array of shape ``(nz, ny, nx)`` is therefore the IANE view with extents
``[nx, ny, nz]`` and byte strides ``[s_x, s_y, s_z]`` -- the reversed shape and strides.
"""
from __future__ import annotations

import ctypes

ABI_VERSION = 2
MAX_RANK = 3

U8, U16, I16, I32, F32, F64, BF16, I8, U32, RGB8 = 1, 2, 3, 4, 5, 6, 7, 8, 9, 10
DTYPE_SIZE = {U8: 1, U16: 2, I16: 2, I32: 4, F32: 4, F64: 8, BF16: 2, I8: 1, U32: 4, RGB8: 3}
TEXEL_DTYPES = (U8, I8, U16, I16, I32, U32, F32)

BORDER_CLAMP, BORDER_ZERO, BORDER_MIRROR = 0, 1, 2
BORDERS = {"clamp": BORDER_CLAMP, "zero": BORDER_ZERO, "mirror": BORDER_MIRROR}

ACC_FAST, ACC_EXACT = 0, 1
CONV_FFT, CONV_AUTO = 2, 4

RL_INIT_OBSERVED, RL_INIT_MEAN, RL_INIT_GIVEN = 0, 1, 2
ERODE, DILATE, OPENING, CLOSING = 0, 1, 2, 3
MORPHOLOGY_OPS = {"erode": ERODE, "dilate": DILATE, "opening": OPENING, "closing": CLOSING}
RL_BF16_TENSOR = 1
RL_PER_PASS = 2
PROBE_MBARRIER = 0
PROBE_COUNTER = 1
PROBE_COUNTER_ABORT = 2
BATCH_AUTOTUNE = 1

OK = 0
INVALID_ARGUMENT = -1
UNSUPPORTED = -2
CUDA_ERROR = -3
DEVICE_TIMEOUT = -4
OUT_OF_MEMORY = -5
LENGTH_ERROR = -6

STATUS_NAMES = {
    INVALID_ARGUMENT: "invalid argument",
    UNSUPPORTED: "unsupported",
    CUDA_ERROR: "CUDA error",
    DEVICE_TIMEOUT: "device timeout",
    OUT_OF_MEMORY: "out of memory",
    LENGTH_ERROR: "scratch too small",
}

_NUMPY_DTYPES = {
    "uint8": U8, "uint16": U16, "int16": I16, "int32": I32, "float32": F32, "float64": F64,
    "int8": I8, "uint32": U32,
}
_TORCH_DTYPES = {
    "torch.uint8": U8, "torch.uint16": U16, "torch.int16": I16, "torch.int32": I32,
    "torch.float32": F32, "torch.float64": F64, "torch.bfloat16": BF16, "torch.int8": I8,
    "torch.uint32": U32,
}


class View(ctypes.Structure):
    _fields_ = [
        ("ptr", ctypes.c_void_p),
        ("dtype", ctypes.c_int32),
        ("rank", ctypes.c_int32),
        ("extent", ctypes.c_int32 * 3),
        ("reserved", ctypes.c_int32),
        ("stride", ctypes.c_int64 * 3),
    ]


class TextureView(ctypes.Structure):
    _fields_ = [
        ("texture", ctypes.c_uint64),
        ("dtype", ctypes.c_int32),
        ("rank", ctypes.c_int32),
        ("extent", ctypes.c_int32 * 3),
        ("origin", ctypes.c_int32 * 3),
    ]


def make_view(ptr: int, dtype: int, shape, strides_bytes) -> View:
    """Build a view from a C-ordered shape/strides (slowest axis first)."""
    rank = len(shape)
    if not 1 <= rank <= MAX_RANK:
        raise ValueError(f"rank {rank} outside 1..{MAX_RANK}")
    v = View()
    v.ptr = ptr
    v.dtype = dtype
    v.rank = rank
    for i in range(rank):
        v.extent[i] = int(shape[rank - 1 - i])
        v.stride[i] = int(strides_bytes[rank - 1 - i])
    return v


def numpy_view(arr) -> View:
    """View of a host numpy array (the oracle's memory)."""
    code = _NUMPY_DTYPES.get(str(arr.dtype))
    if code is None:
        raise TypeError(f"unsupported numpy dtype {arr.dtype}")
    return make_view(arr.ctypes.data, code, arr.shape, arr.strides)


def rgb8_view(ptr: int, shape, strides_bytes) -> View:
    """View of packed (r, g, b) pixels held as a uint8 array of shape (..., 3) whose last
    axis is contiguous; ``shape``/``strides_bytes`` are the array's, channel axis included."""
    if len(shape) < 2 or shape[-1] != 3 or strides_bytes[-1] != 1:
        raise ValueError("an rgb8 image is a uint8 array of shape (..., 3) with contiguous channels")
    return make_view(ptr, RGB8, tuple(shape[:-1]), tuple(strides_bytes[:-1]))


def torch_view(t) -> View:
    """View of a torch tensor (device memory for the CUDA library)."""
    code = _TORCH_DTYPES.get(str(t.dtype))
    if code is None:
        raise TypeError(f"unsupported torch dtype {t.dtype}")
    size = t.element_size()
    return make_view(t.data_ptr(), code, tuple(t.shape), tuple(s * size for s in t.stride()))
