"""The reference's own CUDA convolution kernel on the GPU -- TEST INFRASTRUCTURE ONLY.

``oracle/_ref/ref_conv_f32_3d.cubin`` (built by ``oracle/build.py`` from the reference's headers
where they exist; a cubin is device code, so it also runs on a GPU host of another CPU
architecture) holds the reference's ``visit_positions`` kernel
(include/iane/algorithms/for_each.hpp:19-29) instantiated with the functor ``iane::convolve``
builds for f32 3-D CUDA views. This module loads it with the CUDA driver API and launches it as
the reference's ``visit_coordinates`` does (for_each.hpp:143-160): one thread per output voxel,
256-thread blocks. The functor argument is filled from the byte layout recorded next to the
cubin. Used by the tests (its results are the reference's bits) and by bench.py's reference arm
(the reference's own GPU path timed on the same GPU); never by the product.
"""
from __future__ import annotations

import ctypes
import json
import struct
from pathlib import Path

HERE = Path(__file__).resolve().parent
CUBIN = HERE / "_ref" / "ref_conv_f32_3d.cubin"
LAYOUT = HERE / "_ref" / "ref_conv_f32_3d.json"
BORDERS = {"clamp": 0, "zero": 1}  # the reference's border_mode (image_locator.hpp:14)


def available() -> bool:
    return CUBIN.exists() and LAYOUT.exists()


class ReferenceConvolution:
    """The reference kernel loaded into the current device's primary context (torch's)."""

    def __init__(self):
        import torch

        torch.zeros(1, device="cuda")  # make torch's primary context current on this thread
        self.layout = json.loads(LAYOUT.read_text())
        self.cu = cu = ctypes.CDLL("libcuda.so.1")
        vp = ctypes.c_void_p
        self._check(cu.cuInit(0), "cuInit")
        ctx = vp()
        self._check(cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        self.module = vp()
        self._check(cu.cuModuleLoad(ctypes.byref(self.module), str(CUBIN).encode()), "cuModuleLoad")
        count = ctypes.c_uint()
        self._check(cu.cuModuleGetFunctionCount(ctypes.byref(count), self.module), "cuModuleGetFunctionCount")
        funcs = (vp * count.value)()
        self._check(cu.cuModuleEnumerateFunctions(funcs, count, self.module), "cuModuleEnumerateFunctions")
        self.function = None
        for f in funcs:
            name = ctypes.c_char_p()
            self._check(cu.cuFuncGetName(ctypes.byref(name), vp(f)), "cuFuncGetName")
            if b"visit_positions" in name.value:
                self.function = vp(f)
                self.name = name.value.decode()
        if self.function is None:
            raise RuntimeError("the reference cubin holds no visit_positions kernel")
        # refuse to launch unless the kernel's parameters are exactly (functor, count, extents)
        # with the recorded sizes: a layout mismatch must not reach the GPU
        want = [self.layout["size"], 8, self.layout["extents_bytes"]]
        for i, size in enumerate(want):
            off, got = ctypes.c_size_t(), ctypes.c_size_t()
            self._check(cu.cuFuncGetParamInfo(self.function, ctypes.c_size_t(i), ctypes.byref(off), ctypes.byref(got)),
                        "cuFuncGetParamInfo")
            if got.value != size:
                raise RuntimeError(f"reference kernel parameter {i} has {got.value} bytes, expected {size}")
        off, got = ctypes.c_size_t(), ctypes.c_size_t()
        if cu.cuFuncGetParamInfo(self.function, ctypes.c_size_t(3), ctypes.byref(off), ctypes.byref(got)) == 0:
            raise RuntimeError("reference kernel takes more than three parameters")
        cu.cuLaunchKernel.argtypes = [vp, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                      ctypes.c_uint, ctypes.c_uint, vp, ctypes.POINTER(vp), ctypes.POINTER(vp)]

    @staticmethod
    def _check(status: int, what: str) -> None:
        if status != 0:
            raise RuntimeError(f"{what} failed with CUDA driver status {status}")

    @staticmethod
    def _view(t):
        """(pointer, extents x y z, byte strides x y z) of a C-ordered (nz, ny, nx) f32 tensor."""
        assert t.dtype.itemsize == 4 and t.dim() == 3 and t.is_cuda
        nz, ny, nx = t.shape
        sz, sy, sx = (4 * s for s in t.stride())
        for v in (sx, sy, sz):
            assert 0 <= v < 2 ** 31, "the reference's views hold int byte strides"
        return t.data_ptr(), (nx, ny, nz), (sx, sy, sz)

    def convolve(self, src, kernel, dst, border: str = "zero", stream=None):
        """dst = iane::convolve(src, kernel, dst, {border}) by the reference's own kernel: f32 3-D
        CUDA tensors, C-ordered (nz, ny, nx); asynchronous on `stream` (torch's current stream
        when None)."""
        import torch

        L = self.layout
        fn = bytearray(L["size"])
        for name, t in (("dst", dst), ("src", src), ("ker", kernel)):
            ptr, ext, strides = self._view(t)
            struct.pack_into("<Q", fn, L[f"{name}_ptr"], ptr)
            struct.pack_into("<3i", fn, L[f"{name}_size"], *ext)
            struct.pack_into("<3i", fn, L[f"{name}_strides"], *strides)
        struct.pack_into("<3i", fn, L["filter_size"], *self._view(kernel)[1])
        struct.pack_into("<i", fn, L["border"], BORDERS[border])
        nx, ny, nz = self._view(dst)[1]
        count = nx * ny * nz
        if count == 0:
            return dst
        fn_buf = (ctypes.c_char * len(fn)).from_buffer(fn)
        count_buf = ctypes.c_uint64(count)
        size_buf = (ctypes.c_int32 * 3)(nx, ny, nz)
        params = (ctypes.c_void_p * 3)(ctypes.addressof(fn_buf), ctypes.addressof(count_buf),
                                       ctypes.addressof(size_buf))
        s = stream if stream is not None else torch.cuda.current_stream()
        handle = s.cuda_stream if hasattr(s, "cuda_stream") else int(s)
        blocks = 1 + (count - 1) // 256
        self._check(self.cu.cuLaunchKernel(self.function, blocks, 1, 1, 256, 1, 1, 0, ctypes.c_void_p(handle), params,
                                           None), "cuLaunchKernel")
        return dst

    def close(self) -> None:
        if getattr(self, "module", None) is not None and self.module.value:
            self.cu.cuModuleUnload(self.module)
            self.module = None
