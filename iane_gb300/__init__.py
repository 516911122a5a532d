"""GB300-native IANE convolution and Richardson-Lucy deconvolution.

Python mirror of the reference interface for this path, over torch CUDA tensors (torch
supplies device memory and streams only; every computation runs in ``libiane_gb300.so``):

* :func:`convolve` -- ``iane::convolve(src, kernel, dst, {border}, cuda_policy{stream})``
  (reference include/iane/algorithms/convolution.hpp:97-117): odd kernel extents, the
  kernel flipped, same extents in and out, reference casts for integer outputs.
* :func:`convolve_separable` -- the same with an outer-product kernel, one fused pass.
* :func:`convolve_rgb8` -- packed (r, g, b) byte pixels, each channel summed on its own: the
  custom element of the reference's convolution example (examples/convolution/main.cu:20-56).
* :class:`Wiener` -- prepared Wiener deconvolution (examples/wiener/main.cu:44-83).
* :func:`morphology` -- flat erosion, dilation, opening and closing
  (include/iane/algorithms/morphology/morphology.hpp).
* :class:`Texture` / :class:`TextureView` -- the reference's texture_image and
  texture_image_view (include/iane/resource/cuda/texture_image.hpp,
  include/iane/view/texture_image_view.hpp); a :class:`TextureView` is a valid ``src`` of
  :func:`convolve`.
* :class:`RichardsonLucy` -- the prepared-algorithm protocol of
  include/iane/execution/prepared.hpp:120-146 (``prepare`` sizes the scratch, ``run``
  consumes it) applied to the RL loop of examples/rl_deconvolution/main.cu:51-81.

Tensors are C-ordered (slowest axis first): a tensor of shape ``(nz, ny, nx)`` is the IANE
view with extents ``[nx, ny, nz]``. Kernels are indexed the same way.
"""
from __future__ import annotations

import ctypes

from . import abi
from ._lib import IaneError, IaneInvalidArgument, IaneLengthError, check, lib

__all__ = [
    "abi", "convolve", "convolve_separable", "convolve_rgb8", "morphology", "Texture", "TextureView", "Wiener",
    "RichardsonLucy",
    "RichardsonLucyBatch", "device_status", "IaneError", "IaneInvalidArgument", "IaneLengthError",
]


def _stream_handle(stream) -> int:
    import torch

    if stream is None:
        stream = torch.cuda.current_stream()
    return int(stream.cuda_stream)


def _border(border) -> int:
    if isinstance(border, str):
        if border not in abi.BORDERS:
            raise ValueError(f"unknown border {border!r}")
        return abi.BORDERS[border]
    return int(border)


def _device_view(t) -> abi.View:
    if not t.is_cuda:
        raise ValueError("iane_gb300 works on CUDA tensors; copy host data to the device first")
    return abi.torch_view(t)


def convolve(src, kernel, dst, border="clamp", exact: bool = False, method: str = "direct", stream=None):
    """Convolution of ``src`` with ``kernel`` into ``dst`` (all CUDA tensors).

    ``exact=True`` accumulates in FP64 in the reference's tap order, giving results
    bit-identical to the reference's CPU convolution; the default is FP32 accumulation
    (int64 for integer image/kernel pairs). ``method="fft"`` uses the spectral path (FP64
    cuFFT transforms of the border-padded source; float types), ``method="auto"`` picks
    direct or spectral by a cost model. Asynchronous on ``stream``."""
    if method not in ("direct", "fft", "auto"):
        raise ValueError(f"unknown method {method!r}")
    flags = abi.ACC_EXACT if exact else abi.ACC_FAST
    flags |= {"direct": 0, "fft": abi.CONV_FFT, "auto": abi.CONV_AUTO}[method]
    k, d = _device_view(kernel), _device_view(dst)
    if isinstance(src, TextureView):
        tv = src._abi()
        check(lib().iane_gb_convolve_texture(ctypes.byref(tv), ctypes.byref(k), ctypes.byref(d), _border(border),
                                             flags, _stream_handle(stream)))
        return dst
    s = _device_view(src)
    check(lib().iane_gb_convolve(ctypes.byref(s), ctypes.byref(k), ctypes.byref(d), _border(border), flags,
                                 _stream_handle(stream)))
    return dst


def _rgb8_device_view(t) -> abi.View:
    if not t.is_cuda or str(t.dtype) != "torch.uint8":
        raise ValueError("an rgb8 image is a CUDA uint8 tensor of shape (..., 3)")
    return abi.rgb8_view(t.data_ptr(), tuple(t.shape), tuple(t.stride()))


def convolve_rgb8(src, kernel, dst, border="clamp", exact: bool = False, stream=None):
    """Convolution of packed rgb8 pixels: ``src`` and ``dst`` are uint8 CUDA tensors of shape
    ``(..., 3)`` (channels contiguous), ``kernel`` an f32 tensor of the image rank. Each
    channel is convolved on its own and converted with the byte rule; ``exact=True`` gives the
    reference's per-channel double sums bit for bit."""
    s, d, k = _rgb8_device_view(src), _rgb8_device_view(dst), _device_view(kernel)
    flags = abi.ACC_EXACT if exact else abi.ACC_FAST
    check(lib().iane_gb_convolve(ctypes.byref(s), ctypes.byref(k), ctypes.byref(d), _border(border), flags,
                                 _stream_handle(stream)))
    return dst


def morphology(src, dst, radius, op: str = "erode", border="clamp", footprint=None, scratch=None, stream=None):
    """Flat morphology (include/iane/algorithms/morphology/morphology.hpp): ``op`` is
    "erode", "dilate", "opening" or "closing"; ``radius`` is C-ordered like the tensors;
    ``footprint`` is None (the whole box) or a CUDA uint8/bool tensor of shape 2 * radius + 1
    whose nonzero cells are contained. Opening and closing run through ``scratch`` (allocated
    when None) and may run in place (``src is dst``); erode and dilate need disjoint views."""
    if op not in abi.MORPHOLOGY_OPS:
        raise ValueError(f"unknown morphology op {op!r}")
    s, d = _device_view(src), _device_view(dst)
    rank = len(src.shape)
    radius = tuple(int(r) for r in radius)
    if len(radius) != rank:
        raise ValueError("radius needs one entry per axis")
    r = (ctypes.c_int32 * 3)(*([radius[rank - 1 - i] for i in range(rank)] + [0] * (3 - rank)))
    mask = None
    if footprint is not None:
        if tuple(footprint.shape) != tuple(2 * v + 1 for v in radius) or not footprint.is_cuda:
            raise ValueError("footprint must be a CUDA tensor of shape 2 * radius + 1")
        mask = footprint.contiguous().to(dtype=__import__("torch").uint8)
    code = abi.MORPHOLOGY_OPS[op]
    mp = None if mask is None else mask.data_ptr()
    if code in (abi.ERODE, abi.DILATE):
        check(lib().iane_gb_morphology(ctypes.byref(s), ctypes.byref(d), r, mp, code, _border(border),
                                       _stream_handle(stream)))
        return dst
    ext = (ctypes.c_int32 * 3)(*[s.extent[i] for i in range(3)])
    need = int(lib().iane_gb_morphology_scratch_bytes(s.dtype, rank, ext))
    if scratch is None:
        import torch

        scratch = torch.empty(max(need, 1), dtype=torch.uint8, device=src.device)
    check(lib().iane_gb_morphology_compound(ctypes.byref(s), ctypes.byref(d), r, mp, code, _border(border),
                                            scratch.data_ptr(), scratch.numel(), _stream_handle(stream)))
    return dst


class Wiener:
    """Prepared Wiener deconvolution (the reference's examples/wiener/main.cu:44-83): the
    PSF (f32 CUDA tensor of the image rank, centred at the origin with periodic wrap-around)
    becomes the filter conj(H) / (|H|^2 + noise) once; ``run`` restores an observed image of
    ``shape`` into ``restored`` (uint8: the example's to_gray8; float32: the plain value)."""

    def __init__(self, psf, shape, noise: float = 0.002, stream=None):
        self.shape = tuple(int(n) for n in shape)
        rank = len(self.shape)
        k = _device_view(psf)
        ext = (ctypes.c_int32 * 3)(*([self.shape[rank - 1 - i] for i in range(rank)] + [1] * (3 - rank)))
        handle = ctypes.c_void_p()
        check(lib().iane_gb_wiener_prepare(ctypes.byref(k), rank, ext, float(noise), _stream_handle(stream),
                                           ctypes.byref(handle)))
        self._plan = handle
        self.scratch_bytes = int(lib().iane_gb_wiener_scratch_bytes(handle))

    def run(self, observed, restored, scratch=None, stream=None):
        import torch

        if scratch is None:
            scratch = torch.empty(self.scratch_bytes, dtype=torch.uint8, device=observed.device)
        s, d = _device_view(observed), _device_view(restored)
        check(lib().iane_gb_wiener_run(self._plan, ctypes.byref(s), ctypes.byref(d), scratch.data_ptr(),
                                       scratch.numel(), _stream_handle(stream)))
        return restored

    def close(self) -> None:
        if getattr(self, "_plan", None):
            lib().iane_gb_wiener_destroy(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Texture:
    """A CUDA array with its point-sampled texture object (the reference's texture_image).

    ``shape`` is C-ordered like tensors; ``dtype`` a torch or numpy dtype name of a texel type
    (u8, i8, u16, i16, i32, u32, f32). ``upload`` copies a host (numpy) or CUDA (torch) array of
    that shape and type; ``view()`` borrows the whole texture as a convolution source."""

    def __init__(self, shape, dtype):
        code = abi._TORCH_DTYPES.get(str(dtype), abi._NUMPY_DTYPES.get(str(dtype)))
        if code not in abi.TEXEL_DTYPES:
            raise TypeError(f"texture element type {dtype} is not one of u8, i8, u16, i16, i32, u32, f32")
        self.shape = tuple(int(n) for n in shape)
        self.dtype = code
        rank = len(self.shape)
        ext = (ctypes.c_int32 * 3)(*([self.shape[rank - 1 - i] for i in range(rank)] + [1] * (3 - rank)))
        handle = ctypes.c_uint64(0)
        check(lib().iane_gb_texture_create(code, rank, ext, ctypes.byref(handle)))
        self.handle = handle.value

    def upload(self, array, stream=None) -> "Texture":
        if hasattr(array, "is_cuda"):
            v = abi.torch_view(array)
        else:
            v = abi.numpy_view(array)
        check(lib().iane_gb_texture_upload(self.handle, ctypes.byref(v), _stream_handle(stream)))
        return self

    def view(self) -> "TextureView":
        return TextureView(self, (0,) * len(self.shape), self.shape)

    def close(self) -> None:
        if getattr(self, "handle", 0):
            check(lib().iane_gb_texture_destroy(self.handle))
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class TextureView:
    """A region of a :class:`Texture` (texture_image_view): ``origin`` and ``shape`` C-ordered."""

    def __init__(self, texture: Texture, origin, shape):
        if len(origin) != len(texture.shape) or len(shape) != len(texture.shape):
            raise ValueError("origin and shape need the texture's rank")
        self.texture = texture
        self.origin = tuple(int(o) for o in origin)
        self.shape = tuple(int(n) for n in shape)

    def subview(self, origin, shape) -> "TextureView":
        """An in-bounds region whose coordinates start at zero (texture_image_view::subview)."""
        if any(o < 0 or n < 0 or o + n > m for o, n, m in zip(origin, shape, self.shape)):
            raise ValueError("subview outside the view")
        return TextureView(self.texture, tuple(a + b for a, b in zip(self.origin, origin)), shape)

    def _abi(self) -> abi.TextureView:
        rank = len(self.shape)
        tv = abi.TextureView()
        tv.texture = self.texture.handle
        tv.dtype = self.texture.dtype
        tv.rank = rank
        for i in range(3):
            tv.extent[i] = self.shape[rank - 1 - i] if i < rank else 1
            tv.origin[i] = self.origin[rank - 1 - i] if i < rank else 0
        return tv


def convolve_separable(src, taps, dst, border="clamp", stream=None):
    """Convolution with the outer product of 1-D f32 ``taps`` (``taps[i]`` for IANE axis i,
    i.e. ``taps[0]`` runs along the last tensor dimension)."""
    s, d = _device_view(src), _device_view(dst)
    views = [_device_view(t) for t in taps]
    arr = (ctypes.POINTER(abi.View) * max(1, len(views)))(*[ctypes.pointer(v) for v in views])
    check(lib().iane_gb_convolve_separable(ctypes.byref(s), arr, ctypes.byref(d), _border(border),
                                           _stream_handle(stream)))
    return dst


def device_status(stream=None) -> None:
    """Raise if a bounded device-side wait of an earlier launch gave up."""
    check(lib().iane_gb_device_status(_stream_handle(stream)))


def fp32_peak(paired: bool = False, stream=None) -> float:
    """Measured FP32 FMA throughput of the current device in TFLOP/s: scalar FFMA, or the
    packed two-lane form (``paired``). Synchronises the stream."""
    out = ctypes.c_double(0.0)
    check(lib().iane_gb_fp32_peak_probe(1 if paired else 0, ctypes.byref(out), _stream_handle(stream)))
    return float(out.value)


class RichardsonLucy:
    """Prepared Richardson-Lucy deconvolution for one image shape and PSF.

    ``prepare`` copies the PSF, builds its adjoint and the exact edge-sensitivity table
    (the reference computes sensitivity = convolve(1, adjoint, zero border) per prepare,
    examples/rl_deconvolution/main.cu:62-64). ``scratch_bytes`` is what ``run`` needs, as
    in the reference's prepared protocol; ``run`` allocates it with torch when no scratch
    tensor is passed.
    """

    INIT_OBSERVED = abi.RL_INIT_OBSERVED
    INIT_MEAN = abi.RL_INIT_MEAN
    INIT_GIVEN = abi.RL_INIT_GIVEN

    def __init__(self, psf, shape, stream=None, precision: str = "f32", per_pass: bool = False):
        """``precision="bf16"`` selects the tensor-core path: BF16 images and PSF in the
        convolutions (tcgen05 implicit GEMM, FP32 accumulation), FP32 everything else.
        ``per_pass=True`` makes the FP32 path launch once per pass instead of once per run
        (same results)."""
        self.shape = tuple(int(s) for s in shape)
        self.precision = precision
        if precision not in ("f32", "bf16"):
            raise ValueError(f"unknown precision {precision!r}")
        rank = len(self.shape)
        ext = (ctypes.c_int32 * 3)(*([self.shape[rank - 1 - i] for i in range(rank)] + [1] * (3 - rank)))
        handle = ctypes.c_void_p()
        v = _device_view(psf)
        flags = abi.RL_BF16_TENSOR if precision == "bf16" else 0
        if per_pass:
            flags |= abi.RL_PER_PASS
        check(lib().iane_gb_rl_prepare_ex(ctypes.byref(v), rank, ext, flags, _stream_handle(stream),
                                          ctypes.byref(handle)))
        self._plan = handle
        self.scratch_bytes = int(lib().iane_gb_rl_scratch_bytes(handle))

    def host_scratch_bytes(self, observed_u8: bool = False) -> int:
        return int(lib().iane_gb_rl_host_scratch_bytes(self._plan, abi.U8 if observed_u8 else abi.F32))

    def run(self, observed, estimate, iterations: int, epsilon: float = 1e-6, init: int = abi.RL_INIT_OBSERVED,
            scratch=None, stats=None, stream=None):
        """Run ``iterations`` RL iterations; ``estimate`` receives the result (f32 or u8).

        ``stats``: optional CUDA float64 tensor with ``2 * iterations`` entries receiving
        per-iteration flux and relative L2 change."""
        import torch

        if self._plan is None:
            raise RuntimeError("plan destroyed")
        if scratch is None:
            scratch = torch.empty(self.scratch_bytes, dtype=torch.uint8, device=observed.device)
        o, e = _device_view(observed), _device_view(estimate)
        stats_ptr = None
        if stats is not None:
            if stats.dtype != torch.float64 or not stats.is_cuda or stats.numel() < 2 * iterations:
                raise ValueError("stats must be a CUDA float64 tensor with 2*iterations entries")
            stats_ptr = stats.data_ptr()
        check(lib().iane_gb_rl_run(self._plan, ctypes.byref(o), ctypes.byref(e), int(iterations),
                                   ctypes.c_float(epsilon), int(init), scratch.data_ptr(), scratch.numel(),
                                   stats_ptr, _stream_handle(stream)))
        return estimate

    def run_host(self, observed_host, estimate_host, iterations: int, epsilon: float = 1e-6,
                 init: int = abi.RL_INIT_OBSERVED, scratch=None, stream=None):
        """End-to-end run from host (ideally pinned) CPU tensors; blocks until done."""
        import torch

        u8 = observed_host.dtype == torch.uint8
        if scratch is None:
            scratch = torch.empty(self.host_scratch_bytes(u8), dtype=torch.uint8, device="cuda")
        assert estimate_host.dtype == torch.float32 and estimate_host.is_contiguous()
        assert observed_host.is_contiguous() and not observed_host.is_cuda
        check(lib().iane_gb_rl_run_host(self._plan, observed_host.data_ptr(), abi.U8 if u8 else abi.F32,
                                        estimate_host.data_ptr(), int(iterations), ctypes.c_float(epsilon),
                                        int(init), scratch.data_ptr(), scratch.numel(), _stream_handle(stream)))
        return estimate_host

    def close(self) -> None:
        if self._plan is not None:
            lib().iane_gb_rl_destroy(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RichardsonLucyBatch:
    """Richardson-Lucy over many 2-D images of uneven size, each with its own PSF.

    The whole run -- every pass of every iteration of every image -- is one persistent launch
    over a device work queue of 64x64 tiles, each image's pass waiting only for that image's
    previous pass; the run (counter reset, start values, the launch) is captured into a CUDA
    graph and replayed while the tensors and parameters stay the same. ``autotune=True`` times
    the launch's CTAs per SM and queue order on this batch and caches the choice per batch
    signature (file named by ``IANE_GB_TUNE_CACHE``)."""

    def __init__(self, psfs, shapes, autotune: bool = False, stream=None):
        self.shapes = [tuple(int(v) for v in s) for s in shapes]
        if len(psfs) != len(self.shapes) or not psfs:
            raise ValueError("one PSF per image shape, at least one image")
        self._psf_views = (abi.View * len(psfs))(*[_device_view(p) for p in psfs])
        ext = (ctypes.c_int32 * (2 * len(psfs)))(*[v for (ny, nx) in self.shapes for v in (nx, ny)])
        handle = ctypes.c_void_p()
        flags = abi.BATCH_AUTOTUNE if autotune else 0
        check(lib().iane_gb_rl_batch_prepare(self._psf_views, len(psfs), ext, flags, _stream_handle(stream),
                                             ctypes.byref(handle)))
        self._batch = handle
        self.scratch_bytes = int(lib().iane_gb_rl_batch_scratch_bytes(handle))

    def tile_widths(self):
        out = (ctypes.c_int32 * len(self.shapes))()
        check(lib().iane_gb_rl_batch_tiles(self._batch, out))
        return list(out)

    def launch_config(self):
        """(CTAs per SM, queue order, grouping) of the persistent launch: order 0 = largest
        images first, 1 = grouped by PSF width; grouping 0-3 = the work items' shapes (tiles per
        item by PSF width, see ``tile_widths``)."""
        bps, order, group = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_int32(0)
        check(lib().iane_gb_rl_batch_config(self._batch, ctypes.byref(bps), ctypes.byref(order),
                                            ctypes.byref(group)))
        return int(bps.value), int(order.value), int(group.value)

    def configure(self, blocks_per_sm: int, order: int, grouping: int) -> None:
        """Pin the launch configuration (same results for any configuration)."""
        check(lib().iane_gb_rl_batch_configure(self._batch, int(blocks_per_sm), int(order), int(grouping)))

    def run(self, observed, estimates, iterations: int, epsilon: float = 1e-6, init: int = abi.RL_INIT_OBSERVED,
            scratch=None, stream=None):
        import torch

        if scratch is None:
            scratch = torch.empty(self.scratch_bytes, dtype=torch.uint8, device=observed[0].device)
        self._keep = (observed, estimates, scratch)
        o = (abi.View * len(observed))(*[_device_view(t) for t in observed])
        e = (abi.View * len(estimates))(*[_device_view(t) for t in estimates])
        check(lib().iane_gb_rl_batch_run(self._batch, o, e, int(iterations), ctypes.c_float(epsilon), int(init),
                                         scratch.data_ptr(), scratch.numel(), _stream_handle(stream)))
        return estimates

    def close(self) -> None:
        if getattr(self, "_batch", None) is not None:
            lib().iane_gb_rl_batch_destroy(self._batch)
            self._batch = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
