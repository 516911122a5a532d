"""CPU oracle for the convolution and Richardson-Lucy path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use this module,
always as the checker or the timed CPU baseline, never as the product. It loads

* ``liboracle.so``: the C restatement of the reference algorithm (``iane_oracle.c``), and
* ``_ref/libiane_ref.so`` (where it was built): the reference's own ``iane::convolve`` and a
  restated ``prepare_rl`` built from the reference's views and algorithms.

``wiener`` is a numpy restatement: the reference's Wiener example runs on FFTW (CPU) or
cuFFT, and FFTW is not installed here, so the oracle uses float64 DFTs (numpy's FFT),
pinned by tests to the direct DFT definition the reference's own FFT tests check
(test/unit/prepared/real_fft_cases.hpp:47-75) and to closed-form answers.

Arrays are C-ordered numpy arrays (slowest axis first); see ``iane_gb300.abi`` for the
mapping to IANE's axis-0-fastest views.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

from iane_gb300 import abi

HERE = Path(__file__).resolve().parent
_VIEW_P = ctypes.POINTER(abi.View)


def default_threads() -> int:
    return max(1, len(os.sched_getaffinity(0)))


def _load(path: Path):
    if not path.exists():
        raise FileNotFoundError(f"{path} is not built; run `python oracle/build.py`")
    return ctypes.CDLL(str(path))


_oracle = None
_ref = None


def oracle_lib():
    global _oracle
    if _oracle is None:
        lib = _load(HERE / "liboracle.so")
        lib.oracle_convolve.argtypes = [_VIEW_P, _VIEW_P, _VIEW_P, ctypes.c_int, ctypes.c_int]
        lib.oracle_convolve.restype = ctypes.c_int
        lib.oracle_convolve_separable.argtypes = [_VIEW_P, ctypes.POINTER(_VIEW_P), _VIEW_P,
                                                  ctypes.c_int, ctypes.c_int]
        lib.oracle_convolve_separable.restype = ctypes.c_int
        lib.oracle_rl.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int32),
                                  ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_int, ctypes.c_float,
                                  ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        lib.oracle_rl.restype = ctypes.c_int
        lib.oracle_to_gray8.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
        lib.oracle_to_gray8.restype = None
        lib.oracle_morphology.argtypes = [_VIEW_P, _VIEW_P, ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p,
                                          ctypes.c_int, ctypes.c_int]
        lib.oracle_morphology.restype = ctypes.c_int
        lib.oracle_sensitivity.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p, ctypes.c_int]
        lib.oracle_sensitivity.restype = ctypes.c_int
        lib.oracle_det_rl_volume.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                             ctypes.c_double, ctypes.c_uint64, ctypes.c_void_p,
                                             ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_int]
        lib.oracle_det_rl_volume.restype = ctypes.c_int
        _oracle = lib
    return _oracle


def reference_available() -> bool:
    return (HERE / "_ref" / "libiane_ref.so").exists()


def ref_lib():
    global _ref
    if _ref is None:
        lib = _load(HERE / "_ref" / "libiane_ref.so")
        lib.ref_convolve.argtypes = [_VIEW_P, _VIEW_P, _VIEW_P, ctypes.c_int, ctypes.c_int]
        lib.ref_convolve.restype = ctypes.c_int
        lib.ref_morphology.argtypes = [_VIEW_P, _VIEW_P, ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p,
                                       ctypes.c_int, ctypes.c_int]
        lib.ref_morphology.restype = ctypes.c_int
        lib.ref_rl.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p,
                               ctypes.POINTER(ctypes.c_int32), ctypes.c_int, ctypes.c_float, ctypes.c_int,
                               ctypes.c_void_p, ctypes.c_int]
        lib.ref_rl.restype = ctypes.c_int
        _ref = lib
    return _ref


def _extent(shape) -> ctypes.Array:
    rank = len(shape)
    return (ctypes.c_int32 * 3)(*([int(shape[rank - 1 - i]) for i in range(rank)] + [1] * (3 - rank)))


def _check(status: int, what: str) -> None:
    if status != 0:
        raise ValueError(f"{what} failed with status {status} ({abi.STATUS_NAMES.get(status, '?')})")


def convolve(src: np.ndarray, kernel: np.ndarray, out: np.ndarray, border: str = "clamp",
             threads: int | None = None, use_reference: bool = False) -> np.ndarray:
    """dst = iane::convolve(src, kernel) with the given border, on the host."""
    threads = default_threads() if threads is None else threads
    s, k, d = abi.numpy_view(src), abi.numpy_view(kernel), abi.numpy_view(out)
    if use_reference:
        status = ref_lib().ref_convolve(ctypes.byref(s), ctypes.byref(k), ctypes.byref(d),
                                        abi.BORDERS[border], threads)
    else:
        status = oracle_lib().oracle_convolve(ctypes.byref(s), ctypes.byref(k), ctypes.byref(d),
                                              abi.BORDERS[border], threads)
    _check(status, "convolve")
    return out


def convolve_rgb8(src: np.ndarray, kernel: np.ndarray, out: np.ndarray, border: str = "clamp",
                  threads: int | None = None, use_reference: bool = False) -> np.ndarray:
    """convolve() for packed (r, g, b) pixels: uint8 arrays of shape (..., 3), f32 kernel of
    the image rank (the custom element of examples/convolution/main.cu:20-56)."""
    threads = default_threads() if threads is None else threads
    s = abi.rgb8_view(src.ctypes.data, src.shape, src.strides)
    d = abi.rgb8_view(out.ctypes.data, out.shape, out.strides)
    k = abi.numpy_view(kernel)
    if use_reference:
        status = ref_lib().ref_convolve(ctypes.byref(s), ctypes.byref(k), ctypes.byref(d), abi.BORDERS[border], threads)
    else:
        status = oracle_lib().oracle_convolve(ctypes.byref(s), ctypes.byref(k), ctypes.byref(d), abi.BORDERS[border],
                                              threads)
    _check(status, "convolve rgb8")
    return out


def convolve_separable(src: np.ndarray, taps, out: np.ndarray, border: str = "clamp",
                       threads: int | None = None) -> np.ndarray:
    """Successive 1-D convolutions along axis 0 (fastest), 1, 2 with f32 intermediates.

    ``taps[i]`` is the 1-D f32 tap array for IANE axis i (axis 0 = last numpy axis)."""
    threads = default_threads() if threads is None else threads
    keep = [np.ascontiguousarray(t, dtype=np.float32) for t in taps]
    views = [abi.numpy_view(t) for t in keep]
    arr = (_VIEW_P * len(views))(*[ctypes.pointer(v) for v in views])
    s, d = abi.numpy_view(src), abi.numpy_view(out)
    _check(oracle_lib().oracle_convolve_separable(ctypes.byref(s), arr, ctypes.byref(d),
                                                  abi.BORDERS[border], threads), "separable convolve")
    return out


def rl(observed: np.ndarray, psf: np.ndarray, iterations: int, epsilon: float = 1e-6,
       init: int = abi.RL_INIT_OBSERVED, estimate: np.ndarray | None = None, threads: int | None = None,
       use_reference: bool = False, with_stats: bool = False):
    """Richardson-Lucy on the host (examples/rl_deconvolution/main.cu:51-81 of the reference).

    Returns the f32 estimate (and per-iteration [flux, rel_change] when ``with_stats``)."""
    threads = default_threads() if threads is None else threads
    observed = np.ascontiguousarray(observed)
    psf = np.ascontiguousarray(psf, dtype=np.float32)
    if estimate is None:
        estimate = np.zeros(observed.shape, dtype=np.float32)
    assert estimate.dtype == np.float32 and estimate.flags.c_contiguous
    rank = observed.ndim
    ext, kext = _extent(observed.shape), _extent(psf.shape)
    stats = np.zeros((max(iterations, 1), 2), dtype=np.float64)
    if use_reference:
        assert observed.dtype == np.float32 and not with_stats
        status = ref_lib().ref_rl(observed.ctypes.data, rank, ext, psf.ctypes.data, kext, iterations,
                                  ctypes.c_float(epsilon), init, estimate.ctypes.data, threads)
    else:
        code = abi.U8 if observed.dtype == np.uint8 else abi.F32
        assert observed.dtype in (np.uint8, np.float32)
        status = oracle_lib().oracle_rl(observed.ctypes.data, code, rank, ext, psf.ctypes.data, kext,
                                        iterations, ctypes.c_float(epsilon), init, estimate.ctypes.data,
                                        stats.ctypes.data if with_stats else None, threads)
    _check(status, "rl")
    return (estimate, stats[:iterations]) if with_stats else estimate


def sensitivity(psf_adjoint: np.ndarray, shape, threads: int | None = None) -> np.ndarray:
    """convolve(1, kernel, zero border): the RL edge-correction image."""
    threads = default_threads() if threads is None else threads
    k = np.ascontiguousarray(psf_adjoint, dtype=np.float32)
    out = np.zeros(shape, dtype=np.float32)
    _check(oracle_lib().oracle_sensitivity(k.ctypes.data, _extent(k.shape), k.ndim, _extent(shape),
                                           out.ctypes.data, threads), "sensitivity")
    return out


def det_rl_volume(extent_xyz, count: int, psf: np.ndarray, seed: int, radius=(2.0, 20.0),
                  intensity=(50.0, 1000.0), background: float = 10.0, threads: int | None = None):
    """Deterministic ellipsoid phantom, its zero-border blur by ``psf`` and Poisson counts
    (``det_synth.c``): the same bits on every platform. Returns (observed, truth), float32
    C-ordered arrays of shape (nz, ny, nx)."""
    threads = default_threads() if threads is None else threads
    nx, ny, nz = (int(v) for v in extent_xyz)
    k = np.ascontiguousarray(psf, dtype=np.float32)
    assert k.ndim == 3
    truth = np.zeros((nz, ny, nx), np.float32)
    observed = np.zeros((nz, ny, nx), np.float32)
    status = oracle_lib().oracle_det_rl_volume(nx, ny, nz, count, radius[0], radius[1], intensity[0], intensity[1],
                                               background, seed, k.ctypes.data, _extent(k.shape),
                                               truth.ctypes.data, observed.ctypes.data, threads)
    _check(status, "det_rl_volume")
    return observed, truth


def to_gray8(values: np.ndarray) -> np.ndarray:
    v = np.ascontiguousarray(values, dtype=np.float32)
    out = np.zeros(v.shape, dtype=np.uint8)
    oracle_lib().oracle_to_gray8(v.ctypes.data, out.ctypes.data, v.size)
    return out


def mirror_pad(src: np.ndarray, radii) -> np.ndarray:
    """Half-sample symmetric padding by ``radii`` (C order: slowest axis first), period 2n."""
    out = src
    for axis, r in enumerate(radii):
        n = src.shape[axis]
        idx = np.arange(-r, n + r)
        m = np.mod(idx, 2 * n)
        idx = np.where(m < n, m, 2 * n - 1 - m)
        out = np.take(out, idx, axis=axis)
    return np.ascontiguousarray(out)


def wiener_pad_psf(psf: np.ndarray, shape) -> np.ndarray:
    """The PSF in an image-sized buffer with its centre (extent // 2 per axis) at the origin,
    wrapped periodically (examples/wiener/main.cu:112-120)."""
    pad = np.zeros(shape, np.float64)
    pad[tuple(slice(0, e) for e in psf.shape)] = psf
    return np.roll(pad, [-(e // 2) for e in psf.shape], axis=tuple(range(psf.ndim)))


def to_gray8(values: np.ndarray) -> np.ndarray:
    """examples/common/deconvolution.hpp:43-55 on float32 values: round half up, saturate."""
    v = values.astype(np.float32)
    out = np.zeros(v.shape, np.uint8)
    inside = (v > 0) & (v < 255)
    whole = np.floor(v[inside])
    out[inside] = (whole + ((v[inside] - whole) >= np.float32(0.5))).astype(np.uint8)
    out[v >= 255] = 255
    return out


def wiener(observed: np.ndarray, psf: np.ndarray, noise: float, out_dtype=np.uint8) -> np.ndarray:
    """Wiener deconvolution (examples/wiener/main.cu:44-83): IFFT(FFT(observed) * conj(H) /
    (|H|^2 + noise)) / N with H the spectrum of the wrapped PSF; u8 output through to_gray8,
    float32 output as the value."""
    h = np.fft.fftn(wiener_pad_psf(psf.astype(np.float64), observed.shape))
    o = np.fft.fftn(observed.astype(np.float64))
    r = np.fft.ifftn(o * np.conj(h) / (h.real ** 2 + h.imag ** 2 + float(np.float32(noise)))).real
    if np.dtype(out_dtype) == np.uint8:
        return to_gray8(r)
    return r.astype(out_dtype)


MORPHOLOGY_OPS = {"erode": 0, "dilate": 1, "opening": 2, "closing": 3}


def morphology(src: np.ndarray, out: np.ndarray, radius, op: str = "erode", border: str = "clamp",
               footprint: np.ndarray | None = None, use_reference: bool = False) -> np.ndarray:
    """Flat erosion / dilation, or opening / closing as the two passes through a packed
    intermediate (morphology.hpp:118-125). ``radius`` is C-ordered like the arrays;
    ``footprint`` (optional) is a boolean array of shape 2 * radius + 1 (C order)."""
    if op in ("opening", "closing"):
        first, second = ("erode", "dilate") if op == "opening" else ("dilate", "erode")
        mid = np.zeros(src.shape, src.dtype)
        morphology(src, mid, radius, first, border, footprint, use_reference)
        return morphology(mid, out, radius, second, border, footprint, use_reference)
    rank = src.ndim
    r = (ctypes.c_int32 * 3)(*([int(radius[rank - 1 - i]) for i in range(rank)] + [0] * (3 - rank)))
    mask = None
    if footprint is not None:
        mask = np.ascontiguousarray(footprint, dtype=np.uint8)
    s, d = abi.numpy_view(src), abi.numpy_view(out)
    fn = ref_lib().ref_morphology if use_reference else oracle_lib().oracle_morphology
    status = fn(ctypes.byref(s), ctypes.byref(d), r, None if mask is None else mask.ctypes.data,
                MORPHOLOGY_OPS[op], abi.BORDERS[border])
    _check(status, "morphology")
    return out

