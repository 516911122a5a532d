"""Helpers for the GPU parity tests: host<->device copies that keep numpy layouts."""
from __future__ import annotations

import numpy as np

import oracle

_TORCH = None


def torch():
    global _TORCH
    if _TORCH is None:
        import torch as t

        _TORCH = t
    return _TORCH


def to_gpu(arr: np.ndarray):
    t = torch()
    a = np.ascontiguousarray(arr)
    if a.dtype == np.uint16:
        return t.from_numpy(a.view(np.int16)).cuda().view(t.uint16)
    if a.dtype == np.uint32:
        return t.from_numpy(a.view(np.int32)).cuda().view(t.uint32)
    return t.from_numpy(a).cuda()


def to_host(tensor) -> np.ndarray:
    t = torch()
    torch().cuda.synchronize()
    if tensor.dtype == t.uint16:
        return tensor.contiguous().view(t.int16).cpu().numpy().view(np.uint16)
    if tensor.dtype == t.uint32:
        return tensor.contiguous().view(t.int32).cpu().numpy().view(np.uint32)
    return tensor.contiguous().cpu().numpy()


def empty_like_np(shape, dtype):
    t = torch()
    table = {np.float32: t.float32, np.float64: t.float64, np.uint8: t.uint8, np.int32: t.int32,
             np.int16: t.int16, np.uint16: t.uint16, np.int8: t.int8, np.uint32: t.uint32}
    return t.zeros(shape, dtype=table[np.dtype(dtype).type], device="cuda")


def magnitude(src: np.ndarray, kernel: np.ndarray, border: str) -> np.ndarray:
    """conv(|src|, |kernel|): the scale of each output's rounding error."""
    out = np.zeros(src.shape, np.float64)
    oracle.convolve(np.abs(src.astype(np.float64)), np.abs(kernel.astype(np.float64)), out, border)
    return out


def gaussian(shape, sigma):
    grids = np.meshgrid(*[np.arange(n) - n // 2 for n in shape], indexing="ij")
    g = np.exp(-sum((x / s) ** 2 for x, s in zip(grids, sigma)) / 2.0)
    return (g / g.sum()).astype(np.float32)


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    a64, b64 = a.astype(np.float64), b.astype(np.float64)
    return float(np.linalg.norm(a64 - b64) / max(np.linalg.norm(b64), 1e-300))
