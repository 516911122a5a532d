"""The allocation-free Richardson-Lucy entry point (iane_gb_rl_run_noalloc).

It serves callers that cannot allocate device memory -- plugins whose host application owns
the device allocator or a memory budget, loops that must not block in the allocator -- by
keeping all scratch in one static device array. These tests call it through the C ABI, twice
in a row on different inputs (the second call reuses the array the first one left behind),
and compare each result with the CPU oracle (the reference's RL loop restated in C) and with
the plan-based entry point on the same inputs, within the tolerance the RL tests use; a third
case writes the u8 estimate through the reference's to_gray8. The file is collected last and
passes alone or after the rest.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import iane_gb300
import oracle
from iane_gb300 import _lib, abi
from gpu_helpers import empty_like_np, gaussian, rel_l2, to_gpu, to_host, torch

pytestmark = pytest.mark.gpu

TOL = 1e-5


def noalloc_run(psf, obs, iterations, init, out_dtype=np.float32):
    p, o = to_gpu(psf), to_gpu(obs)
    est = empty_like_np(obs.shape, out_dtype)
    pv, ov, ev = abi.torch_view(p), abi.torch_view(o), abi.torch_view(est)
    stream = torch().cuda.current_stream().cuda_stream
    status = _lib.lib().iane_gb_rl_run_noalloc(ctypes.byref(pv), ctypes.byref(ov), ctypes.byref(ev), iterations,
                                              ctypes.c_float(1e-6), init, stream)
    _lib.check(status)
    return to_host(est)


def plan_run(psf, obs, iterations, init, out_dtype=np.float32):
    rl = iane_gb300.RichardsonLucy(to_gpu(psf), obs.shape)
    est = empty_like_np(obs.shape, out_dtype)
    rl.run(to_gpu(obs), est, iterations, 1e-6, init=init)
    out = to_host(est)
    rl.close()
    return out


def check(got, ref):
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)
    assert float(np.max(np.abs(got.astype(np.float64) - ref))) <= TOL * float(np.max(np.abs(ref)))


def test_noalloc_matches_oracle_twice_in_a_row(cuda):
    rng = np.random.default_rng(2026)
    first_obs = rng.poisson(rng.random((24, 80, 96)) * 300 + 10).astype(np.float32)
    first_psf = gaussian((7, 15, 15), (1.0, 2.0, 2.0))
    second_obs = rng.poisson(rng.random((130, 170)) * 200 + 5).astype(np.float32)
    second_psf = gaussian((9, 5), (2.5, 1.0))
    for obs, psf, init in ((first_obs, first_psf, abi.RL_INIT_MEAN), (second_obs, second_psf, abi.RL_INIT_OBSERVED)):
        got = noalloc_run(psf, obs, 6, init)
        check(got, oracle.rl(obs, psf, 6, 1e-6, init=init))
        check(got, plan_run(psf, obs, 6, init))
    iane_gb300.device_status()


def test_noalloc_u8_estimate_like_the_reference_example(cuda):
    # the reference example's byte path: u8 observed, start max(obs, eps), u8 result through
    # to_gray8; bytes agree except where the float estimate sits within FP32 rounding of .5
    rng = np.random.default_rng(2027)
    obs = rng.integers(0, 256, (50, 70)).astype(np.uint8)
    psf = gaussian((5, 7), (1.0, 1.5))
    ref_f = oracle.rl(obs, psf, 10, 1e-6, init=abi.RL_INIT_OBSERVED)
    ref_u8 = oracle.to_gray8(ref_f)
    for _ in range(2):
        got = noalloc_run(psf, obs, 10, abi.RL_INIT_OBSERVED, out_dtype=np.uint8)
        diff = got.astype(np.int32) - ref_u8.astype(np.int32)
        near_half = np.abs(ref_f - np.floor(ref_f) - 0.5) < 1e-3
        assert np.all((diff == 0) | near_half)
        assert np.all(np.abs(diff) <= 1)
    iane_gb300.device_status()


def test_noalloc_rejects_images_beyond_its_static_scratch(cuda):
    psf = gaussian((3, 3), (1.0, 1.0))
    big = np.ones((2049, 2048), np.float32)  # 4196352 voxels > 4194304
    with pytest.raises(iane_gb300.IaneLengthError):
        noalloc_run(psf, big, 1, abi.RL_INIT_OBSERVED)
