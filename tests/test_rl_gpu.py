"""GPU Richardson-Lucy parity against the oracle (the reference's RL loop restated in C)
and the golden vectors made by the reference.

Tolerance: RL compounds the FP32 rounding of two convolutions per iteration, so the bar
is on the final estimate as a whole: relative L2 error <= 1e-5 and max |diff| <= 1e-5 *
max |ref| against the reference's FP64-accumulated result."""
from __future__ import annotations

import numpy as np
import pytest

import iane_gb300
import oracle
from golden_cases import rl_cases
from gpu_helpers import empty_like_np, gaussian, rel_l2, to_gpu, to_host, torch

pytestmark = pytest.mark.gpu

TOL = 1e-5


def gpu_rl(obs, psf, iterations, init, eps=1e-6, out_dtype=np.float32, stats=False):
    rl = iane_gb300.RichardsonLucy(to_gpu(psf), obs.shape)
    est = empty_like_np(obs.shape, out_dtype)
    st = torch().zeros(2 * max(iterations, 1), dtype=torch().float64, device="cuda") if stats else None
    rl.run(to_gpu(obs), est, iterations, eps, init=init, stats=st)
    out = to_host(est)
    rl.close()
    return (out, to_host(st)[: 2 * iterations].reshape(-1, 2)) if stats else out


def check(est, ref):
    assert rel_l2(est, ref) <= TOL, rel_l2(est, ref)
    assert float(np.max(np.abs(est.astype(np.float64) - ref))) <= TOL * float(np.max(np.abs(ref)))


@pytest.mark.parametrize("case", rl_cases(), ids=lambda c: c[0])
def test_golden_rl(cuda, case):
    name, obs, psf, expected, init, iters = case
    check(gpu_rl(obs, psf, iters, init), expected)


def phantom(shape, rng, count=30, background=10.0):
    grids = np.meshgrid(*[np.arange(n, dtype=np.float32) for n in shape], indexing="ij")
    vol = np.full(shape, background, np.float32)
    for _ in range(count):
        c = [rng.uniform(0, n) for n in shape]
        r = [rng.uniform(1.5, max(2.0, n / 4)) for n in shape]
        inside = sum(((g - ci) / ri) ** 2 for g, ci, ri in zip(grids, c, r)) <= 1.0
        vol[inside] += rng.uniform(50, 1000)
    return vol


CASES = [
    ((61,), (9,), 0), ((40, 53), (7, 5), 1), ((33, 47), (31, 3), 0), ((5, 6), (9, 11), 1),
    ((12, 40, 44), (5, 7, 9), 1), ((16, 64, 72), (7, 15, 15), 1), ((9, 17, 23), (3, 5, 29), 0),
    ((3, 4, 5), (5, 9, 7), 1),
    # a 29791-tap PSF: planes stream through shared memory, kz unbounded
    ((12, 40, 36), (31, 31, 31), 1),
]


@pytest.mark.parametrize("shape,pshape,init", CASES, ids=[f"{s}-{p}-{i}" for s, p, i in CASES])
def test_random_rl_matches_oracle(cuda, shape, pshape, init):
    rng = np.random.default_rng(sum(shape) * 31 + sum(pshape))
    truth = phantom(shape, rng)
    psf = gaussian(pshape, [max(0.6, n / 5) for n in pshape])
    blurred = np.zeros_like(truth)
    oracle.convolve(truth, psf, blurred, "zero")
    obs = rng.poisson(np.maximum(blurred, 0)).astype(np.float32)
    iters = 6
    ref, ref_stats = oracle.rl(obs, psf, iters, 1e-6, init=init, with_stats=True)
    est, stats = gpu_rl(obs, psf, iters, init, stats=True)
    check(est, ref)
    assert np.allclose(stats[:, 0], ref_stats[:, 0], rtol=1e-5)
    assert np.allclose(stats[:, 1], ref_stats[:, 1], rtol=1e-3, atol=1e-7)


def test_u8_observed_and_output_like_the_reference_example(cuda):
    # examples/rl_deconvolution: uint8 input, start max(obs, eps), uint8 output via to_gray8
    rng = np.random.default_rng(12)
    obs = rng.integers(0, 256, (48, 64)).astype(np.uint8)
    psf = gaussian((5, 5), (1.0, 1.0))
    ref_f = oracle.rl(obs, psf, 10, 1e-6, init=0)
    ref_u8 = oracle.to_gray8(ref_f)
    out = gpu_rl(obs, psf, 10, 0, out_dtype=np.uint8)
    diff = out.astype(np.int32) != ref_u8.astype(np.int32)
    # bytes agree except where the float estimate sits within FP32 rounding of a .5 boundary
    near_half = np.abs(ref_f - np.floor(ref_f) - 0.5) < 1e-3
    assert np.all(~diff | near_half)
    assert np.all(np.abs(out.astype(np.int32) - ref_u8.astype(np.int32)) <= 1)


def test_given_start_strided_estimate_and_zero_iterations(cuda):
    t = torch()
    rng = np.random.default_rng(13)
    obs = (rng.random((6, 30, 31)) * 100 + 1).astype(np.float32)
    psf = gaussian((3, 5, 5), (1.0, 1.0, 1.0))
    start = (rng.random(obs.shape) * 50 + 1).astype(np.float32)
    ref = oracle.rl(obs, psf, 4, 1e-6, init=2, estimate=start.copy())
    rl = iane_gb300.RichardsonLucy(to_gpu(psf), obs.shape)
    big = t.zeros((8, 32, 70), device="cuda")
    view = big[1:7, 1:31, 2:64:2]
    view.copy_(to_gpu(start))
    rl.run(to_gpu(obs), view, 4, 1e-6, init=rl.INIT_GIVEN)
    check(to_host(view), ref)
    # zero iterations returns the start
    e2 = empty_like_np(obs.shape, np.float32)
    rl.run(to_gpu(obs), e2, 0, 1e-6, init=rl.INIT_OBSERVED)
    assert np.array_equal(to_host(e2), np.maximum(obs, np.float32(1e-6)))
    rl.close()


def test_run_host_equals_device_run(cuda):
    t = torch()
    rng = np.random.default_rng(14)
    obs = (rng.random((8, 40, 36)) * 100 + 1).astype(np.float32)
    psf = gaussian((3, 7, 5), (1.0, 1.5, 1.2))
    rl = iane_gb300.RichardsonLucy(to_gpu(psf), obs.shape)
    est_dev = empty_like_np(obs.shape, np.float32)
    rl.run(to_gpu(obs), est_dev, 5, 1e-6, init=rl.INIT_MEAN)
    host_obs = t.from_numpy(obs).pin_memory()
    host_est = t.zeros(obs.shape, dtype=t.float32).pin_memory()
    rl.run_host(host_obs, host_est, 5, 1e-6, init=rl.INIT_MEAN)
    assert np.array_equal(host_est.numpy(), to_host(est_dev))
    rl.close()


def test_scratch_too_small_is_length_error(cuda):
    t = torch()
    psf = gaussian((3, 3), (1.0, 1.0))
    rl = iane_gb300.RichardsonLucy(to_gpu(psf), (16, 16))
    small = t.zeros(16, dtype=t.uint8, device="cuda")
    with pytest.raises(iane_gb300.IaneLengthError):
        rl.run(to_gpu(np.ones((16, 16), np.float32)), empty_like_np((16, 16), np.float32), 2, scratch=small)
    rl.close()


def test_full_size_flux_invariant(cuda):
    # The 3-D RL configuration at full size (256x256x64, PSF 15x15x7 sigma (2,2,1), flat
    # start): after every iteration sum(sensitivity * estimate) equals sum(observed)
    # (each ratio voxel redistributes exactly its observed count), a size-independent check
    # of both fused passes and of the exact edge-sensitivity table.
    rng = np.random.default_rng(15)
    shape = (64, 256, 256)
    obs = rng.poisson(phantom(shape, rng, count=200)).astype(np.float32)
    psf = gaussian((7, 15, 15), (1.0, 2.0, 2.0))
    adj = np.ascontiguousarray(psf[::-1, ::-1, ::-1])
    ones = to_gpu(np.ones(shape, np.float32))
    sens = empty_like_np(shape, np.float32)
    iane_gb300.convolve(ones, to_gpu(adj), sens, "zero", exact=True)
    rl = iane_gb300.RichardsonLucy(to_gpu(psf), shape)
    est = empty_like_np(shape, np.float32)
    g_obs = to_gpu(obs)
    total = float(obs.astype(np.float64).sum())
    for iters in (1, 3):
        rl.run(g_obs, est, iters, 1e-6, init=rl.INIT_MEAN)
        weighted = float((sens.double() * est.double()).sum())
        assert abs(weighted - total) <= 1e-5 * total, (iters, weighted, total)
    iane_gb300.device_status()
    rl.close()
