"""The FP32 Richardson-Lucy run as one persistent launch (the default for images of at least
two waves of 64x64 tiles) against one launch per pass: the same tile body and epilogues in a
different schedule, so the results must be the same bits. Plus the persistent run against the
oracle (the reference's RL loop restated in C) at the FP32 bar: rel-L2 <= 1e-5 and max |diff|
<= 1e-5 * max |ref|."""
from __future__ import annotations

import numpy as np
import pytest

import iane_gb300
import oracle
from gpu_helpers import empty_like_np, gaussian, rel_l2, to_gpu, to_host, torch
from test_rl_gpu import phantom

pytestmark = pytest.mark.gpu

TOL = 1e-5


def run(obs, psf, iterations, init, per_pass, out=None, start=None):
    rl = iane_gb300.RichardsonLucy(to_gpu(psf), obs.shape, per_pass=per_pass)
    est = empty_like_np(obs.shape, np.float32) if out is None else out
    if start is not None:
        est.copy_(to_gpu(start))
    rl.run(to_gpu(obs), est, iterations, 1e-6, init=init)
    iane_gb300.device_status()
    host = to_host(est)
    rl.close()
    return host


def observed(shape, psf, seed):
    rng = np.random.default_rng(seed)
    truth = phantom(shape, rng, count=40)
    blurred = empty_like_np(shape, np.float32)
    iane_gb300.convolve(to_gpu(truth), to_gpu(psf), blurred, "zero")
    return rng.poisson(np.maximum(to_host(blurred), 0)).astype(np.float32)


# (z, y, x) shapes with at least 2 x 152 tiles of 64 x 64 (the persistent schedule), ragged
# edges, PSF widths from both instantiation units, kz above and below the volume depth
CASES = [
    ((20, 256, 256), (7, 15, 15), 3, 1),
    ((19, 200, 301), (3, 5, 9), 4, 0),
    ((24, 130, 520), (5, 9, 31), 2, 1),
    ((13, 300, 300), (9, 3, 3), 3, 1),
    ((320, 64, 64), (1, 7, 7), 5, 0),
    # one tile per plane and a deep PSF: most items wait for their neighbours' previous pass
    ((400, 64, 64), (15, 3, 3), 4, 1),
    ((16, 128, 600), (3, 3, 21), 1, 1),
]


@pytest.mark.parametrize("shape,pshape,iters,init", CASES, ids=[f"{s}-{p}" for s, p, _, _ in CASES])
def test_persistent_equals_per_pass(cuda, shape, pshape, iters, init):
    psf = gaussian(pshape, [max(0.6, n / 5) for n in pshape])
    obs = observed(shape, psf, sum(shape) + sum(pshape))
    a = run(obs, psf, iters, init, per_pass=False)
    b = run(obs, psf, iters, init, per_pass=True)
    assert np.array_equal(a, b)


def test_persistent_u8_and_strided_outputs_equal_per_pass(cuda):
    t = torch()
    shape, psf = (18, 260, 270), gaussian((3, 7, 7), (1.0, 1.5, 1.5))
    obs = observed(shape, psf, 3)
    # u8 estimate: the float estimate lives in scratch and is written with to_gray8 at the end
    u8 = [run(obs, psf, 4, 1, per_pass=p, out=empty_like_np(shape, np.uint8)) for p in (False, True)]
    assert np.array_equal(u8[0], u8[1])
    # a strided f32 estimate with a given start: the run works on a packed copy
    rng = np.random.default_rng(4)
    start = (rng.random(shape) * 50 + 1).astype(np.float32)
    outs = []
    for p in (False, True):
        big = t.zeros((shape[0], shape[1], 2 * shape[2]), device="cuda")
        view = big[:, :, ::2]
        outs.append(run(obs, psf, 3, 2, per_pass=p, out=view, start=start))
        assert float(big[:, :, 1::2].abs().max()) == 0.0
    assert np.array_equal(outs[0], outs[1])


def test_persistent_matches_oracle(cuda):
    shape = (24, 192, 448)  # 3 x 7 x 24 = 504 tiles: the persistent schedule
    psf = gaussian((5, 7, 9), (1.0, 1.5, 2.0))
    obs = observed(shape, psf, 5)
    ref = oracle.rl(obs, psf, 4, 1e-6, init=1)
    est = run(obs, psf, 4, 1, per_pass=False)
    assert rel_l2(est, ref) <= TOL
    assert float(np.max(np.abs(est.astype(np.float64) - ref))) <= TOL * float(np.max(np.abs(ref)))


def test_persistent_statistics_match_per_pass_and_oracle(cuda):
    # per-iteration flux and relative change from the persistent run: the same estimate bits as
    # one launch per pass, statistics equal to rounding (the schedules group the FP32 partial
    # sums differently) and to the oracle's within the RL test's bars
    t = torch()
    shape, psf = (18, 200, 280), gaussian((5, 7, 7), (1.0, 1.5, 1.5))  # 4 x 5 x 18 = 360 tiles
    obs = observed(shape, psf, 9)
    iters = 5
    results = []
    for per_pass in (False, True):
        rl = iane_gb300.RichardsonLucy(to_gpu(psf), shape, per_pass=per_pass)
        est = empty_like_np(shape, np.float32)
        st = t.zeros(2 * iters, dtype=t.float64, device="cuda")
        rl.run(to_gpu(obs), est, iters, 1e-6, init=rl.INIT_MEAN, stats=st)
        iane_gb300.device_status()
        results.append((to_host(est), to_host(st).reshape(-1, 2)))
        rl.close()
    (e_p, s_p), (e_s, s_s) = results
    assert np.array_equal(e_p, e_s)
    assert np.allclose(s_p, s_s, rtol=1e-6, atol=0.0)
    ref, ref_stats = oracle.rl(obs, psf, iters, 1e-6, init=1, with_stats=True)
    assert rel_l2(e_p, ref) <= TOL
    assert np.allclose(s_p[:, 0], ref_stats[:, 0], rtol=1e-5)
    assert np.allclose(s_p[:, 1], ref_stats[:, 1], rtol=1e-3, atol=1e-7)
