"""Parity at the benchmark configurations themselves.

* 2-D convolution (512x512 f32 U[0, 1) from seed 0, normalised 7x7 Gaussian sigma 1.5, mirror
  border): the exact mode is bit-identical to the reference's own result (a SHA-256 made by the
  reference, tests/golden/configs.npz); the fast FP32 modes of the direct and the separable
  filter satisfy |gpu - oracle| <= 1e-5 * conv(|src|, |k|) element-wise.
* 3-D Richardson-Lucy with the configuration's PSF (15x15x7, sigma 2, 2, 1), flat start and
  all 50 iterations, against the oracle on a 96x96x16 volume the oracle finishes in seconds:
  relative L2 <= 1e-5 and max |diff| <= 1e-5 * max |ref|, per-iteration flux within 1e-5.
* The same run at full size (256x256x64, 200 ellipsoids, Poisson): the input comes from the
  deterministic generator (its SHA-256 must equal the fixture's), and planes z = 0, 31, 63, every
  plane's sum and sum of squares, the flux and the norm are compared with the reference's own
  50-iteration result (the fixture) at the same bars.
"""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

import iane_gb300
import oracle
from conftest import rel_err_bound
from gpu_helpers import empty_like_np, magnitude, rel_l2, to_gpu, to_host, torch
from golden_cases import configs

pytestmark = pytest.mark.gpu

TOL = 1e-5


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def c1_image():
    return np.random.default_rng(0).random((512, 512), dtype=np.float32)


def test_c1_direct_exact_is_the_reference_result(cuda):
    g = configs()
    img, k = c1_image(), g["c1__kernel"]
    out = empty_like_np(img.shape, np.float32)
    iane_gb300.convolve(to_gpu(img), to_gpu(k), out, "mirror", exact=True)
    assert sha(to_host(out)) == str(g["c1__direct_sha256"])


def test_c1_direct_fast_within_bar(cuda):
    g = configs()
    img, k = c1_image(), g["c1__kernel"]
    ref = np.zeros_like(img)
    oracle.convolve(img, k, ref, "mirror")
    out = empty_like_np(img.shape, np.float32)
    iane_gb300.convolve(to_gpu(img), to_gpu(k), out, "mirror")
    assert rel_err_bound(to_host(out), ref, magnitude(img, k, "mirror")) <= TOL


def test_c1_separable_within_bar(cuda):
    g = configs()
    img, taps = c1_image(), g["c1__taps"]
    ref = np.zeros_like(img)
    oracle.convolve_separable(img, [taps, taps], ref, "mirror")
    out = empty_like_np(img.shape, np.float32)
    iane_gb300.convolve_separable(to_gpu(img), [to_gpu(taps), to_gpu(taps)], out, "mirror")
    outer = np.outer(taps, taps).astype(np.float32)
    assert rel_err_bound(to_host(out), ref, magnitude(img, outer, "mirror")) <= TOL


def gpu_rl(obs, psf, iterations):
    rl = iane_gb300.RichardsonLucy(to_gpu(psf), obs.shape)
    est = empty_like_np(obs.shape, np.float32)
    stats = torch().zeros(2 * iterations, dtype=torch().float64, device="cuda")
    rl.run(to_gpu(obs), est, iterations, 1e-6, init=rl.INIT_MEAN, stats=stats)
    out = to_host(est)
    iane_gb300.device_status()
    rl.close()
    return out, to_host(stats).reshape(-1, 2)


def test_c2_psf_all_50_iterations_against_oracle(cuda):
    psf = configs()["c2__psf"]
    obs, _ = oracle.det_rl_volume((96, 96, 16), 12, psf, seed=5)
    ref, ref_stats = oracle.rl(obs, psf, 50, 1e-6, init=1, with_stats=True)
    est, stats = gpu_rl(obs, psf, 50)
    assert rel_l2(est, ref) <= TOL, rel_l2(est, ref)
    assert float(np.max(np.abs(est.astype(np.float64) - ref))) <= TOL * float(np.max(np.abs(ref)))
    assert np.allclose(stats[:, 0], ref_stats[:, 0], rtol=TOL)


def test_c2_full_size_against_the_reference_run(cuda):
    g = configs()
    psf = g["c2__psf"]
    obs, _ = oracle.det_rl_volume((256, 256, 64), 200, psf, seed=0)
    assert sha(obs) == str(g["c2__observed_sha256"]), "the deterministic generator gave another input"
    est, stats = gpu_rl(obs, psf, int(g["c2__iterations"]))
    e64 = est.astype(np.float64)
    for plane, want in zip(g["c2__plane_index"], g["c2__planes"]):
        got = est[int(plane)]
        assert rel_l2(got, want) <= TOL, (int(plane), rel_l2(got, want))
        assert float(np.max(np.abs(got.astype(np.float64) - want))) <= TOL * float(np.max(np.abs(want)))
    assert np.allclose(e64.sum(axis=(1, 2)), g["c2__plane_sums"], rtol=TOL)
    assert np.allclose((e64 * e64).sum(axis=(1, 2)), g["c2__plane_sumsq"], rtol=2 * TOL)
    assert abs(e64.sum() - float(g["c2__flux"])) <= TOL * float(g["c2__flux"])
    assert abs(np.sqrt((e64 * e64).sum()) - float(g["c2__norm"])) <= TOL * float(g["c2__norm"])
    assert abs(stats[-1, 0] - float(g["c2__flux"])) <= TOL * float(g["c2__flux"])
