"""The oracle and the deterministic input generator are pinned to the reference's runs of the
benchmark configurations (tests/golden/configs.npz, made by the reference itself): the oracle's
2-D mirror convolution and separable filter at the 2-D configuration are bit-identical to the
reference's, the generator gives the fixture's input bit for bit, and -- where the reference is
built here -- the oracle's 50-iteration RL with the 3-D configuration's PSF equals the live
reference's on a small volume."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

import oracle
from golden_cases import configs


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def c1_image():
    return np.random.default_rng(0).random((512, 512), dtype=np.float32)


def test_oracle_c1_mirror_direct_is_the_reference_result():
    g = configs()
    out = np.zeros((512, 512), np.float32)
    oracle.convolve(c1_image(), g["c1__kernel"], out, "mirror")
    assert sha(out) == str(g["c1__direct_sha256"])


def test_oracle_c1_separable_is_the_reference_result():
    g = configs()
    out = np.zeros((512, 512), np.float32)
    oracle.convolve_separable(c1_image(), [g["c1__taps"], g["c1__taps"]], out, "mirror")
    assert sha(out) == str(g["c1__separable_sha256"])


def test_generator_reproduces_the_fixture_input():
    g = configs()
    obs, truth = oracle.det_rl_volume((256, 256, 64), 200, g["c2__psf"], seed=0)
    assert sha(obs) == str(g["c2__observed_sha256"])
    assert obs.min() >= 0 and float(truth.min()) == 10.0


def test_generator_poisson_statistics():
    # a flat truth of 37 blurred by a normalised PSF is 37 away from the zero border:
    # the counts there have mean and variance 37
    psf = np.full((3, 3, 3), 1.0 / 27.0, np.float32)
    obs, _ = oracle.det_rl_volume((64, 64, 16), 0, psf, seed=9, background=37.0)
    inner = obs[1:-1, 1:-1, 1:-1].astype(np.float64)
    assert abs(inner.mean() - 37.0) < 0.1 and abs(inner.var() - 37.0) < 1.0


@pytest.mark.skipif(not oracle.reference_available(), reason="the reference is built only where its sources are")
def test_oracle_rl_50_iterations_matches_live_reference():
    psf = configs()["c2__psf"]
    obs, _ = oracle.det_rl_volume((64, 64, 8), 4, psf, seed=3)
    ours = oracle.rl(obs, psf, 50, 1e-6, init=1)
    ref = oracle.rl(obs, psf, 50, 1e-6, init=1, use_reference=True)
    assert np.array_equal(ours, ref)
