"""Batched uneven 2-D Richardson-Lucy: one persistent launch over a device work queue, in a
CUDA graph.

Every image of the batch must equal the single-image GPU path bit for bit (same fused tile
body, same tap order) and the CPU oracle within the RL tolerance, also for a batch of many
images whose passes overlap in the queue; graph replays must repeat results; the autotuner
must persist its choice per batch."""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import iane_gb300
import oracle
from gpu_helpers import empty_like_np, gaussian, rel_l2, to_gpu, to_host, torch

pytestmark = pytest.mark.gpu

SHAPES = [(20, 33), (64, 64), (70, 130), (129, 257), (5, 7), (96, 40), (200, 31), (33, 300), (1, 90)]
KS = [3, 5, 7, 9, 15, 21, 31, 11, 3]


def make_batch(seed=0):
    rng = np.random.default_rng(seed)
    obs, psfs = [], []
    for (ny, nx), k in zip(SHAPES, KS):
        truth = rng.random((ny, nx)).astype(np.float32) * 50 + 5
        truth[rng.integers(0, ny, 4), rng.integers(0, nx, 4)] += 2000
        psf = gaussian((k, k), (max(0.6, k / 5), max(0.6, k / 6)))
        blurred = np.zeros_like(truth)
        oracle.convolve(truth, psf, blurred, "zero")
        obs.append(rng.poisson(np.maximum(blurred, 0)).astype(np.float32))
        psfs.append(psf)
    return obs, psfs


def run_batch(batch, obs, iterations, init):
    outs = [empty_like_np(o.shape, np.float32) for o in obs]
    batch.run([to_gpu(o) for o in obs], outs, iterations, 1e-6, init=init)
    return [to_host(o) for o in outs]


def test_batch_matches_single_image_path_and_oracle(cuda):
    obs, psfs = make_batch()
    batch = iane_gb300.RichardsonLucyBatch([to_gpu(p) for p in psfs], [o.shape for o in obs])
    got = run_batch(batch, obs, 6, iane_gb300.RichardsonLucy.INIT_OBSERVED)
    for o, p, g in zip(obs, psfs, got):
        rl = iane_gb300.RichardsonLucy(to_gpu(p), o.shape)
        e = empty_like_np(o.shape, np.float32)
        rl.run(to_gpu(o), e, 6, 1e-6, init=rl.INIT_OBSERVED)
        single = to_host(e)
        rl.close()
        assert np.array_equal(g, single), o.shape
        ref = oracle.rl(o, p, 6, 1e-6, init=0)
        assert rel_l2(g, ref) <= 1e-5
    iane_gb300.device_status()
    batch.close()


def test_graph_replay_and_new_configuration(cuda):
    obs, psfs = make_batch(seed=1)
    batch = iane_gb300.RichardsonLucyBatch([to_gpu(p) for p in psfs], [o.shape for o in obs])
    g_obs = [to_gpu(o) for o in obs]
    outs = [empty_like_np(o.shape, np.float32) for o in obs]
    scratch = torch().empty(batch.scratch_bytes, dtype=torch().uint8, device="cuda")
    batch.run(g_obs, outs, 4, 1e-6, init=1, scratch=scratch)
    first = [to_host(o) for o in outs]
    for o in outs:
        o.zero_()
    batch.run(g_obs, outs, 4, 1e-6, init=1, scratch=scratch)  # graph replay
    assert all(np.array_equal(a, to_host(b)) for a, b in zip(first, outs))
    batch.run(g_obs, outs, 7, 1e-6, init=1, scratch=scratch)  # new schedule
    for o, p, b in zip(obs, psfs, outs):
        assert rel_l2(to_host(b), oracle.rl(o, p, 7, 1e-6, init=1)) <= 1e-5
    batch.close()


def test_many_images_overlapping_passes_match_single_image_path(cuda):
    # 48 images, most of them one or two tiles: each image's next pass starts while other
    # images are still in their previous one, so the per-image waits carry the ordering
    rng = np.random.default_rng(21)
    obs, psfs = [], []
    for i in range(48):
        ny, nx = int(rng.integers(8, 150)), int(rng.integers(8, 150))
        k = int(rng.integers(0, 16)) * 2 + 1
        truth = rng.random((ny, nx)).astype(np.float32) * 100 + 5
        obs.append(rng.poisson(truth).astype(np.float32))
        psfs.append(gaussian((k, k), (max(0.6, k / 5), max(0.6, k / 7))))
    batch = iane_gb300.RichardsonLucyBatch([to_gpu(p) for p in psfs], [o.shape for o in obs])
    got = run_batch(batch, obs, 9, iane_gb300.RichardsonLucy.INIT_MEAN)
    for o, p, g in zip(obs, psfs, got):
        rl = iane_gb300.RichardsonLucy(to_gpu(p), o.shape)
        e = empty_like_np(o.shape, np.float32)
        rl.run(to_gpu(o), e, 9, 1e-6, init=rl.INIT_MEAN)
        assert np.array_equal(g, to_host(e)), o.shape
        rl.close()
    iane_gb300.device_status()
    batch.close()


def test_u8_observed_and_estimates(cuda):
    rng = np.random.default_rng(22)
    shapes = [(70, 90), (33, 20), (128, 64)]
    obs = [rng.integers(0, 256, s).astype(np.uint8) for s in shapes]
    psfs = [gaussian((5, 5), (1.0, 1.0)), gaussian((3, 7), (0.8, 1.5)), gaussian((9, 9), (2.0, 2.0))]
    batch = iane_gb300.RichardsonLucyBatch([to_gpu(p) for p in psfs], shapes)
    outs = [empty_like_np(s, np.uint8) for s in shapes]
    batch.run([to_gpu(o) for o in obs], outs, 5, 1e-6, init=iane_gb300.RichardsonLucy.INIT_OBSERVED)
    for o, p, out in zip(obs, psfs, outs):
        ref = oracle.rl(o, p, 5, 1e-6, init=0)
        diff = to_host(out).astype(np.int32) - oracle.to_gray8(ref).astype(np.int32)
        assert np.all(np.abs(diff) <= 1)
        assert np.all((diff == 0) | (np.abs(ref - np.floor(ref) - 0.5) < 1e-3))
    batch.close()


AUTOTUNE_SCRIPT = r"""
import sys, numpy as np, torch
sys.path.insert(0, {root!r})
import iane_gb300
shapes = [(40, 300), (200, 210), (64, 64)]
psfs = [torch.ones((k, k), device="cuda") / (k * k) for k in (5, 15, 31)]
b = iane_gb300.RichardsonLucyBatch(psfs, shapes, autotune=True)
print(b.tile_widths(), b.launch_config())
"""


def test_autotune_cache_persists(cuda, tmp_path):
    cache = tmp_path / "tune.txt"
    env = dict(os.environ, IANE_GB_TUNE_CACHE=str(cache))
    root = str(Path(__file__).resolve().parent.parent)
    script = AUTOTUNE_SCRIPT.format(root=root)
    first = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=600)
    assert first.returncode == 0, first.stderr
    lines = cache.read_text().strip().splitlines()
    assert len(lines) == 1 and lines[0].count(" | ") == 2  # one measured line for the batch
    widths = [int(w) for w in first.stdout.strip().splitlines()[-1].split("]")[0].strip("[").split(",")]
    assert all(w in (64, 128, 256) for w in widths) and widths[2] == 64  # the 31-wide PSF: one tile per item
    second = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=600)
    assert second.returncode == 0, second.stderr
    assert second.stdout.strip() == first.stdout.strip()
    assert len(cache.read_text().strip().splitlines()) == 1  # read from the cache, nothing re-measured


@pytest.mark.parametrize("grouping", [0, 1, 2, 3])
def test_every_item_shape_matches_the_single_image_path(cuda, grouping):
    # the autotuner's item shapes (1, 2 or 4 tiles per item by PSF width) pinned one by one,
    # with both queue orders and 1 and 4 CTAs per SM: the same bits as the single-image path
    obs, psfs = make_batch(seed=3)
    singles = []
    for o, p in zip(obs, psfs):
        rl = iane_gb300.RichardsonLucy(to_gpu(p), o.shape)
        e = empty_like_np(o.shape, np.float32)
        rl.run(to_gpu(o), e, 4, 1e-6, init=rl.INIT_MEAN)
        singles.append(to_host(e))
        rl.close()
    batch = iane_gb300.RichardsonLucyBatch([to_gpu(p) for p in psfs], [o.shape for o in obs])
    for bps, order in ((1, 0), (4, 1)):
        batch.configure(bps, order, grouping)
        assert batch.launch_config() == (bps, order, grouping)
        widths = batch.tile_widths()
        assert all(w in (64, 128, 256) for w in widths)
        got = run_batch(batch, obs, 4, iane_gb300.RichardsonLucy.INIT_MEAN)
        for g, s in zip(got, singles):
            assert np.array_equal(g, s)
    with pytest.raises(iane_gb300.IaneError):
        batch.configure(1, 0, 4)
    batch.close()
