"""Seeded synthetic data of the benchmark shapes (no datasets are used).

* ellipsoid phantoms: background plus ellipsoids with given radius and intensity ranges;
* normalised (anisotropic) Gaussian PSFs of odd extents;
* blur by zero-border convolution (FFT, only to make data) and Poisson noise.

Arrays are C-ordered: shape ``(nz, ny, nx)`` for a volume whose IANE extents are
``[nx, ny, nz]``; sigmas are given in IANE axis order (x, y, z).
"""
from __future__ import annotations

import numpy as np


def gaussian_psf(extent_xyz, sigma_xyz) -> np.ndarray:
    """Normalised Gaussian PSF with IANE extents ``extent_xyz`` (odd), C-ordered array."""
    shape = tuple(reversed(extent_xyz))
    sig = tuple(reversed(sigma_xyz))
    grids = np.meshgrid(*[np.arange(n, dtype=np.float64) - n // 2 for n in shape], indexing="ij")
    g = np.exp(-0.5 * sum((x / s) ** 2 for x, s in zip(grids, sig)))
    return (g / g.sum()).astype(np.float32)


def ellipsoid_phantom(extent_xyz, count, radius=(2.0, 20.0), intensity=(50.0, 1000.0), background=10.0,
                      seed=0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    shape = tuple(reversed(extent_xyz))
    vol = np.full(shape, background, dtype=np.float32)
    for _ in range(count):
        centre = [rng.uniform(0, n) for n in shape]
        radii = [rng.uniform(*radius) for _ in shape]
        value = np.float32(rng.uniform(*intensity))
        lo = [max(0, int(np.floor(c - r))) for c, r in zip(centre, radii)]
        hi = [min(n, int(np.ceil(c + r)) + 1) for c, r, n in zip(centre, radii, shape)]
        if any(h <= l for l, h in zip(lo, hi)):
            continue
        grids = np.meshgrid(*[np.arange(l, h, dtype=np.float32) for l, h in zip(lo, hi)], indexing="ij")
        inside = sum(((g - c) / r) ** 2 for g, c, r in zip(grids, centre, radii)) <= 1.0
        box = tuple(slice(l, h) for l, h in zip(lo, hi))
        vol[box][inside] += value
    return vol


def blur_zero_border(vol: np.ndarray, psf: np.ndarray) -> np.ndarray:
    """Zero-border 'same' convolution by FFT (data generation only)."""
    full = [n + k - 1 for n, k in zip(vol.shape, psf.shape)]
    fv = np.fft.rfftn(vol.astype(np.float64), full)
    fk = np.fft.rfftn(psf.astype(np.float64), full)
    out = np.fft.irfftn(fv * fk, full)
    sl = tuple(slice(k // 2, k // 2 + n) for n, k in zip(vol.shape, psf.shape))
    return np.maximum(out[sl], 0.0).astype(np.float32)


def poisson(mean: np.ndarray, seed=1) -> np.ndarray:
    return np.random.default_rng(seed).poisson(mean.astype(np.float64)).astype(np.float32)


def rl_volume_workload(seed=0):
    """The 3-D RL benchmark input: 256x256x64 volume of 200 ellipsoids (radii 2-20, intensity
    50-1000) on background 10, blurred by the normalised 15x15x7 Gaussian PSF with sigma
    (2, 2, 1), with Poisson noise. Returns (observed, psf, truth)."""
    truth = ellipsoid_phantom((256, 256, 64), 200, seed=seed)
    psf = gaussian_psf((15, 15, 7), (2.0, 2.0, 1.0))
    observed = poisson(blur_zero_border(truth, psf), seed=seed + 1)
    return observed, psf, truth


def rl_volume_workload_bf16(seed=0):
    """The 3-D RL precision-path input: the same 256x256x64 ellipsoid phantom blurred by the
    normalised isotropic 9x9x9 Gaussian PSF with sigma 2.5, with Poisson noise."""
    truth = ellipsoid_phantom((256, 256, 64), 200, seed=seed)
    psf = gaussian_psf((9, 9, 9), (2.5, 2.5, 2.5))
    observed = poisson(blur_zero_border(truth, psf), seed=seed + 1)
    return observed, psf, truth


def batch_workload(count=256, seed=0, side=(64, 1024)):
    """Uneven 2-D batch: sides log-uniform in `side` (independently, so non-square), each
    image sparse point sources (0.2% of pixels, intensities 200-5000) on a smooth background
    (two broad Gaussian bumps, 5-40 counts), with its own normalised Gaussian PSF of odd
    size 3-31 and sigma 0.5-5. Returns (truths, psfs) as lists of C-ordered float32 arrays;
    blur and noise are applied by the caller (on the GPU in bench.py)."""
    rng = np.random.default_rng(seed)
    truths, psfs = [], []
    lo, hi = np.log(side[0]), np.log(side[1])
    for _ in range(count):
        nx = int(round(np.exp(rng.uniform(lo, hi))))
        ny = int(round(np.exp(rng.uniform(lo, hi))))
        yy, xx = np.meshgrid(np.arange(ny, dtype=np.float32), np.arange(nx, dtype=np.float32), indexing="ij")
        img = np.zeros((ny, nx), np.float32)
        for _b in range(2):
            cx, cy = rng.uniform(0, nx), rng.uniform(0, ny)
            s = rng.uniform(0.2, 0.6) * max(nx, ny)
            img += np.float32(rng.uniform(5, 40)) * np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) / (2 * s * s))
        npts = max(1, int(0.002 * nx * ny))
        img[rng.integers(0, ny, npts), rng.integers(0, nx, npts)] += rng.uniform(200, 5000, npts).astype(np.float32)
        k = int(rng.integers(1, 16)) * 2 + 1
        sigma = float(rng.uniform(0.5, 5.0))
        truths.append(img)
        psfs.append(gaussian_psf((k, k), (sigma, sigma)))
    return truths, psfs
