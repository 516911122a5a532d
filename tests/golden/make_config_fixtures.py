"""Generate tests/golden/configs.npz: the benchmark configurations run by the reference itself.

Run where the reference checkout is present: ``python tests/golden/make_config_fixtures.py``
(about ten minutes on eight cores: the 3-D run is 101 full-volume 15x15x7 convolutions).

* ``c1``: the 2-D configuration -- a 512x512 f32 image of U[0, 1) values (numpy PCG64, seed
  0; its bits are the same on every platform), the normalised 7x7 Gaussian with sigma 1.5
  (stored: numpy's exp may differ in the last bit between platforms), mirror border. The
  reference has no mirror border, so its result is its own ``iane::convolve`` of the
  explicitly mirror-padded image, cropped; the separable result is two of its convolutions
  with 7x1 and 1x7 kernels on the padded image (f32 in between), cropped. Stored as SHA-256
  digests of the f32 outputs.
* ``c2``: the 3-D Richardson-Lucy configuration at full size -- a 256x256x64 volume of 200
  ellipsoids (radii 2-20, intensities 50-1000, background 10) blurred by the normalised
  15x15x7 Gaussian PSF (sigma 2, 2, 1) with Poisson noise, from the deterministic generator
  ``oracle.det_rl_volume`` (seed 0, same bits everywhere; its SHA-256 is stored), then 50
  iterations of the reference's RL from the flat start at the mean. Stored: z planes 0, 31
  and 63 of the f32 result, the sum and the sum of squares of every z plane (float64), the
  total flux and the L2 norm.
"""
from __future__ import annotations

import hashlib
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from iane_gb300 import synth  # noqa: E402
from oracle import build as oracle_build  # noqa: E402

OUT = Path(__file__).resolve().parent / "configs.npz"

C2_EXTENT = (256, 256, 64)
C2_PSF = ((15, 15, 7), (2.0, 2.0, 1.0))
C2_ITERATIONS = 50
C2_PLANES = (0, 31, 63)


def c1_inputs():
    image = np.random.default_rng(0).random((512, 512), dtype=np.float32)
    kernel = synth.gaussian_psf((7, 7), (1.5, 1.5))
    return image, kernel


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main() -> int:
    if oracle_build.build_reference() is None:
        print("reference checkout not found", file=sys.stderr)
        return 1
    oracle_build.build_oracle()
    g = {}

    image, kernel = c1_inputs()
    padded = oracle.mirror_pad(image, (3, 3))
    full = np.zeros_like(padded)
    oracle.convolve(padded, kernel, full, "clamp", use_reference=True)
    direct = np.ascontiguousarray(full[3:-3, 3:-3])
    g["c1__kernel"] = kernel
    g["c1__direct_sha256"] = np.array(sha(direct))
    # separable: 1-D taps (the normalised 1-D Gaussian, sigma 1.5); the reference convolves the
    # padded image along x with a 1x7 kernel, then along y with a 7x1 kernel
    g1 = synth.gaussian_psf((7,), (1.5,))
    g["c1__taps"] = g1
    along_x = np.zeros_like(padded)
    oracle.convolve(padded, g1.reshape(1, 7), along_x, "clamp", use_reference=True)
    along_y = np.zeros_like(padded)
    oracle.convolve(along_x, g1.reshape(7, 1), along_y, "clamp", use_reference=True)
    g["c1__separable_sha256"] = np.array(sha(np.ascontiguousarray(along_y[3:-3, 3:-3])))

    psf = synth.gaussian_psf(*C2_PSF)
    observed, _ = oracle.det_rl_volume(C2_EXTENT, 200, psf, seed=0)
    g["c2__psf"] = psf
    g["c2__observed_sha256"] = np.array(sha(observed))
    t0 = time.perf_counter()
    est = oracle.rl(observed, psf, C2_ITERATIONS, 1e-6, init=1, use_reference=True)
    print(f"reference RL, {C2_ITERATIONS} iterations: {time.perf_counter() - t0:.0f} s")
    e64 = est.astype(np.float64)
    g["c2__planes"] = np.ascontiguousarray(est[list(C2_PLANES)])
    g["c2__plane_index"] = np.array(C2_PLANES, np.int32)
    g["c2__plane_sums"] = e64.sum(axis=(1, 2))
    g["c2__plane_sumsq"] = (e64 * e64).sum(axis=(1, 2))
    g["c2__flux"] = np.array(e64.sum())
    g["c2__norm"] = np.array(np.sqrt((e64 * e64).sum()))
    g["c2__iterations"] = np.array(C2_ITERATIONS, np.int32)

    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(g)} arrays)")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
