"""Size-independent properties at the full 3-D RL size (256x256x64 f32, 15x15x7 kernels), where
the oracle would take minutes: delta kernels reproduce or shift the input exactly, the
convolution is linear within the FP32 bar, and the separable filter equals the direct
filter of the outer-product kernel within the same bar."""
from __future__ import annotations

import numpy as np
import pytest

import iane_gb300
from gpu_helpers import gaussian, torch

pytestmark = pytest.mark.gpu

SHAPE = (64, 256, 256)
KSHAPE = (7, 15, 15)


def _volume(seed):
    t = torch()
    g = t.Generator(device="cuda")
    g.manual_seed(seed)
    return t.rand(SHAPE, generator=g, device="cuda") * 100


def test_centred_delta_reproduces_the_volume(cuda):
    t = torch()
    vol = _volume(1)
    k = t.zeros(KSHAPE, device="cuda")
    k[3, 7, 7] = 1.0
    out = t.empty_like(vol)
    for border in ("zero", "clamp", "mirror"):
        iane_gb300.convolve(vol, k, out, border)
        assert t.equal(out, vol), border


def test_off_centre_delta_shifts_the_volume(cuda):
    # tap (dz, dy, dx) = (+1, -2, +3) from the centre: out[p] = in[p - d] (true convolution),
    # zeros entering from the zero border
    t = torch()
    vol = _volume(2)
    k = t.zeros(KSHAPE, device="cuda")
    k[3 + 1, 7 - 2, 7 + 3] = 1.0
    out = t.empty_like(vol)
    iane_gb300.convolve(vol, k, out, "zero")
    want = t.zeros_like(vol)
    want[1:, :-2, 3:] = vol[:-1, 2:, :-3]
    assert t.equal(out, want)


def test_linearity(cuda):
    t = torch()
    x, y = _volume(3), _volume(4)
    k = t.from_numpy(gaussian(KSHAPE, (1.0, 2.0, 2.0))).cuda()
    cx, cy, cs = t.empty_like(x), t.empty_like(x), t.empty_like(x)
    iane_gb300.convolve(x, k, cx, "zero")
    iane_gb300.convolve(y, k, cy, "zero")
    iane_gb300.convolve(2 * x + 3 * y, k, cs, "zero")
    # FP32 sums of positive terms: each result within 1e-5 of its magnitude
    mag = 2 * cx + 3 * cy
    assert float(((cs - mag).abs() / mag).max()) <= 1e-5


def test_separable_equals_direct_outer_product(cuda):
    t = torch()
    vol = _volume(5)
    gz, gy, gx = (gaussian((n,), (s,)) for n, s in ((7, 1.0), (15, 2.0), (15, 2.0)))
    k3 = t.from_numpy(np.einsum("i,j,k->ijk", gz, gy, gx).astype(np.float32)).cuda()
    direct, sep = t.empty_like(vol), t.empty_like(vol)
    for border in ("zero", "mirror"):
        iane_gb300.convolve(vol, k3, direct, border)
        iane_gb300.convolve_separable(vol, [t.from_numpy(gx).cuda(), t.from_numpy(gy).cuda(), t.from_numpy(gz).cuda()],
                                      sep, border)
        assert float(((sep - direct).abs() / direct.abs()).max()) <= 1e-5, border
