"""The split y pass of the morphology cube kernel (iane_gb300/csrc/morphology.cu,
cube_y_pass) restated in Python and compared with the reference's direct scan
(include/iane/algorithms/morphology/morphology.hpp:44-71: `value < result` for erosion in
increasing order, `value > result` for dilation in decreasing order): the four windows of a
thread, split between their rows 3 and 4, give the same values and the same signed zeros on
random windows with NaN, signed zeros, infinities and integer ties."""
from __future__ import annotations

import math
import random
import struct

import pytest

OY = 4


def direct(col, k, r, dilate, start):
    m = start
    for o in range(2 * r + 1):
        v = col[k + (2 * r - o if dilate else o)]
        if (v > m) if dilate else (v < m):
            m = v
    return m


def split(col, r, dilate, start):
    out = [None] * OY
    part = [None] * OY
    run = start
    for k in range(OY - 1, -1, -1):
        v = col[k]
        if (v > run) if dilate else (v <= run):
            run = v
        part[k] = run
    edge = start
    for j in range(OY, OY + 2 * r):
        v = col[j]
        if (v >= edge) if dilate else (v < edge):
            edge = v
        k = j - 2 * r
        if k >= 0:
            if dilate:
                out[k] = part[k] if part[k] > edge else edge
            else:
                out[k] = edge if edge < part[k] else part[k]
    return out


def key(v):
    return struct.pack("<d", v) if isinstance(v, float) else v


@pytest.mark.parametrize("dilate", [False, True], ids=["erode", "dilate"])
@pytest.mark.parametrize("radius", [2, 3])
def test_split_windows_match_the_direct_scan(radius, dilate):
    rng = random.Random(radius * 2 + dilate)
    floats = [math.nan, 0.0, -0.0, 1.0, -1.0, 2.5, math.inf, -math.inf]
    for trial in range(20000):
        if trial % 2:
            col = [rng.choice(floats) for _ in range(OY + 2 * radius)]
            start = -math.inf if dilate else math.inf
        else:
            col = [rng.randint(0, 3) for _ in range(OY + 2 * radius)]
            start = -(1 << 31) if dilate else (1 << 31) - 1
        want = [direct(col, k, radius, dilate, start) for k in range(OY)]
        got = split(col, radius, dilate, start)
        assert [key(v) for v in got] == [key(v) for v in want], (col, got, want)
