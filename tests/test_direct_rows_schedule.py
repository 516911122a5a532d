"""The row-strip direct convolution (iane_gb300/csrc/direct_rows.cu) restated in numpy and run on
the CPU with the kernel's own index arithmetic: TMA boxes of 32 input rows into a 3-slot ring of
96 rows, box k issued at the start (k < 3) or after step k - 3, waited for and fixed at the end
of step k - 2 (boxes 0 and 1 before step 0), clamp and mirror fix-ups once per box (the RX
columns beside the image by one reflection, then whole rows outside the image from the rows they
map to), and per lane (4 columns x 8 rows) the window rows base + m with the
ring's wrap taken as `m < room ? lo : hi`.

Every shared-memory read checks that its slot holds the box the index arithmetic expects and
that the box has landed (not in flight), every access stays inside the ring, and the whole
output equals a float64 direct convolution with the border rule -- for square and non-square
kernels (line filters included), the three borders, ragged image sizes and chunkings, including a
last chunk of one row."""
from __future__ import annotations

import numpy as np
import pytest

STEP, SLOTS, SW, LANE_ROWS = 32, 3, 128, 8
RING = STEP * SLOTS


def map_coord(c, n, border):
    """Border rule of the library (common.cuh map_coord): None for a zero sample."""
    if 0 <= c < n:
        return c
    if border == "zero":
        return None
    if border == "clamp":
        return 0 if c < 0 else n - 1
    period = 2 * n
    m = c % period
    return m if m < n else period - 1 - m


def reference(src, k, border):
    ny, nx = src.shape
    ry, rx = k.shape[0] // 2, k.shape[1] // 2
    out = np.zeros_like(src, dtype=np.float64)
    for y in range(ny):
        for x in range(nx):
            acc = 0.0
            for b in range(k.shape[0]):
                gy = map_coord(y + ry - b, ny, border)
                if gy is None:
                    continue
                for q in range(k.shape[1]):
                    gx = map_coord(x + rx - q, nx, border)
                    if gx is not None:
                        acc += k[b, q] * src[gy, gx]
            out[y, x] = acc
    return out


class Block:
    def __init__(self, src, k, border, x0, c0, c1):
        self.src, self.k, self.border = src, k, border
        self.ny, self.nx = src.shape
        self.KY, self.KX = k.shape
        self.RY, self.RX = self.KY // 2, self.KX // 2
        self.RA = (self.RX + 3) & ~3
        self.D = self.RA - self.RX
        self.AW = SW + 2 * self.RA
        self.SEG = (self.D + 4 + 2 * self.RX + 3) & ~3
        self.ROWS = LANE_ROWS + 2 * self.RY
        self.x0, self.c0, self.c1 = x0, c0, c1
        self.g0 = c0 - self.RY
        self.ring = np.full((RING, self.AW), np.nan)
        self.slot_box = [None] * SLOTS      # box issued into each slot
        self.landed = [False] * SLOTS
        self.mapped = border != "zero"
        self.edge_x = self.mapped and (x0 - self.RX < 0 or x0 + SW + self.RX > self.nx)

    def issue(self, kb):
        s = kb % SLOTS
        if self.slot_box[s] is not None:
            assert self.landed[s], "slot reissued before its box was waited for"
        self.slot_box[s], self.landed[s] = kb, False
        # TMA box: x from x0 - RA (16-byte aligned), rows g0 + STEP kb, zero fill outside
        assert ((self.x0 - self.RA) * 4) % 16 == 0
        self.pending = getattr(self, "pending", {})
        self.pending[kb] = s

    def wait(self, kb):
        s = self.pending.pop(kb)
        assert self.slot_box[s] == kb and not self.landed[s]
        top = self.g0 + STEP * kb
        for r in range(STEP):
            g = top + r
            for c in range(self.AW):
                gx = self.x0 - self.RA + c
                inside = 0 <= g < self.ny and 0 <= gx < self.nx
                self.ring[s * STEP + r, c] = self.src[g, gx] if inside else 0.0
        self.landed[s] = True

    def row_of(self, ring_row, box_expected):
        s = ring_row // STEP
        assert 0 <= ring_row < RING
        assert self.slot_box[s] == box_expected and self.landed[s], (ring_row, box_expected, self.slot_box, self.landed)
        return self.ring[ring_row]

    def fix(self, kb):
        s = kb % SLOTS
        RX, RY, AW = self.RX, self.RY, self.AW
        if self.edge_x:
            clamp = self.border == "clamp"
            for t in range(2 * STEP):           # a thread per row and side, one reflection
                r, right = t % STEP, t >= STEP
                for j in range(RX):
                    gx = self.nx + j if right else -RX + j
                    gm = (self.nx - 1 if clamp else 2 * self.nx - 1 - gx) if right else (0 if clamp else -gx - 1)
                    assert gm == map_coord(gx, self.nx, self.border)
                    c, cs = gx - (self.x0 - self.RA), gm - (self.x0 - self.RA)
                    if 0 <= c < AW and 0 <= cs < AW:
                        self.ring[s * STEP + r, c] = self.ring[s * STEP + r, cs]
        top = self.g0 + STEP * kb
        if self.mapped and (top < 0 or top + STEP > self.ny):
            for r in range(STEP):
                g = top + r
                if (0 <= g < self.ny) or g < -RY or g >= self.ny + RY:
                    continue
                gm = map_coord(g, self.ny, self.border)
                src_row = (gm - self.g0) % RING
                # the source row is inside the image and resident: this box or the one before
                want_box = (gm - self.g0) // STEP
                assert want_box in (kb, kb - 1)
                self.row_of(src_row, want_box)
                dst_row = (STEP * kb + r) % RING
                assert dst_row // STEP == s
                self.ring[dst_row] = self.ring[src_row]

    def run(self, dst):
        nsteps = (self.c1 - self.c0 + STEP - 1) // STEP
        nboxes = nsteps + 1
        for kb in range(min(SLOTS, nboxes)):
            self.issue(kb)
        self.wait(0)
        self.fix(0)
        self.wait(1)
        self.fix(1)
        RX, RY, KX, KY = self.RX, self.RY, self.KX, self.KY
        for s in range(nsteps):
            for cy in range(4):
                for cx in range(32):
                    base = STEP * (s % SLOTS) + LANE_ROWS * cy
                    room = RING - base
                    acc = np.zeros((LANE_ROWS, 4))
                    for m in range(self.ROWS):
                        ring_row = (base + m) if m < room else (base + m - RING)
                        # the box this window row belongs to
                        box = (STEP * s + LANE_ROWS * cy + m) // STEP
                        assert box in (s, s + 1)
                        row = self.row_of(ring_row, box)
                        lo_col = 4 * cx
                        assert lo_col % 4 == 0 and lo_col + self.SEG <= self.AW
                        seg = row[lo_col:lo_col + self.SEG]
                        for j in range(LANE_ROWS):
                            b = j + 2 * RY - m
                            if 0 <= b < KY:
                                for q in range(KX):
                                    for i in range(4):
                                        acc[j, i] += self.k[b, q] * seg[self.D + i + 2 * RX - q]
                    x = self.x0 + 4 * cx
                    if x >= self.nx:
                        continue
                    for j in range(LANE_ROWS):
                        y = self.c0 + STEP * s + LANE_ROWS * cy + j
                        if y >= self.c1:
                            break
                        for i in range(4):
                            if x + i < self.nx:
                                assert np.isnan(dst[y, x + i]), "output written twice"
                                dst[y, x + i] = acc[j, i]
            if s + 2 < nboxes:
                self.wait(s + 2)
                self.fix(s + 2)
            if s + SLOTS < nboxes:
                self.issue(s + SLOTS)


def emulate(src, k, border, chunk):
    ny, nx = src.shape
    dst = np.full(src.shape, np.nan)
    for x0 in range(0, nx, SW):
        for c0 in range(0, ny, chunk):
            Block(src, k, border, x0, c0, min(c0 + chunk, ny)).run(dst)
    return dst


# kernel shapes as (ky, kx)
CASES = [((128, 128), (7, 7), "mirror", 128), ((197, 257), (7, 7), "clamp", 70), ((257, 200), (5, 5), "mirror", 128),
         ((140, 130), (3, 3), "zero", 40), ((160, 300), (7, 7), "zero", 65), ((258, 131), (7, 7), "mirror", 128),
         ((129, 256), (5, 5), "clamp", 128), ((130, 200), (1, 7), "mirror", 128), ((200, 129), (7, 1), "clamp", 70),
         ((131, 257), (3, 5), "mirror", 64), ((129, 140), (5, 3), "zero", 128), ((160, 130), (1, 3), "clamp", 128)]


@pytest.mark.parametrize("shape,k,border,chunk", CASES, ids=[f"{s}-{k}-{b}-{c}" for s, k, b, c in CASES])
def test_schedule_reads_resident_boxes_and_matches_direct_sums(shape, k, border, chunk):
    rng = np.random.default_rng(k[0] * 100 + k[1] * 10 + shape[0])
    src = rng.random(shape) * 2 - 1
    taps = rng.random(k)
    got = emulate(src, taps, border, chunk)
    assert not np.isnan(got).any(), "an output was never written"
    np.testing.assert_allclose(got, reference(src, taps, border), rtol=0, atol=1e-12)


def test_a_missing_row_fix_up_is_caught():
    # the checks have teeth: without the row fix-up the mirror border's top rows read zeros
    rng = np.random.default_rng(5)
    src = rng.random((128, 128))
    taps = rng.random((5, 5))
    orig = Block.fix

    def fix_columns_only(self, kb):
        mapped = self.mapped
        self.mapped = False
        orig(self, kb)
        self.mapped = mapped
    Block.fix = fix_columns_only
    try:
        got = emulate(src, taps, "mirror", 128)
    finally:
        Block.fix = orig
    assert not np.allclose(got, reference(src, taps, "mirror"))
