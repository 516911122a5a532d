"""The index arithmetic of the tiled convolution body (iane_gb300/csrc/conv_tile.cuh) restated
in Python and checked on the CPU for every PSF width and both lane geometries (8 x 4 and
16 x 2 outputs per lane): the TMA box starts on a 16-byte boundary, every 128-bit shared load
of a lane's row segment starts on a 16-byte boundary and ends inside the tile's row, every tap
reads a segment element that exists, and the 16 x 2 body's split of the input rows (checked
head and tail rows, unchecked interior rows) visits every row once and leaves no kernel-row
check out of a row that needs one."""
from __future__ import annotations

import pytest

KRX, KRY = 8, 4


def geom(kx):
    rx = kx // 2
    rxa = (rx + 3) & ~3
    d = rxa - rx
    kxp = (kx + 3) & ~3
    return rx, rxa, d, kxp


def segn(kx, rx_out):
    rx, rxa, d, _ = geom(kx)
    return (d + rx_out + kx - 1 + 3) & ~3


def width(kx, wx):
    """TileWidth<KX, WX>: columns read W and pitch P (floats)."""
    tx = 32 * wx
    w = tx - KRX + segn(kx, KRX)
    p = w + 4 if w % 8 == 0 else w
    return w, p


WIDTHS = list(range(1, 32, 2))


@pytest.mark.parametrize("kx", WIDTHS)
@pytest.mark.parametrize("wx", [1, 2])
@pytest.mark.parametrize("rx_out,ry_out", [(8, 4), (16, 2)])
def test_lane_segments_stay_inside_the_tile_row(kx, wx, rx_out, ry_out):
    rx, rxa, d, kxp = geom(kx)
    assert rxa % 4 == 0 and 0 <= d <= 3                  # TMA x start x0 - RXA: 16-byte aligned
    w, p = width(kx, wx)
    assert p % 4 == 0 and p >= w                           # rows start 16-byte aligned
    sn = segn(kx, rx_out)
    assert sn % 4 == 0
    lanes_x = 32 // rx_out
    for lane_x in range(lanes_x * wx):
        start = rx_out * lane_x
        assert start % 4 == 0                              # 128-bit loads at 16-byte boundaries
        assert start + sn <= w                             # the segment ends inside the columns read
    # the tile's width does not depend on the lane geometry
    assert (32 * wx - rx_out + sn) == w
    # every tap of every output reads a loaded segment element
    for i in range(rx_out):
        for q in range(kx):
            idx = d + i + 2 * rx - q
            assert 0 <= idx < sn
    # kernel rows are padded to 16-byte rows of KXP floats
    assert kxp % 4 == 0 and kxp >= kx


@pytest.mark.parametrize("ky", WIDTHS + [33, 63])
@pytest.mark.parametrize("ry_out", [2, 4])
def test_row_split_visits_every_row_once(ky, ry_out):
    # plane_sums for the 16 x 2 geometry: rows [0, lo) and [hi, rows) checked, [lo, hi) not
    ry = ky // 2
    rows = ry_out + 2 * ry
    lo = min(ry_out - 1, 2 * ry + 1)
    hi = max(2 * ry + 1, lo)
    visited = list(range(0, lo)) + list(range(lo, hi)) + list(range(hi, rows))
    assert visited == list(range(rows))
    for r in range(lo, hi):
        for j in range(ry_out):
            b = j + 2 * ry - r
            assert 0 <= b < ky                             # unchecked rows: every kernel row exists
    # and the checked rows hold exactly the pairs the direct definition needs
    pairs = {(r, j) for r in range(rows) for j in range(ry_out) if 0 <= j + 2 * ry - r < ky}
    assert pairs == {(y + 2 * ry - b, y) for y in range(ry_out) for b in range(ky)}


@pytest.mark.parametrize("kx", WIDTHS)
def test_narrow_staging_box_is_16_byte_aligned(kx):
    # kTileTmaNarrow: the raw box starts 16 elements left of the tile and covers its W columns
    # from RXA left of it, so its x coordinate and row bytes are 16-byte multiples
    rx, rxa, _, _ = geom(kx)
    for wx in (1, 2):
        w, _ = width(kx, wx)
        for esize in (1, 2):
            box = (((16 - rxa + w) * esize + 15) & ~15) // esize
            assert (16 * esize) % 16 == 0                   # x start x0 - 16: 16-byte aligned
            assert (box * esize) % 16 == 0 and box >= 16 - rxa + w
            assert (16 - rxa) % 4 == 0                      # the float tile starts on a 4-cell group
