"""Host replica of the 3-D tile kernel's index arithmetic
(csrc/kernel3d_tile.cuh, the planner's geometry3d in csrc/engine.cu): for
every degree the build instantiates and a set of grid shapes, each interior
cell of a plane is stored by exactly one (tile, warp row, lane element);
every store and every fixed-halo load stays inside its plane; each tensor
copy starts on a 16-byte boundary; and every stored cell lies inside the
part of the tile that is still valid after B levels (rows and columns at
least (B-1)*r inside the computed tile). CPU only."""
import numpy as np
import pytest

from gbstencil import capi


def layout(R, V, n):
    """make_layout of csrc/engine.cu for a cube of interior n (3-D)."""
    d = [x + 2 * R for x in n]
    shift = (V - R % V) % V
    need = shift + d[2] + 32 * V
    align = 128 // (16 // V)
    pitch = -(-need // align) * align
    return d, shift, pitch


def tile_shape(R, V, B, TJ):
    ROW = 32 * V
    OFF = -(-((B - 1) * R) // V) * V
    WK = (ROW - (B - 1) * R - OFF) // V * V
    JOUT = TJ - 2 * (B - 1) * R
    PADE = -(-R // V) * V
    return ROW, OFF, WK, JOUT, PADE


def check(R, V, B, TJ, H, n, sl):
    d, shift, pitch = layout(R, V, n)
    ROW, OFF, WK, JOUT, PADE = tile_shape(R, V, B, TJ)
    assert WK > 0 and JOUT > 0
    nk, nj, ni = n[2], n[1], n[0]
    ntk, ntj = -(-nk // WK), -(-nj // JOUT)
    nblocks = -(-ni // sl)
    NW = TJ // H
    plane = d[0] * d[1] * pitch
    cover = np.zeros((d[1], d[2]), np.int32)   # one plane's j x k coverage
    for tk in range(ntk):
        cs = R + tk * WK
        ce = min(cs + WK, d[2] - R)
        ws = shift + cs - OFF
        assert ws % V == 0 and (ws - PADE) % V == 0          # tensor-copy x on a 16-byte boundary
        for tj in range(ntj):
            js = R + tj * JOUT
            je = min(js + JOUT, d[1] - R)
            jt = js - (B - 1) * R
            for w in range(NW):
                for h in range(H):
                    jr = jt + w * H + h
                    for lane in range(32):
                        col0 = ws - shift + lane * V
                        lane_in_row = ws + lane * V >= 0 and ws + lane * V + V <= pitch
                        if lane_in_row and 0 <= jr < d[1]:   # fixed-halo loads (rows of plane q)
                            base = jr * pitch + ws + lane * V
                            assert 0 <= base and base + V <= d[1] * pitch
                        if not (js <= jr < je):
                            continue
                        for e in range(V):
                            c = col0 + e
                            if cs <= c < ce:
                                # valid after B levels: rows and window columns (B-1)R inside
                                assert jt + (B - 1) * R <= jr < jt + TJ - (B - 1) * R
                                wc = c - (ws - shift)
                                assert (B - 1) * R <= wc < ROW - (B - 1) * R
                                el = jr * pitch + ws + lane * V + e
                                assert 0 <= el < d[1] * pitch
                                cover[jr, c] += 1
    inner = cover[R:d[1] - R, R:d[2] - R]
    assert (inner == 1).all(), (int(inner.min()), int(inner.max()))
    assert cover.sum() == inner.sum()                        # nothing outside the interior
    # planes: every interior plane stored by exactly one stream block
    planes = np.zeros(d[0], np.int32)
    for blk in range(nblocks):
        i0 = R + blk * sl
        i1 = min(i0 + sl, d[0] - R)
        pstart, pend = max(0, i0 - B * R), min(d[0], i1 + B * R)
        assert 0 <= pstart and pend <= d[0]
        planes[i0:i1] += 1
    assert (planes[R:d[0] - R] == 1).all() and planes.sum() == ni
    assert plane > 0


SHAPES = [(1, 4, 1, 64, 4), (2, 4, 1, 64, 4), (1, 4, 2, 64, 4), (1, 4, 3, 32, 2), (1, 4, 4, 32, 2),
          (2, 4, 2, 32, 2), (2, 4, 3, 16, 1), (1, 2, 1, 64, 4), (2, 2, 1, 64, 4), (1, 2, 2, 64, 4),
          (2, 2, 2, 32, 2), (3, 4, 1, 16, 1), (4, 2, 1, 16, 1), (3, 2, 2, 16, 1),
          # the high degrees of FMA mode: one row per warp, few output rows
          (1, 4, 5, 16, 1), (1, 4, 8, 16, 1), (1, 2, 6, 16, 1), (1, 2, 8, 16, 1), (2, 4, 4, 16, 1),
          (2, 2, 4, 16, 1)]


@pytest.mark.parametrize("R,V,B,TJ,H", SHAPES)
@pytest.mark.parametrize("n,sl", [([11, 11, 11], 4), ([20, 37, 150], 7), ([9, 70, 257], 9)])
def test_tile_kernel_index_arithmetic(R, V, B, TJ, H, n, sl):
    check(R, V, B, TJ, H, n, sl)
