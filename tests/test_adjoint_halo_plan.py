"""Host replica of the adjoint's halo-cell enumeration (halo_plan and
halo_cell in csrc/adjoint.cu): thread ids 0 .. na + rows_b*nseg*32 map to
(i, j, c) so that every halo cell of the grid (a cell within r of an edge on
any axis) is produced exactly once and no interior cell is, in 2-D and 3-D,
for grids down to a single interior cell. CPU only."""

import numpy as np
import pytest


def halo_plan(dim, d0, d1, last, R):
    rows = d0 if dim == 2 else d0 * d1
    inner_rows = (d0 - 2 * R) if dim == 2 else (d0 - 2 * R) * (d1 - 2 * R)
    na = (inner_rows * 2 * R + 31) // 32 * 32
    return na, rows - inner_rows, (last + 31) // 32


def halo_cell(dim, d0, d1, last, R, plan, tid):
    na, rows_b, nseg = plan
    j = 0
    if tid < na:
        row, e = divmod(tid, 2 * R)
        if dim == 2:
            if row >= d0 - 2 * R:
                return None
            i = R + row
        else:
            w1 = d1 - 2 * R
            if row >= (d0 - 2 * R) * w1:
                return None
            i = R + row // w1
            j = R + (row - (i - R) * w1)
        c = e if e < R else last - 2 * R + e
        return i, j, c
    b = tid - na
    wrow, seg = divmod(b >> 5, nseg)
    if wrow >= rows_b:
        return None
    c = seg * 32 + (b & 31)
    if c >= last:
        return None
    if dim == 2:
        i = wrow if wrow < R else d0 - 2 * R + wrow
    else:
        full = 2 * R * d1
        if wrow < full:
            p = wrow // d1
            i = p if p < R else d0 - 2 * R + p
            j = wrow - p * d1
        else:
            q = wrow - full
            i = R + q // (2 * R)
            jj = q - (i - R) * 2 * R
            j = jj if jj < R else d1 - 2 * R + jj
    return i, j, c


@pytest.mark.parametrize("R", [1, 2, 3, 4])
@pytest.mark.parametrize("n", [(1, 1), (1, 37), (5, 2), (9, 40), (33, 70)])
def test_halo_enumeration_2d(R, n):
    d0, last = n[0] + 2 * R, n[1] + 2 * R
    plan = halo_plan(2, d0, 1, last, R)
    seen = np.zeros((d0, last), np.int32)
    for tid in range(plan[0] + plan[1] * plan[2] * 32):
        cell = halo_cell(2, d0, 1, last, R, plan, tid)
        if cell is not None:
            i, j, c = cell
            assert j == 0 and 0 <= i < d0 and 0 <= c < last
            seen[i, c] += 1
    halo = np.ones((d0, last), bool)
    halo[R:d0 - R, R:last - R] = False
    assert (seen[halo] == 1).all() and (seen[~halo] == 0).all()


@pytest.mark.parametrize("R", [1, 2, 3])
@pytest.mark.parametrize("n", [(1, 1, 1), (2, 3, 40), (6, 5, 4), (7, 9, 33)])
def test_halo_enumeration_3d(R, n):
    d0, d1, last = (x + 2 * R for x in n)
    plan = halo_plan(3, d0, d1, last, R)
    seen = np.zeros((d0, d1, last), np.int32)
    for tid in range(plan[0] + plan[1] * plan[2] * 32):
        cell = halo_cell(3, d0, d1, last, R, plan, tid)
        if cell is not None:
            i, j, c = cell
            assert 0 <= i < d0 and 0 <= j < d1 and 0 <= c < last
            seen[i, j, c] += 1
    halo = np.ones((d0, d1, last), bool)
    halo[R:d0 - R, R:d1 - R, R:last - R] = False
    assert (seen[halo] == 1).all() and (seen[~halo] == 0).all()
