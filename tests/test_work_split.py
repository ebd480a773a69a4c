"""Work split of single-shot launches (FLETCHER_PlanSegments, host code):
every tile-plane is covered exactly once, CTA by CTA, and the busiest CTA
carries little more than an equal share.  Cases: the 504^3 and 256^3+8-cell
layer grids (648 and 153 tiles on 152 CTAs), a 128^3 grid, a tiny grid and
a fixed chunk count."""
import ctypes as C

import numpy as np
import pytest

from fletcher_petrobras_gb300 import _lib


def plan(ctas, ntx, nty, rows, zlo, depth, zchunks=0):
    lib = _lib.load()
    first = np.zeros(ctas + 1, np.int32)
    cost = C.c_long(0)
    n = lib.FLETCHER_PlanSegments(ctas, ntx, nty, rows, zlo, depth, zchunks, None, 0, _lib.iptr(first),
                                  C.byref(cost))
    assert n > 0
    seg = np.zeros((n, 4), np.int32)
    assert lib.FLETCHER_PlanSegments(ctas, ntx, nty, rows, zlo, depth, zchunks, _lib.iptr(seg), n,
                                     _lib.iptr(first), C.byref(cost)) == n
    return seg, first, cost.value


@pytest.mark.parametrize("ctas,ntx,nty,rows,depth,zchunks", [
    (152, 18, 36, 16, 568, 0),   # 576^3 grid, 16-row tiles
    (152, 9, 17, 16, 272, 0),    # 280^3 grid
    (152, 9, 23, 12, 272, 0),    # 280^3 grid, 12-row tiles
    (304, 18, 71, 8, 568, 0),    # 8-row tiles, two CTAs per SM
    (152, 4, 8, 16, 128, 0),     # 136^3 grid
    (152, 1, 2, 16, 14, 0),      # tiny grid
    (152, 18, 36, 16, 568, 3),   # fixed chunk count, partial round shared out
    (152, 18, 36, 16, 568, -3),  # fixed chunk count, all round-robin
])
def test_segments_cover_every_tile_plane_once(ctas, ntx, nty, rows, depth, zchunks):
    zlo = 4
    seg, first, cost = plan(ctas, ntx, nty, rows, zlo, depth, zchunks)
    assert first[0] == 0 and first[-1] == len(seg) and np.all(np.diff(first) >= 0)
    cover = np.zeros((nty, ntx, depth), np.int32)
    for x0, y0, z0, z1 in seg:
        assert z1 > z0 and zlo <= z0 and z1 <= zlo + depth
        tx, r = divmod(x0 - 4, 32)
        ty, r2 = divmod(y0 - 4, rows)
        assert r == 0 and r2 == 0 and 0 <= tx < ntx and 0 <= ty < nty
        cover[ty, tx, z0 - zlo:z1 - zlo] += 1
    assert np.all(cover == 1)
    # balance: the busiest CTA's planes (+4 a segment) against an equal share;
    # the planner's cost weighs shared-out pieces by 3/2, so it is no smaller
    share = ntx * nty * depth / ctas
    per = [sum(int(s[3] - s[2]) + 4 for s in seg[first[b]:first[b + 1]]) for b in range(ctas)]
    assert cost >= max(per)
    if zchunks == 0 and share >= 64:
        assert max(per) <= 1.06 * share + 24, (max(per), share)


def test_partial_round_is_shared_out():
    """153 tiles on 152 CTAs: every CTA gets close to 1/152 of the work,
    not two whole columns for one CTA."""
    seg, first, cost = plan(152, 9, 17, 16, 4, 272)
    share = 9 * 17 * 272 / 152
    per = [sum(int(s[3] - s[2]) + 4 for s in seg[first[b]:first[b + 1]]) for b in range(152)]
    assert max(per) < 1.1 * share
    assert np.count_nonzero(np.diff(first)) > 100
