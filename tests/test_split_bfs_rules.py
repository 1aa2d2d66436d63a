"""The split BFS's output rule (st_spix_gb300/csrc/k_splitmerge.cu: bfs_reg), restated in
Python and checked against explicit distances.

The split (calc_split_candidate / calc_seg_split, split_merge.cu:758-859) needs, per pixel
of a superpixel, only d1 > d2, where d1 and d2 are the 4-connected BFS distances from the
two seeds (seed = 1, unreached = -1).  bfs_reg runs both searches layer by layer as bit
masks and keeps `early2`, the pixels seed 2 reached in a layer where seed 1 had not yet
reached them (seed 2 itself included); at the end d1 > d2 holds on
v1 & (~v2 | early2).  It writes d1 := 2 there and d1 := -1 at seed 1 when it is not in that
set, while d2 keeps -1 except 1 at seed 2 (kb_split_seed): the comparison of those stand-in
distances must equal the comparison of the true ones on every pixel.
"""
from collections import deque

import numpy as np
import pytest


def _bfs(mask, seed):
    d = -np.ones(mask.shape, int)
    if seed is None:
        return d
    d[seed] = 1
    q = deque([seed])
    while q:
        y, x = q.popleft()
        for dy, dx in ((1, 0), (-1, 0), (0, 1), (0, -1)):
            yy, xx = y + dy, x + dx
            if 0 <= yy < mask.shape[0] and 0 <= xx < mask.shape[1] and mask[yy, xx] and d[yy, xx] < 0:
                d[yy, xx] = d[y, x] + 1
                q.append((yy, xx))
    return d


def _layer(f, v, mask):
    a = np.zeros_like(f)
    a[1:, :] |= f[:-1, :]
    a[:-1, :] |= f[1:, :]
    a[:, 1:] |= f[:, :-1]
    a[:, :-1] |= f[:, 1:]
    return a & mask & ~v


@pytest.mark.parametrize("seed", range(6))
def test_stand_in_distances_give_the_same_split(seed):
    rng = np.random.default_rng(seed)
    for _ in range(60):
        H, W = int(rng.integers(2, 14)), int(rng.integers(2, 14))
        mask = rng.random((H, W)) < 0.7
        pts = np.argwhere(mask)
        if len(pts) == 0:
            continue
        s1 = tuple(pts[rng.integers(len(pts))]) if rng.random() < 0.9 else None
        s2 = tuple(pts[rng.integers(len(pts))]) if rng.random() < 0.9 else None
        if s1 is not None and s1 == s2:
            continue
        want = (_bfs(mask, s1) > _bfs(mask, s2)) & mask
        f1 = np.zeros_like(mask)
        f2 = np.zeros_like(mask)
        if s1 is not None:
            f1[s1] = True
        if s2 is not None:
            f2[s2] = True
        v1, v2 = f1.copy(), f2.copy()
        early2 = f2 & ~f1
        for _ in range(H * W + 1):
            f1, f2 = _layer(f1, v1, mask), _layer(f2, v2, mask)
            v1 |= f1
            v2 |= f2
            early2 |= f2 & ~v1
            if not (f1.any() or f2.any()):
                break
        second = v1 & (~v2 | early2)
        d1 = -np.ones(mask.shape, int)
        d2 = -np.ones(mask.shape, int)
        if s1 is not None:
            d1[s1] = 1
        if s2 is not None:
            d2[s2] = 1
        d1[second] = 2
        if s1 is not None and not second[s1]:
            d1[s1] = -1
        np.testing.assert_array_equal((d1 > d2) & mask, want)
