"""The union rules of the disconnected-region kernels (st_spix_gb300/csrc/k_prop.cu:
kb_cc_local, kb_cc_hook), restated in Python and checked against 8-connected labelling.

kb_cc_local joins the pixels of each 32 x 32 tile: runs of equal labels within a tile row
(a pixel's parent starts at its run's first pixel), a pixel unites with N unless its left
pixel and NW both carry its label, with NW when neither the left pixel nor N carries it,
and with NE when N does not (pairs inside the tile only).  kb_cc_hook makes the unions of
the 8-connected rule (split_disconnected.cu:33-96 as restated in cc_unions) across tile
edges.  Union-find with min-index hooking then gives every pixel the smallest pixel index
of its component.  The two rule sets together must connect exactly the 8-connected
same-label components; this is what the test checks, on random label images with holes
(-1) and frame sizes that leave partial tiles.
"""
import numpy as np
import pytest

ndimage = pytest.importorskip("scipy.ndimage")

TILE = 32


def _find(p, x):
    while p[x] != x:
        p[x] = p[p[x]]
        x = p[x]
    return x


def _unite(p, a, b):
    a, b = _find(p, a), _find(p, b)
    if a == b:
        return
    if a < b:
        a, b = b, a
    p[a] = b


def _kernel_roots(seg):
    H, W = seg.shape
    flat = seg.ravel()
    par = np.arange(H * W)
    par[flat < 0] = -1
    # kb_cc_local: runs, then the run unions
    for y in range(H):
        for x in range(W):
            L = seg[y, x]
            if L >= 0 and x % TILE > 0 and seg[y, x - 1] == L:
                par[y * W + x] = par[y * W + x - 1]
    for y in range(H):
        for x in range(W):
            L = seg[y, x]
            if L < 0 or y % TILE == 0:
                continue
            lx, t = x % TILE, y * W + x
            n = seg[y - 1, x]
            w = lx > 0 and seg[y, x - 1] == L
            nw = seg[y - 1, x - 1] if lx > 0 else -1
            ne = seg[y - 1, x + 1] if (lx < TILE - 1 and x + 1 < W) else -1
            if n == L:
                if not (w and nw == L):
                    _unite(par, t, t - W)
            else:
                if not w and nw == L:
                    _unite(par, t, t - W - 1)
                if ne == L:
                    _unite(par, t, t - W + 1)
    # kb_cc_hook: the 8-connected rule for pairs in different tiles
    for y in range(H):
        for x in range(W):
            L = seg[y, x]
            if L < 0:
                continue
            t = y * W + x

            def other(x2, y2):
                return x2 // TILE != x // TILE or y2 // TILE != y // TILE

            w = x > 0 and seg[y, x - 1] == L
            if w and other(x - 1, y):
                _unite(par, t, t - 1)
            if y > 0:
                if seg[y - 1, x] == L:
                    if other(x, y - 1):
                        _unite(par, t, t - W)
                else:
                    if not w and x > 0 and seg[y - 1, x - 1] == L and other(x - 1, y - 1):
                        _unite(par, t, t - W - 1)
                    if x < W - 1 and seg[y - 1, x + 1] == L and other(x + 1, y - 1):
                        _unite(par, t, t - W + 1)
    return np.array([_find(par, t) if par[t] >= 0 else -1 for t in range(H * W)]).reshape(H, W)


def _component_min_index(seg):
    H, W = seg.shape
    out = -np.ones((H, W), int)
    idx = np.arange(H * W).reshape(H, W)
    for L in np.unique(seg[seg >= 0]):
        lab, nc = ndimage.label(seg == L, structure=np.ones((3, 3)))
        for c in range(1, nc + 1):
            m = lab == c
            out[m] = idx[m].min()
    return out


@pytest.mark.parametrize("seed", range(12))
def test_tile_and_edge_unions_give_8_connected_components(seed):
    rng = np.random.default_rng(seed)
    H, W = int(rng.integers(20, 90)), int(rng.integers(20, 100))
    k = int(rng.integers(2, 6))
    base = rng.integers(-1, k, size=(H // 4 + 1, W // 4 + 1))
    seg = np.kron(base, np.ones((4, 4), int))[:H, :W]
    noise = rng.random((H, W)) < 0.15
    seg[noise] = rng.integers(-1, k, size=int(noise.sum()))
    np.testing.assert_array_equal(_kernel_roots(seg), _component_min_index(seg))
