"""Index maps of the engine's kernels, restated in Python and checked to cover every pixel
exactly once (st_spix_gb300/csrc/engine.h FOR_PIX / FOR_PIX_ALL / warp_block,
capi.cu pix_units / tiles64, k_prop.cu kb_cc_hook's tile-edge enumeration), for frame
sizes that leave partial blocks and tiles."""
import numpy as np
import pytest

THREADS = 256          # kThreads
PIX_PER_THREAD = 4     # kPixPerThread
CC_TILE = 32           # kCcTile


def _pix_units(n):
    return (n + PIX_PER_THREAD - 1) // PIX_PER_THREAD


def _blocks_for(n):
    return max(1, (n + THREADS - 1) // THREADS)


@pytest.mark.parametrize("n", [1, 255, 256, 1023, 1024, 1025, 409920, 480 * 853 + 7])
def test_for_pix_covers_each_pixel_once(n):
    hits = np.zeros(n, np.int64)
    uniform_iters = set()
    for b in range(_blocks_for(_pix_units(n))):
        base = b * PIX_PER_THREAD * THREADS
        t = base + np.arange(THREADS)
        for j in range(PIX_PER_THREAD):
            # FOR_PIX_ALL: the block-uniform condition (the block's first pixel of iteration j)
            if base + j * THREADS >= n:
                break
            uniform_iters.add((b, j))
            tj = t + j * THREADS
            m = tj < n                  # FOR_PIX's per-thread condition
            np.add.at(hits, tj[m], 1)
    assert (hits == 1).all()


@pytest.mark.parametrize("H,W", [(480, 854), (33, 65), (1, 1), (720, 1280), (31, 97)])
def test_warp_blocks_cover_each_pixel_once(H, W):
    tiles_x = (W + 63) // 64
    ntiles = tiles_x * ((H + 31) // 32)
    hits = np.zeros((H, W), np.int64)
    for blk in range(ntiles):
        for warp in range(8):
            gx0 = (blk % tiles_x) * 64 + (warp & 1) * 32
            by = (blk // tiles_x) * 32 + (warp >> 1) * 8
            for lane in range(32):
                gx = gx0 + lane
                for i in range(8):
                    gy = by + i
                    if gx < W and gy < H:
                        hits[gy, gx] += 1
    assert (hits == 1).all()


@pytest.mark.parametrize("H,W", [(480, 854), (40, 70), (32, 32), (5, 100)])
def test_cc_edge_enumeration(H, W):
    tiles_x = (W + CC_TILE - 1) // CC_TILE
    ntiles = tiles_x * ((H + CC_TILE - 1) // CC_TILE)
    edge = CC_TILE + 2 * (CC_TILE - 1)
    hits = np.zeros((H, W), np.int64)
    for u in range(ntiles * edge):
        tile, e = divmod(u, edge)
        lx = e if e < CC_TILE else (0 if e < 2 * CC_TILE - 1 else CC_TILE - 1)
        ly = 0 if e < CC_TILE else (e - CC_TILE + 1 if e < 2 * CC_TILE - 1 else e - 2 * CC_TILE + 2)
        x, y = (tile % tiles_x) * CC_TILE + lx, (tile // tiles_x) * CC_TILE + ly
        if x < W and y < H:
            hits[y, x] += 1
    ys, xs = np.mgrid[0:H, 0:W]
    lx, ly = xs % CC_TILE, ys % CC_TILE
    on_edge = (lx == 0) | (ly == 0) | (lx == CC_TILE - 1)
    assert (hits[on_edge] == 1).all() and (hits[~on_edge] == 0).all()
    # every pair of 8-neighbours in different tiles has a pixel on a tile edge whose earlier
    # neighbour (W, NW, N, NE) it is: the pixel the cross-tile pass runs for
    for y in range(H):
        for x in range(W):
            for dx, dy in ((-1, 0), (-1, -1), (0, -1), (1, -1)):
                xn, yn = x + dx, y + dy
                if 0 <= xn < W and 0 <= yn < H and (x // CC_TILE != xn // CC_TILE or
                                                    y // CC_TILE != yn // CC_TILE):
                    assert on_edge[y, x]
