"""CPU restatement of the legacy prop_cuda kernels with self-contained arithmetic
(gauenk/st_spix st_spix/csrc/prop/) -- test infrastructure: the oracle that
st_spix_gb300.prop_cuda's exact entries are checked against.  Parity unpinned against
the legacy extension itself, which the reference does not build (its sources are
restated here line by line and cited)."""
from __future__ import annotations

import numpy as np


def shift_labels(spix: np.ndarray, flow: np.ndarray):
    """shift_labels_kernel (prop/shift_labels.cu:31-80): spix [H,W] i32, flow [nspix,2]
    (dx, dy) -> (shifted, counts): arrivals per pixel and the largest arriving label."""
    H, W = spix.shape
    nspix = flow.shape[0]
    shifted = np.full((H, W), -1, np.int32)
    counts = np.zeros((H, W), np.int32)
    ys, xs = np.nonzero((spix >= 0) & (spix < nspix))
    s = spix[ys, xs]
    yd = ys + flow[s, 1]
    xd = xs + flow[s, 0]
    ok = (yd >= 0) & (yd < H) & (xd >= 0) & (xd < W)
    np.add.at(counts, (yd[ok], xd[ok]), 1)
    np.maximum.at(shifted, (yd[ok], xd[ok]), s[ok])
    return shifted, counts


def fill_missing(spix: np.ndarray, centers: np.ndarray, missing: np.ndarray, break_iter: int):
    """fill_missing (prop/fill_missing.cu:26-90) with find_border_along_missing
    (:258-292) and update_missing_seg_nn (:142-256); FP32 distances as the kernel.
    Returns (filled, iterations, still missing)."""
    seg = spix.astype(np.int32).copy()
    H, W = seg.shape
    flat = seg.reshape(-1)
    c = centers.astype(np.float32)
    miss = missing.reshape(-1).astype(np.int64)
    nc = c.shape[0]

    def count_border():
        border = np.zeros(len(miss), bool)
        neg = 0
        for j, idx in enumerate(miss):
            x, y = idx % W, idx // W
            C = flat[idx]
            N = flat[idx - W] if y > 0 else -1
            Wl = flat[idx - 1] if x > 0 else -1
            S = flat[idx + W] if y < H - 1 else -1
            E = flat[idx + 1] if x < W - 1 else -1
            border[j] = (N >= 0 or Wl >= 0 or S >= 0 or E >= 0) and C < 0
            neg += int(C < 0)
        return border, neg

    neg, prev, it = 1, 1, 0
    while neg > 0:
        if break_iter > 0 and it >= break_iter:
            break
        border, neg = count_border()
        for xm in range(2):
            for ym in range(2):
                for j, idx in enumerate(miss):
                    if not border[j]:
                        continue
                    x, y = idx % W, idx // W
                    if x % 2 != xm or y % 2 != ym:
                        continue
                    Wl = flat[idx - 1] if x > 0 else -1
                    N = flat[idx - W] if y > 0 else -1
                    E = flat[idx + 1] if x < W - 1 else -1
                    S = flat[idx + W] if y < H - 1 else -1
                    best, lab = np.float32(-999999.0), -1

                    def consider(l, best, lab):
                        if l >= nc:
                            return best, lab
                        dx = (np.float32(x) - c[l, 0]) / np.float32(W)
                        dy = (np.float32(y) - c[l, 1]) / np.float32(H)
                        sim = np.float32(-dx * dx) - np.float32(dy * dy)
                        return (sim, l) if sim > best else (best, lab)

                    if N >= 0:
                        best, lab = consider(N, best, lab)
                    if S >= 0 and S != N:
                        best, lab = consider(S, best, lab)
                    if Wl >= 0 and Wl != S and Wl != N:
                        best, lab = consider(Wl, best, lab)
                    if E >= 0 and E != Wl and E != S and E != N:
                        best, lab = consider(E, best, lab)
                    flat[idx] = lab
        it += 1
        if neg == prev:
            break
        prev = neg
    _, neg = count_border()
    return seg, it, neg


def find_border(spix: np.ndarray) -> np.ndarray:
    """find_border_pixels (prop/seg_utils.cu:35-66): image edge, or a 4-neighbour
    differs."""
    H, W = spix.shape
    b = np.ones((H, W), bool)
    C = spix[1:-1, 1:-1]
    b[1:-1, 1:-1] = ((C != spix[:-2, 1:-1]) | (C != spix[2:, 1:-1]) |
                     (C != spix[1:-1, :-2]) | (C != spix[1:-1, 2:]))
    return b


def sp_video_pooling(img: np.ndarray, seg: np.ndarray, nspix: int):
    """sp_video_pooling (prop/sp_video_pooling.cu:62-120): img [B,T,H,W,F], seg
    [B,T,H,W] -> (pooled, down [B,nspix,F], counts [B,nspix]) with FP64 sums."""
    B, T, H, W, F = img.shape
    down = np.zeros((B, nspix, F), np.float32)
    counts = np.zeros((B, nspix), np.float32)
    pooled = np.zeros_like(img, dtype=np.float32)
    for b in range(B):
        s = seg[b].reshape(-1)
        v = img[b].reshape(-1, F).astype(np.float64)
        ok = s >= 0
        cnt = np.bincount(s[ok], minlength=nspix)
        counts[b] = cnt.astype(np.float32)
        for f in range(F):
            sm = np.bincount(s[ok], weights=v[ok, f], minlength=nspix)
            down[b, :, f] = sm.astype(np.float32) / (cnt.astype(np.float32) + np.float32(1e-10))
        pv = pooled[b].reshape(-1, F)
        pv[ok] = down[b][s[ok]]
    return pooled, down, counts
