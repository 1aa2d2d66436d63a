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


def update_prior(spix: np.ndarray, mu_app, prior_mu_app, mu_shape, prior_mu_shape, sigma_shape,
                 prior_sigma_shape, prev_nspix: int, invert: bool):
    """run_update_prior (prop/sparams_io.cu:795-834) with update_prior_kernel
    (:743-792): for each unique id >= prev_nspix, priors := estimates (the shape prior
    the covariance, inverted when `invert`, a negative determinant replaced by 1e-6).
    Returns updated copies of the three prior arrays."""
    pma, pms, pss = prior_mu_app.copy(), prior_mu_shape.copy(), prior_sigma_shape.copy()
    for k in np.unique(spix):
        if k < 0 or k < prev_nspix:
            continue
        pma[k] = mu_app[k]
        pms[k] = mu_shape[k]
        xx, xy, yy = (float(v) for v in sigma_shape[k])
        det = xx * yy - xy * xy
        if det < 0:
            det = 0.000001
        pss[k] = (yy / det, -xy / det, xx / det) if invert else (xx, xy, yy)
    return pma, pms, pss


def shift_tensor(in_tensor: np.ndarray, spix: np.ndarray, flow: np.ndarray, selected=None):
    """shift_tensor_kernel (prop/shift_tensor.cu:15-57) / shift_tensor_ordered_kernel
    (prop/shift_tensor_ordered.cu:14-50) for one batch item: in [H,W,F], spix [H,W],
    flow [nspix,2] (dx, dy).  Features summed in FP64, rounded to FP32.  Returns (out,
    counts, contributors [H,W,nspix])."""
    H, W, F = in_tensor.shape
    nspix = flow.shape[0]
    acc = np.zeros((H, W, F), np.float64)
    counts = np.zeros((H, W), np.int32)
    contrib = np.zeros((H, W, nspix), bool)
    for y in range(H):
        for x in range(W):
            s = int(spix[y, x])
            if s < 0 or s >= nspix:
                continue
            yd, xd = y + int(flow[s, 1]), x + int(flow[s, 0])
            if not (0 <= yd <= H - 1 and 0 <= xd <= W - 1):
                continue
            if selected is not None and int(selected[yd, xd]) != s:
                continue
            counts[yd, xd] += 1
            acc[yd, xd] += in_tensor[y, x].astype(np.float64)
            contrib[yd, xd, s] = True
    return acc.astype(np.float32), counts, contrib


def shift_order(contributors: np.ndarray, sizes: np.ndarray):
    """shift_order_kernel (prop/shift_order.cu:14-40), restated literally for one batch
    item: contributors [H,W,nspix], sizes [nspix] -> selected [H,W]."""
    H, W, nspix = contributors.shape
    sel = np.full((H, W), -1, np.int32)
    for y in range(H):
        for x in range(W):
            curr_val, argmin, min_val = -1, -1, 1000000
            for si in range(nspix):
                upd = (curr_val < min_val) if contributors[y, x, si] else False
                if not upd:
                    continue
                curr_val = int(sizes[si])
                argmin = si
                min_val = curr_val
            if argmin >= 0:
                sel[y, x] = argmin
    return sel


def split_disconnected(spix: np.ndarray, nspix: int):
    """split_disconnected (prop/split_disconnected.cu:31-255, 300-330): regions of equal
    labels connected through neighbours within Chebyshev distance 2 (find_spix_min
    iterated to its fixed point), numbered by their smallest pixel index; per label the
    regions are ranked in that order and the first largest swaps ranks with the first
    (compute_offsets); get_split_starts' prefix sums; update_spix relabels ranks > 0.
    Returns (relabelled spix, children [nspix, max_nsplits], split_starts [nspix])."""
    H, W = spix.shape
    seg = spix.astype(np.int64)
    npix = H * W
    parent = np.arange(npix)

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    flat = seg.reshape(-1)
    for t in range(npix):
        y, x = divmod(t, W)
        for dy in (-2, -1, 0):
            for dx in (-2, -1, 0, 1, 2):
                if dy == 0 and dx >= 0:
                    break
                yy, xx = y + dy, x + dx
                if yy < 0 or xx < 0 or xx >= W:
                    continue
                q = yy * W + xx
                if flat[q] != flat[t]:
                    continue
                a, b = find(t), find(q)
                if a != b:
                    parent[max(a, b)] = min(a, b)
    root = np.array([find(t) for t in range(npix)])
    ids = np.unique(root)
    rank = {int(r): i for i, r in enumerate(ids)}
    region_of = np.array([rank[int(r)] for r in root])
    nreg = len(ids)
    region_spix = flat[ids]
    region_size = np.bincount(region_of, minlength=nreg)
    counts = np.zeros(nspix, np.int64)
    for s in region_spix:
        counts[s] += 1
    c = np.maximum(counts - 1, 0)
    starts = np.zeros(nspix, np.int32)
    cum, first = 0, None
    for s in range(nspix):
        if c[s] <= 0:
            continue
        cum += int(c[s])
        if first is None:
            first = cum
        starts[s] = cum - first
    mx = cum
    offset = np.full(nreg, -1, np.int64)
    for s in range(nspix):
        child, cur_max, idx_max, idx_zero = 0, -1, -1, -1
        for r in range(nreg):
            if region_spix[r] != s:
                continue
            if child == 0:
                idx_zero = r
            offset[r] = child
            if region_size[r] > cur_max:
                idx_max, cur_max = r, region_size[r]
            child += 1
        if child > 0 and idx_max != idx_zero:
            offset[idx_zero] = offset[idx_max]
            offset[idx_max] = 0
    children = np.full((nspix, mx), -1, np.int32)
    out = flat.copy()
    for t in range(npix):
        off = offset[region_of[t]]
        if off > 0:
            s = flat[t]
            nid = nspix + starts[s] + off
            out[t] = nid
            children[s, off - 1] = nid
    return out.reshape(H, W).astype(np.int32), children, starts
