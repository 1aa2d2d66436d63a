"""CPU restatement of the reference's superpixel quality metrics
(gauenk/st_spix st_spix/spix_utils/evaluate.py) -- test infrastructure: the oracle
that the GPU metrics (st_spix_gb300.metrics) are checked against; nothing in the
package imports it.

Integer tables (per-frame id counts, id x ground-truth overlaps) are exact int64;
every other value is FP64.  Pinned against the reference's own functions by
tests/golden/quality_ref.npz (generated by tests/golden/make_quality_golden.py).

Deliberate choices where the reference leaves the arithmetic open:
  * variances of superpixel sizes are formed as (n*sum(c^2) - sum(c)^2) / (n(n-1))
    from exact integers (the reference divides int64 tensors, evaluate.py:296-299,
    which gives torch's default float type);
  * "at least half" tests (evaluate.py:459,465) are 2*in >= count on integers;
  * PSNR of the superpixel-pooled video uses the usual 10*log10(1/mse) per frame
    (data range 1), averaged over frames: the reference calls
    st_spix.metrics.compute_psnrs (evaluate.py:227), which is not in the repository;
  * the 3D explained variance pools each id over the whole video and compares
    every pixel with its frame's mean colour; the reference's version (evaluate.py:
    254-281) subtracts a [T,1,1,3] mean from a [T,3,H,W] pooled video, which only
    broadcasts when W == 3, so the evident intent is restated.
"""
from __future__ import annotations

import math

import numpy as np


def count_spix(spix: np.ndarray) -> np.ndarray:
    """Per-frame pixel count of every id 0..max (evaluate.py:71-92): int64 [T, max+1].
    Negative ids are an error (the reference prints and exits)."""
    T = spix.shape[0]
    s = spix.reshape(T, -1).astype(np.int64)
    if s.min() < 0:
        raise ValueError("invalid spix: negative id")
    S = int(s.max()) + 1
    return np.stack([np.bincount(s[t], minlength=S) for t in range(T)]).astype(np.int64)


def mean_duration_and_size_variation(counts: np.ndarray):
    """(TEX, SZV) of scoreMeanDurationAndSizeVariation (evaluate.py:284-327): TEX is
    the fraction of ids alive per frame, averaged over frames; SZV the mean over ids
    alive in more than one frame of the unbiased standard deviation of their size
    over the frames they are alive in (NaN if there is none)."""
    c = counts.astype(np.int64)
    T, S = c.shape
    alive = c > 0
    tex = float(np.mean(np.mean(alive, axis=1)))
    n = alive.sum(0).astype(np.int64)
    s1 = c.sum(0)
    s2 = (c * c).sum(0)
    keep = n > 1
    if not np.any(keep):
        return tex, float("nan")
    num = n[keep] * s2[keep] - s1[keep] * s1[keep]
    var = num.astype(np.float64) / (n[keep] * (n[keep] - 1)).astype(np.float64)
    return tex, float(np.mean(np.sqrt(var)))


def _frame_pool(vid64, spix, S):
    """Per-frame id means as sp_pooling computes them (sp_pooling.py:10-47):
    sum / (count + 1e-8).  Returns (means [T,S,3], counts [T,S])."""
    T = vid64.shape[0]
    means = np.zeros((T, S, 3))
    counts = np.zeros((T, S), np.int64)
    for t in range(T):
        s = spix[t].reshape(-1)
        v = vid64[t].reshape(-1, 3)
        cnt = np.bincount(s, minlength=S)
        for ch in range(3):
            means[t, :, ch] = np.bincount(s, weights=v[:, ch], minlength=S) / (cnt + 1e-8)
        counts[t] = cnt
    return means, counts


def explained_variance(vid: np.ndarray, spix: np.ndarray) -> float:
    """scoreExplainedVariance (evaluate.py:230-252): per frame, the squared distance of
    the superpixel-pooled frame from the frame's mean colour over that of the frame
    itself, averaged over frames."""
    v = vid.astype(np.float64)
    T = v.shape[0]
    S = int(spix.max()) + 1
    m = v.reshape(T, -1, 3).mean(1)                      # [T,3]
    pix2mean = ((v - m[:, None, None, :]) ** 2).reshape(T, -1).sum(1)
    means, _ = _frame_pool(v, spix, S)
    pooled = np.stack([means[t][spix[t]] for t in range(T)])
    pool2mean = ((pooled - m[:, None, None, :]) ** 2).reshape(T, -1).sum(1)
    return float(np.mean(pool2mean / (pix2mean + 1e-10)))


def explained_variance_3d(vid: np.ndarray, spix: np.ndarray) -> float:
    """scoreExplainedVariance3D (evaluate.py:254-281), intent restated: colours x255,
    each id pooled over the whole video (sp_video_pooling.cu: sum / (count + 1e-10)),
    each pixel compared with its frame's mean colour."""
    v = 255.0 * vid.astype(np.float64)
    T = v.shape[0]
    S = int(spix.max()) + 1
    m = v.reshape(T, -1, 3).mean(1)
    pix2mean = ((v - m[:, None, None, :]) ** 2).reshape(T, -1).sum(1)
    s = spix.reshape(-1)
    vv = v.reshape(-1, 3)
    cnt = np.bincount(s, minlength=S)
    mu = np.stack([np.bincount(s, weights=vv[:, ch], minlength=S) for ch in range(3)], 1)
    mu = mu / (cnt[:, None] + 1e-10)
    pooled = mu[spix]                                     # [T,H,W,3]
    pool2mean = ((pooled - m[:, None, None, :]) ** 2).reshape(T, -1).sum(1)
    return float(np.mean(pool2mean / (pix2mean + 1e-10)))


def pooling_psnr(vid: np.ndarray, spix: np.ndarray) -> float:
    """PSNR (data range 1) of the superpixel-pooled video against the video, per frame,
    averaged over frames (scoreSpixPoolingQuality, evaluate.py:214-227)."""
    v = vid.astype(np.float64)
    T = v.shape[0]
    S = int(spix.max()) + 1
    means, _ = _frame_pool(v, spix, S)
    out = []
    for t in range(T):
        mse = float(np.mean((v[t] - means[t][spix[t]]) ** 2))
        out.append(math.inf if mse == 0 else 10.0 * math.log10(1.0 / mse))
    return float(np.mean(out))


def ue_and_sa(spix: np.ndarray, gt: np.ndarray):
    """scoreUEandSA (evaluate.py:372-512) with counts = count_spix(spix), gtSize =
    count_spix(gt)[:, 1:], gtList = unique(gt), gtPos = all frames.  Ground-truth ids
    must be 0..max, each present somewhere (the reference aligns its columns on that
    and asserts every object has pixels).  Returns (UE2d, SA2d, UE3d, SA3d)."""
    T, H, W = spix.shape
    counts = count_spix(spix)
    S = counts.shape[1]
    G1 = int(gt.max()) + 1
    if gt.min() < 0:
        raise ValueError("negative ground-truth id")
    J = np.zeros((T, S, G1), np.int64)                    # overlap counts
    for t in range(T):
        key = spix[t].reshape(-1).astype(np.int64) * G1 + gt[t].reshape(-1)
        J[t] = np.bincount(key, minlength=S * G1).reshape(S, G1)
    gt_size = J.sum(1)                                    # [T,G1]
    if np.any(gt_size.sum(0) == 0):
        raise ValueError("ground-truth ids must be 0..max, each present")
    n = counts[:, :, None]
    inside = J > 0
    out = np.where(inside, n - J, 0)
    gt_ue = np.where(inside, np.minimum(out, J), 0).sum(1)          # [T,G1]
    gt_sa = np.where(2 * J >= n, J, 0).sum(1)                       # [T,G1]
    in_s = J.sum(0)                                                 # [S,G1]
    out_s = out.sum(0)
    gt_ue3 = np.where(in_s > 0, np.minimum(out_s, in_s), 0).sum(0)  # [G1]
    tot = counts.sum(0)[:, None]
    gt_sa3 = np.where(2 * in_s >= tot, in_s, 0).sum(0)
    ue2d = float(np.mean(gt_ue / (H * W)))
    size = gt_size[:, 1:]
    mask = size + (size == 0)
    sa2d = float(np.mean(np.sum(gt_sa[:, 1:] / mask, axis=0) / np.sum(size > 0, axis=0)))
    ue3d = float(np.mean(gt_ue3 / (T * H * W)))
    sa3d = float(np.mean(gt_sa3[1:] / size.sum(0)))
    return ue2d, sa2d, ue3d, sa3d


def compute_summary(vid: np.ndarray, spix: np.ndarray, gt=None) -> dict:
    """computeSummary (evaluate.py:94-176) without the strred score (skvideo):
    ids are offset by their minimum first."""
    spix = (spix - spix.min()).astype(np.int64)
    counts = count_spix(spix)
    tex, szv = mean_duration_and_size_variation(counts)
    out = dict(tex=tex, szv=szv, ev=explained_variance(vid, spix),
               ev3d=explained_variance_3d(vid, spix), pooling=pooling_psnr(vid, spix),
               spnum=int(spix.max()) + 1,
               ave_nsp=float(np.mean(np.sum(counts > 0, axis=1))),
               ue2d=-1.0, sa2d=-1.0, ue3d=-1.0, sa3d=-1.0, strred0=-1.0, strred1=-1.0)
    if gt is not None:
        out["ue2d"], out["sa2d"], out["ue3d"], out["sa3d"] = ue_and_sa(spix, gt)
    return out
