"""Superpixel quality metrics on the GPU, under the names of the reference's
evaluation module (gauenk/st_spix st_spix/spix_utils/evaluate.py and
st_spix/sp_pooling.py).

Every score is computed by the engine's CUDA kernels (C ABI: stspix_evaluate,
stspix_count_spix, stspix_size_variation, stspix_sp_pooling); the integer tables
(per-frame id sizes, id x ground-truth overlaps) are exact and the colour sums FP64.
Inputs may be CUDA tensors or numpy arrays (copied to the current CUDA device):
video f32 [T,H,W,3], labels and ground truth integer [T,H,W].

computeSummary(vid, seg, spix) returns the reference's keys (tex, szv, ev, ev3d,
pooling, ue2d, sa2d, ue3d, sa3d, spnum, ave_nsp); the strred scores need
scikit-video's STRRED and are reported as -1, the reference's value when that
step is off.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .bist_cuda import _ctx, _stream


class Summary(dict):
    """A dict with attribute access (the reference returns an EasyDict)."""
    __getattr__ = dict.__getitem__
    __setattr__ = dict.__setitem__


def _device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("st_spix_gb300.metrics needs a CUDA device")
    return torch.device("cuda", torch.cuda.current_device())


def _as_cuda(x, dtype, name, device=None) -> torch.Tensor:
    if isinstance(x, np.ndarray):
        x = torch.from_numpy(np.ascontiguousarray(x))
    if not isinstance(x, torch.Tensor):
        raise TypeError(f"{name} must be a torch tensor or a numpy array")
    dev = device if device is not None else (x.device if x.is_cuda else _device())
    return x.to(device=dev, dtype=dtype).contiguous()


def _video(vid, spix, gt=None):
    sp = _as_cuda(spix, torch.int32, "spix")
    v = _as_cuda(vid, torch.float32, "vid", sp.device)
    if sp.dim() != 3 or v.dim() != 4 or v.shape[:3] != sp.shape or v.shape[3] != 3:
        raise RuntimeError("expected vid [T,H,W,3] and spix [T,H,W]")
    g = None
    if gt is not None:
        g = _as_cuda(gt, torch.int32, "gt", sp.device)
        if g.shape != sp.shape:
            raise RuntimeError("ground truth must match spix in shape")
    return v, sp, g


def evaluate(vid, spix, gt=None) -> Summary:
    """All scores of one labelled video in one pass (stspix_evaluate)."""
    v, sp, g = _video(vid, spix, gt)
    T, H, W = sp.shape
    ctx = _ctx(sp.device)
    q = _lib.QualityC()
    ctx.check(ctx.lib.stspix_evaluate(ctx.handle, _stream(sp.device), v.data_ptr(),
                                      sp.data_ptr(), g.data_ptr() if g is not None else None,
                                      T, H, W, C.byref(q)))
    return Summary(tex=q.tex, szv=q.szv, ev=q.ev, ev3d=q.ev3d, pooling=q.psnr,
                   ue2d=q.ue2d, sa2d=q.sa2d, ue3d=q.ue3d, sa3d=q.sa3d, spnum=q.spnum,
                   ave_nsp=q.ave_nsp, strred0=-1.0, strred1=-1.0)


def computeSummary(vid, seg, spix) -> Summary:
    """evaluate.py:94 computeSummary(vid, seg, spix); seg may be None (no UE / SA)."""
    return evaluate(vid, spix, seg)


def count_spix(spix) -> torch.Tensor:
    """evaluate.py:71 count_spix: int32 [T, max+1] per-frame id sizes (negative ids
    raise, where the reference exits)."""
    sp = _as_cuda(spix, torch.int32, "spix")
    T = sp.shape[0]
    npix = sp[0].numel()
    ctx = _ctx(sp.device)
    rng = (C.c_int32 * 2)()
    ctx.check(ctx.lib.stspix_label_range(ctx.handle, _stream(sp.device), sp.data_ptr(),
                                         sp.numel(), rng))
    if rng[0] < 0:
        raise RuntimeError("invalid spix: negative id")
    S = rng[1] + 1
    out = torch.empty((T, S), dtype=torch.int32, device=sp.device)
    ctx.check(ctx.lib.stspix_count_spix(ctx.handle, _stream(sp.device), sp.data_ptr(), T, npix,
                                        0, S, out.data_ptr()))
    return out


def _size_scores(counts):
    c = _as_cuda(counts, torch.int32, "counts")
    T, S = c.shape
    ctx = _ctx(c.device)
    tex, szv, nsp = C.c_double(), C.c_double(), C.c_double()
    ctx.check(ctx.lib.stspix_size_variation(ctx.handle, _stream(c.device), c.data_ptr(), T, S,
                                            C.byref(tex), C.byref(szv), C.byref(nsp)))
    return tex.value, szv.value, nsp.value


def scoreMeanDurationAndSizeVariation(counts):
    """evaluate.py:284: (TEX, SZV) of a per-frame id size table [T, S]."""
    tex, szv, _ = _size_scores(counts)
    return tex, szv


def averge_unique_spix_v1(sizes) -> float:
    """evaluate.py:184: mean number of ids alive per frame."""
    return _size_scores(sizes)[2]


def scoreExplainedVariance(vid, spix) -> float:
    """evaluate.py:230 (per-frame pooled colours)."""
    return evaluate(vid, spix).ev


def scoreExplainedVariance3D(vid, spix) -> float:
    """evaluate.py:254 (ids pooled over the whole video, each pixel against its
    frame's mean colour)."""
    return evaluate(vid, spix).ev3d


def sp_pooling(vid, spix, nspix=None):
    """st_spix/sp_pooling.py:10 for 3-channel frames: (pooled f32 [T,H,W,3],
    down f32 [T,nspix,3]), down = per-frame id sum / (count + 1e-8)."""
    v, sp, _ = _video(vid, spix)
    T, H, W = sp.shape
    ctx = _ctx(sp.device)
    if nspix is None:
        rng = (C.c_int32 * 2)()
        ctx.check(ctx.lib.stspix_label_range(ctx.handle, _stream(sp.device), sp.data_ptr(),
                                             sp.numel(), rng))
        nspix = rng[1] + 1
    pooled = torch.empty((T, H, W, 3), dtype=torch.float32, device=sp.device)
    down = torch.empty((T, int(nspix), 3), dtype=torch.float32, device=sp.device)
    ctx.check(ctx.lib.stspix_sp_pooling(ctx.handle, _stream(sp.device), v.data_ptr(),
                                        sp.data_ptr(), T, H, W, int(nspix), pooled.data_ptr(),
                                        down.data_ptr()))
    return pooled, down


def scoreSpixPoolingQuality(vid, spix):
    """evaluate.py:214: (mean per-frame PSNR of the pooled video, data range 1; the
    pooled video f32 [T,3,H,W] as the reference returns it)."""
    psnr = evaluate(vid, spix).pooling
    pooled, _ = sp_pooling(vid, spix)
    return psnr, pooled.permute(0, 3, 1, 2).contiguous()


def scoreUEandSA(spix, counts, gtSeg, gtSize, gtList, gtPos):
    """evaluate.py:372: (UE2d, SA2d, UE3d, SA3d).  counts, gtSize and gtList are
    recomputed on the device from spix and gtSeg (they are count_spix(spix),
    count_spix(gtSeg)[:, 1:] and the unique ground-truth ids, which must be 0..max);
    gtPos selects the annotated frames of spix."""
    sp = _as_cuda(spix, torch.int32, "spix")
    pos = torch.as_tensor(np.asarray(gtPos), dtype=torch.long, device=sp.device)
    sp = sp.index_select(0, pos).contiguous()
    ids = np.asarray(gtList)
    gt = _as_cuda(gtSeg, torch.int32, "gtSeg", sp.device)
    if gt.shape != sp.shape:
        return -1., -1., -1., -1.   # the reference's dimension-mismatch result
    if len(ids) and not np.array_equal(np.sort(ids), np.arange(len(ids))):
        raise RuntimeError("ground-truth ids must be 0..max")
    T, H, W = sp.shape
    # the video only feeds the colour scores, which are not returned here
    dummy = torch.zeros((T, H, W, 3), dtype=torch.float32, device=sp.device)
    s = evaluate(dummy, sp, gt)
    return s.ue2d, s.sa2d, s.ue3d, s.sa3d
