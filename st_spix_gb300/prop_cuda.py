"""The legacy `prop_cuda` extension surface (gauenk/st_spix st_spix/csrc/pybind_prop.cpp),
as called by st_spix/prop and st_spix/models/bass.py, on this engine.

Same names, argument order, shapes and dtypes as the legacy bindings (batch size 1 where
the legacy functions assert it).  Two kinds of entries:

  * exact restatements of the legacy kernels (C ABI stspix_legacy_* and the pooling
    entries): shift_labels, fill_missing, find_border, init_spix, rgb_to_lab,
    lab_to_rgb, sp_video_pooling, downsampled_video_to_pooled;
  * the BASS drivers bass, prop_bass, refine, refine_missing and split, which run this
    engine's BASS (run_bass) and propagated BASS (run_prop) -- the algorithm of the
    newer bist extension -- with the legacy arguments mapped onto its configuration.
    refine is propagated BASS with split/merge disabled; split is one split step of
    the propagated model (stspix_legacy_split; the legacy kernel's development-only
    acceptance score is not restated); refine_missing lets every pixel move (the
    legacy version moves only the missing ones).  refine and refine_missing return a
    zero log.

SuperpixelParams carries the legacy 17 tensors.  The engine's appearance model has a
fixed isotropic variance, so sigma_app / prior_sigma_app hold sigma2_app and
logdet_sigma_app 3 log(sigma2_app); the appearance / shape prior counts hold the
prior counts.  A SuperpixelParams made by bass / prop_bass keeps the engine's full
parameter set for the next prop_bass call.
"""
from __future__ import annotations

import ctypes as C
import math

import torch

from . import _lib, bist_cuda
from .bist_cuda import _check_input, _ctx, _stream

KEYS = ["mu_app", "sigma_app", "logdet_sigma_app", "prior_mu_app", "prior_sigma_app",
        "prior_mu_app_count", "prior_sigma_app_count", "mu_shape", "sigma_shape",
        "logdet_sigma_shape", "prior_mu_shape", "prior_sigma_shape", "prior_mu_shape_count",
        "prior_sigma_shape_count", "counts", "prior_counts", "ids"]


class SuperpixelParams:
    """pybind_prop.cpp:54-83: the 17 per-superpixel tensors (KEYS order)."""

    def __init__(self, *tensors):
        if tensors and len(tensors) != len(KEYS):
            raise TypeError(f"SuperpixelParams takes 0 or {len(KEYS)} tensors")
        for k, t in zip(KEYS, tensors or [None] * len(KEYS)):
            setattr(self, k, t)
        self._engine = None        # the engine's parameters, when made by this module

    def __repr__(self):
        return "Superpixel Parameters"


def _legacy_params(p: bist_cuda.SuperpixelParams, sigma2_app: float) -> SuperpixelParams:
    n = p.n
    dev = p._mu_app.device
    f = p.field
    pc = f("prior_counts").clone()
    out = SuperpixelParams(
        f("mu_app").clone(),
        torch.full((n, 3), float(sigma2_app), dtype=torch.float32, device=dev),
        torch.full((n,), 3.0 * math.log(sigma2_app), dtype=torch.float32, device=dev),
        f("prior_mu_app").clone(),
        torch.full((n, 3), float(sigma2_app), dtype=torch.float32, device=dev),
        pc.to(torch.int32), pc.to(torch.int32),
        f("mu_shape").clone(), f("sigma_shape").clone(), f("logdet_sigma_shape").clone(),
        f("prior_mu_shape").clone(), f("prior_sigma_shape").clone(),
        pc.to(torch.int32), pc.to(torch.int32),
        f("counts").clone(), pc, f("ids").clone())
    out._engine = p
    return out


def _engine_params(params: SuperpixelParams) -> bist_cuda.SuperpixelParams:
    """The engine's parameters of a legacy object: kept ones, else built from the legacy
    tensors (the sample shape covariance, which the legacy object lacks, as the inverse
    of sigma_shape)."""
    if params._engine is not None:
        return params._engine
    n = int(params.mu_app.shape[0])
    dev = params.mu_app.device
    p = bist_cuda.SuperpixelParams(n, dev)
    p.n = n

    def put(name, t):
        getattr(p, "_" + name).copy_(t.reshape(-1).to(getattr(p, "_" + name).dtype))

    put("mu_app", params.mu_app)
    put("prior_mu_app", params.prior_mu_app)
    put("mu_shape", params.mu_shape)
    put("sigma_shape", params.sigma_shape)
    put("logdet_sigma_shape", params.logdet_sigma_shape)
    put("prior_mu_shape", params.prior_mu_shape)
    put("prior_sigma_shape", params.prior_sigma_shape)
    put("counts", params.counts)
    put("prior_counts", params.prior_counts)
    put("ids", params.ids)
    s = params.sigma_shape.to(torch.float64)
    det = s[:, 0] * s[:, 2] - s[:, 1] * s[:, 1]
    det = torch.where(det > 0, det, torch.ones_like(det))
    inv = torch.stack([s[:, 2] / det, -s[:, 1] / det, s[:, 0] / det], 1)
    put("sample_sigma_shape", inv)
    return p


def _frame(img: torch.Tensor, name="img") -> torch.Tensor:
    _check_input(img, name)
    if img.dim() != 4 or img.shape[0] != 1:
        raise RuntimeError(f"{name} must be [1,H,W,C] (batch size 1)")
    return img[0]


def bass(img, niters, niters_seg, sm_start, sp_size, sigma2_app, sigma2_size, potts,
         alpha_hastings):
    """prop/bass.cu:179 run_bass: img f32 [1,H,W,3] -> (spix i32 [1,H,W], params)."""
    frame = _frame(img)
    lab, p = bist_cuda.run_bass(frame, niters=int(niters), niters_seg=int(niters_seg),
                                sm_start=int(sm_start), sp_size=int(sp_size),
                                sigma2_app=float(sigma2_app), potts=float(potts),
                                alpha=float(alpha_hastings), sigma2_size=float(sigma2_size))
    return lab[None], _legacy_params(p, float(sigma2_app))


def prop_bass(img, spix, params, niters, niters_seg, sm_start, sp_size, sigma2_app,
              sigma2_size, potts, alpha_hastings):
    """prop/prop_bass.cu:269 run_prop_bass: propagated BASS from the filled labels spix
    [1,H,W] and the previous frame's params -> (spix [1,H,W], params)."""
    frame = _frame(img)
    _check_input(spix, "spix")
    if spix.dim() != 3 or spix.shape[0] != 1:
        raise RuntimeError("spix must be [1,H,W] (batch size 1)")
    lab0 = spix[0].contiguous()
    pe = _engine_params(params)
    lab, p = bist_cuda.run_prop(frame, int(niters), lab0, lab0, pe,
                                niters_seg=int(niters_seg), sm_start=int(sm_start),
                                sp_size=int(sp_size), sigma2_app=float(sigma2_app),
                                potts=float(potts), alpha=float(alpha_hastings),
                                sigma2_size=float(sigma2_size))
    return lab[None], _legacy_params(p, float(sigma2_app))


def refine_missing(img, spix, missing, prior_params, nspix, niters, niters_seg, sp_size,
                   sigma2_app, potts):
    """prop/refine_missing.cu:101 run_refine_missing -> (spix, params, log f64
    [niters,1]); runs propagated BASS on the whole frame (see the module docstring)."""
    out, p = prop_bass(img, spix, prior_params, niters, niters_seg, 0, sp_size, sigma2_app,
                       0.0, potts, math.log(0.5))
    log = torch.zeros((int(niters), 1), dtype=torch.float64, device=img.device)
    return out, p, log


def refine(img, spix, params, niters, niters_seg, sp_size, sigma2_app, potts):
    """prop/refine.cu:99 run_refine: niters rounds of update_params + update_seg on the
    labels spix [1,H,W] from params, no split or merge -> (spix, params, log f64
    [niters,1]); propagated BASS with split/merge disabled."""
    out, p = prop_bass(img, spix, params, niters, niters_seg, int(niters), sp_size, sigma2_app,
                       0.0, potts, math.log(0.5))
    log = torch.zeros((int(niters), 1), dtype=torch.float64, device=img.device)
    return out, p, log


def split(img, spix, params, direction, sp_size, sigma2_app, sigma2_size, alpha_hastings):
    """prop/bass.cu:389 run_split_py: one split step of the propagated model on the
    labels spix [1,H,W] with params, in direction 2 (direction == 0) or 1 -> (spix,
    params)."""
    frame = _frame(img)
    _check_input(spix, "spix")
    if spix.dim() != 3 or spix.shape[0] != 1:
        raise RuntimeError("spix must be [1,H,W] (batch size 1)")
    H, W = frame.shape[:2]
    pe = _engine_params(params)
    cfg = bist_cuda.make_config(sp_size=int(sp_size), sigma2_app=float(sigma2_app),
                                sigma2_size=float(sigma2_size), alpha=float(alpha_hastings))
    out = bist_cuda.SuperpixelParams(10 * pe.n, img.device)
    lab = torch.zeros((1, H, W), dtype=torch.int32, device=img.device)
    pprev, ps, n = pe.struct(), out.struct(), C.c_int(0)
    ctx = _ctx(img.device)
    ctx.check(ctx.lib.stspix_legacy_split(ctx.handle, _stream(img.device), frame.data_ptr(), H, W,
                                          C.byref(cfg), int(direction), spix[0].contiguous().data_ptr(),
                                          C.byref(pprev), pe.n, lab.data_ptr(), C.byref(ps),
                                          C.byref(n)))
    out.n = n.value
    return lab, _legacy_params(out, float(sigma2_app))


def init_spix(img, sp_size):
    """prop/bass.cu:357 run_init_spix: the hexagonal initial labels -> (spix [1,H,W],)."""
    frame = _frame(img)
    H, W = frame.shape[:2]
    lab = torch.empty((1, H, W), dtype=torch.int32, device=img.device)
    n = C.c_int(0)
    ctx = _ctx(img.device)
    ctx.check(ctx.lib.stspix_init_seg(ctx.handle, _stream(img.device), lab.data_ptr(), H, W,
                                      int(sp_size), C.byref(n)))
    return (lab,)


def find_border(spix):
    """prop/seg_utils.cu:137 run_find_border: bool [1,H,W] (4-neighbour differs or image
    edge)."""
    _check_input(spix, "spix")
    B, H, W = spix.shape
    border = torch.empty((B, H, W), dtype=torch.bool, device=spix.device)
    ctx = _ctx(spix.device)
    for b in range(B):
        ctx.check(ctx.lib.stspix_find_border(ctx.handle, _stream(spix.device), spix[b].data_ptr(),
                                             border[b].data_ptr(), H, W, 0))
    return border


def shift_labels(spix, flow):
    """prop/shift_labels.cu:82: spix i32 [1,H,W], flow i32 [1,nspix,2] (dx, dy per
    superpixel) -> (shifted i32 [1,H,W], counts i32 [1,H,W])."""
    _check_input(spix, "spix")
    _check_input(flow, "flow")
    if spix.dtype != torch.int32 or flow.dtype != torch.int32:
        raise RuntimeError("spix and flow must be int32")
    _, H, W = spix.shape
    shifted = torch.empty_like(spix)
    counts = torch.empty_like(spix)
    ctx = _ctx(spix.device)
    ctx.check(ctx.lib.stspix_legacy_shift_labels(ctx.handle, _stream(spix.device),
                                                 spix.data_ptr(), flow.data_ptr(),
                                                 int(flow.shape[1]), H, W, shifted.data_ptr(),
                                                 counts.data_ptr()))
    return shifted, counts


def fill_missing(spix, centers, missing, break_iter):
    """prop/fill_missing.cu:317: spix i32 [1,H,W], centers f32 [nspix,2] (x, y),
    missing i32 [1,M] (pixel indices) -> filled spix (a copy)."""
    _check_input(spix, "spix")
    _check_input(centers, "centers")
    _check_input(missing, "missing")
    _, H, W = spix.shape
    out = spix.clone()
    it, rem = C.c_int(0), C.c_int(0)
    ctx = _ctx(spix.device)
    ctx.check(ctx.lib.stspix_legacy_fill_missing(ctx.handle, _stream(spix.device),
                                                 out.data_ptr(), centers.float().contiguous().data_ptr(),
                                                 int(centers.shape[0]), missing.data_ptr(),
                                                 int(missing.numel()), H, W, int(break_iter),
                                                 C.byref(it), C.byref(rem)))
    return out


def rgb_to_lab(img):
    """prop/rgb2lab.cu:167 (channels read in RGB order)."""
    _check_input(img, "img")
    out = img.clone()
    ctx = _ctx(img.device)
    ctx.check(ctx.lib.stspix_legacy_rgb_to_lab(ctx.handle, _stream(img.device), img.data_ptr(),
                                               out.data_ptr(), img.numel() // 3))
    return out


def lab_to_rgb(img):
    """prop/rgb2lab.cu:186 (the same conversion as bist's lab2rgb)."""
    return bist_cuda.lab2rgb(img)


def sp_video_pooling(img, seg):
    """prop/sp_video_pooling.cu:62: img f32 [B,T,H,W,F], seg i32 [B,T,H,W] ->
    (pooled [B,T,H,W,F], downsampled [B,nspix,F], counts f32 [B,nspix]) with
    nspix = max id + 1."""
    _check_input(img, "img")
    _check_input(seg, "seg")
    B, T, H, W, F = img.shape
    nspix = int(seg.max().item()) + 1
    pooled = torch.empty_like(img)
    down = torch.empty((B, nspix, F), dtype=torch.float32, device=img.device)
    counts = torch.empty((B, nspix), dtype=torch.float32, device=img.device)
    ctx = _ctx(img.device)
    ctx.check(ctx.lib.stspix_sp_video_pooling(ctx.handle, _stream(img.device), img.data_ptr(),
                                              seg.data_ptr(), B, T, H, W, F, nspix,
                                              pooled.data_ptr(), down.data_ptr(),
                                              counts.data_ptr()))
    return pooled, down, counts


def downsampled_video_to_pooled(downsampled, seg):
    """prop/sp_video_pooling.cu:211: downsampled f32 [B,nspix,F], seg i32 [B,T,H,W] ->
    pooled f32 [B,T,H,W,F]."""
    _check_input(downsampled, "downsampled")
    _check_input(seg, "seg")
    B, T, H, W = seg.shape
    nspix, F = int(downsampled.shape[1]), int(downsampled.shape[2])
    if int(seg.max().item()) + 1 > nspix:
        raise RuntimeError("seg holds ids beyond downsampled")
    pooled = torch.empty((B, T, H, W, F), dtype=torch.float32, device=seg.device)
    ctx = _ctx(seg.device)
    ctx.check(ctx.lib.stspix_downsampled_video_to_pooled(ctx.handle, _stream(seg.device),
                                                         downsampled.data_ptr(), seg.data_ptr(),
                                                         B, T, H, W, F, nspix,
                                                         pooled.data_ptr()))
    return pooled


def run_update_prior(spix, params, prev_nspix, invert):
    """prop/sparams_io.cu:795 run_update_prior: for every id present in spix at or
    above prev_nspix, params' priors (prior_mu_app, prior_mu_shape, prior_sigma_shape)
    take the estimates (mu_app, mu_shape, sigma_shape; its inverse when invert), in
    place."""
    _check_input(spix, "spix")
    for k in ("mu_app", "prior_mu_app", "mu_shape", "prior_mu_shape", "sigma_shape",
              "prior_sigma_shape"):
        _check_input(getattr(params, k), k)
    nids = int(params.mu_app.shape[0])
    if spix.numel() and int(spix.max().item()) >= nids:
        raise RuntimeError("spix holds ids beyond the parameter rows")
    if params.mu_app.dtype != torch.float32 or params.prior_mu_app.dtype != torch.float32 or \
            params.mu_shape.dtype != torch.float64 or params.sigma_shape.dtype != torch.float64:
        raise RuntimeError("mu_app / prior_mu_app must be float32, shape fields float64")
    ctx = _ctx(spix.device)
    ctx.check(ctx.lib.stspix_legacy_update_prior(
        ctx.handle, _stream(spix.device), spix.data_ptr(), spix.numel(), nids,
        params.mu_app.data_ptr(), params.prior_mu_app.data_ptr(), params.mu_shape.data_ptr(),
        params.prior_mu_shape.data_ptr(), params.sigma_shape.data_ptr(),
        params.prior_sigma_shape.data_ptr(), int(prev_nspix), int(bool(invert))))
    params._engine = None      # the legacy tensors changed: rebuild on the next prop_bass


def _shift_tensor(in_tensor, spix, flow, selected):
    _check_input(in_tensor, "in_tensor")
    _check_input(spix, "spix")
    _check_input(flow, "flow")
    if spix.dtype != torch.int32 or flow.dtype != torch.int32 or in_tensor.dtype != torch.float32:
        raise RuntimeError("spix and flow must be int32, in_tensor float32")
    B, H, W = spix.shape
    F = int(in_tensor.shape[3])
    nspix = int(spix.max().item()) + 1
    if int(flow.shape[1]) != nspix:
        raise RuntimeError("flow must have one row per superpixel (spix.max() + 1)")
    out = torch.empty((B, H, W, F), dtype=torch.float32, device=spix.device)
    counts = torch.empty((B, H, W), dtype=torch.int32, device=spix.device)
    contrib = None
    if selected is None:
        contrib = torch.empty((B, H, W, nspix), dtype=torch.bool, device=spix.device)
    ctx = _ctx(spix.device)
    ctx.check(ctx.lib.stspix_legacy_shift_tensor(
        ctx.handle, _stream(spix.device), in_tensor.data_ptr(), spix.data_ptr(), flow.data_ptr(),
        B, H, W, F, nspix, selected.data_ptr() if selected is not None else None, out.data_ptr(),
        counts.data_ptr(), contrib.data_ptr() if contrib is not None else None))
    return out, counts, contrib


def shift_tensor(in_tensor, spix, flow):
    """prop/shift_tensor.cu:60 run_shift_tensor: in f32 [B,H,W,F], spix i32 [B,H,W], flow
    i32 [B,nspix,2] -> (shifted features f32 [B,H,W,F] (sums of the arrivals), counts
    i32 [B,H,W], contributors bool [B,H,W,nspix])."""
    return _shift_tensor(in_tensor, spix, flow, None)


def shift_tensor_ordered(in_tensor, spix, flow, select):
    """prop/shift_tensor_ordered.cu:53: as shift_tensor, but a pixel takes only the
    arrivals of its selected id (select i32 [B,H,W]) -> (shifted features, counts)."""
    _check_input(select, "select")
    out, counts, _ = _shift_tensor(in_tensor, spix, flow, select.to(torch.int32).contiguous())
    return out, counts


def shift_order(contributors, sizes):
    """prop/shift_order.cu:43 run_shift_order: contributors bool [B,H,W,nspix], sizes i32
    [B,nspix] -> selected i32 [B,H,W]: the first contributing id (-1 if none), which is
    what the legacy loop returns whatever the sizes."""
    _check_input(contributors, "contributors")
    _check_input(sizes, "sizes")
    B, H, W, nspix = contributors.shape
    sel = torch.empty((B, H, W), dtype=torch.int32, device=contributors.device)
    ctx = _ctx(contributors.device)
    ctx.check(ctx.lib.stspix_legacy_shift_order(ctx.handle, _stream(contributors.device),
                                                contributors.contiguous().data_ptr(), B, H, W,
                                                nspix, sel.data_ptr()))
    return sel


def split_disconnected(spix, nspix):
    """prop/split_disconnected.cu:390 split_disconnected: spix i32 [1,H,W] (relabelled in
    place) -> (spix, children i32 [nspix, max_nsplits], split_starts i32 [nspix])."""
    _check_input(spix, "spix")
    if spix.dtype != torch.int32 or spix.shape[0] != 1:
        raise RuntimeError("spix must be int32 [1,H,W]")
    _, H, W = spix.shape
    nspix = int(nspix)
    starts = torch.empty((nspix,), dtype=torch.int32, device=spix.device)
    ctx = _ctx(spix.device)
    mx = C.c_int(0)
    cap = nspix * 8
    children = torch.empty((cap,), dtype=torch.int32, device=spix.device)
    st = ctx.lib.stspix_legacy_split_disconnected(ctx.handle, _stream(spix.device),
                                                  spix.data_ptr(), H, W, nspix, starts.data_ptr(),
                                                  children.data_ptr(), cap, C.byref(mx))
    if st == _lib.STSPIX_ERR_CAPACITY:
        cap = nspix * mx.value
        children = torch.empty((max(cap, 1),), dtype=torch.int32, device=spix.device)
        st = ctx.lib.stspix_legacy_split_disconnected(ctx.handle, _stream(spix.device),
                                                      spix.data_ptr(), H, W, nspix,
                                                      starts.data_ptr(), children.data_ptr(),
                                                      cap, C.byref(mx))
    ctx.check(st)
    return spix, children[: nspix * mx.value].view(nspix, mx.value), starts
