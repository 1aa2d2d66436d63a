"""Drop-in replacement of the reference's `bist_cuda` torch extension
(gauenk/st_spix: st_spix/csrc/pybind_bist.cpp:16-18, st_spix/csrc/bist/pyapi.cu:46-310).

    import st_spix_gb300.bist_cuda as bist_cuda
    spix = bist_cuda.bist_forward(vid, flows, niters, sp_size, potts, sigma2_app,
                                  alpha, split_alpha, video_mode, rgb2lab)
    marked = bist_cuda.get_marked_video(vid, spix, color)

Same argument order, meaning, shapes and error behaviour (inputs must be CUDA and
contiguous, else RuntimeError).  Work runs on torch's current CUDA stream through
the C ABI of libstspix_gb300.so; torch only provides device memory and the stream.

The reference's C++ entry points on this path are exposed too: run_bass
(bass.cu:221), shift_and_fill (shift_and_fill.cu:108), run_prop (prop.cu:677), with
the cross-frame parameters as a SuperpixelParams of tensors (structs.h:13-48).
"""
from __future__ import annotations

import ctypes as C
import threading

import torch

from . import _lib

_ctx_lock = threading.Lock()
_contexts = {}


def _ctx(device: torch.device) -> _lib.Context:
    """The engine context (device workspace) of torch's current stream on `device`:
    one per CUDA stream, so concurrent streams never share a workspace."""
    idx = device.index if device.index is not None else torch.cuda.current_device()
    key = (idx, torch.cuda.current_stream(idx).cuda_stream)
    with _ctx_lock:
        c = _contexts.get(key)
        if c is None:
            c = _contexts[key] = _lib.Context(idx)
        return c


def _check_input(x: torch.Tensor, name: str):
    if not isinstance(x, torch.Tensor) or not x.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor")
    if not x.is_contiguous():
        raise RuntimeError(f"{name} must be contiguous")


def _stream(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def make_config(niters=15, sp_size=15, potts=0.5, sigma2_app=0.009 ** 2,
                alpha=-0.6931471805599453, split_alpha=0.0, **kw) -> _lib.Config:
    return _lib.default_config(niters=int(niters), sp_size=int(sp_size), potts=float(potts),
                               sigma2_app=float(sigma2_app), alpha_hastings=float(alpha),
                               split_alpha=float(split_alpha), **kw)


def bist_forward(vid: torch.Tensor, flows: torch.Tensor, niters: int, sp_size: int,
                 potts: float, sigma2_app: float, alpha: float, split_alpha: float,
                 video_mode: bool, rgb2lab: bool, **extra) -> torch.Tensor:
    """pyapi.cu:200 bist_forward_cuda: vid f32 [T,H,W,3], flows f32 [T-1|T,H,W,2]
    (dx,dy interleaved) -> int32 superpixel labels [T,H,W].  Extra keyword
    arguments set further stspix_config fields (e.g. sm_period, prop_niters)."""
    _check_input(vid, "vid")
    _check_input(flows, "flows")
    if vid.dtype != torch.float32 or flows.dtype != torch.float32:
        raise RuntimeError("vid and flows must be float32")
    if vid.dim() != 4:
        raise RuntimeError("vid must be [T,H,W,C]")
    T, H, W, F = vid.shape
    if video_mode and T > 1:
        if flows.dim() != 4 or flows.shape[0] < T - 1 or tuple(flows.shape[1:]) != (H, W, 2):
            raise RuntimeError("flows must be [T-1,H,W,2] (or longer) in video mode")
    cfg = make_config(niters, sp_size, potts, sigma2_app, alpha, split_alpha, **extra)
    out = torch.zeros((T, H, W), dtype=torch.int32, device=vid.device)
    ctx = _ctx(vid.device)
    with torch.cuda.device(vid.device):
        st = ctx.lib.stspix_bist_forward(ctx.handle, _stream(vid.device), vid.data_ptr(),
                                         flows.data_ptr(), T, H, W, F, C.byref(cfg),
                                         int(bool(video_mode)), int(bool(rgb2lab)),
                                         out.data_ptr())
    ctx.check(st)
    return out


def get_marked_video(vid: torch.Tensor, spix: torch.Tensor, color: torch.Tensor) -> torch.Tensor:
    """pyapi.cu:260 get_marked_video: superpixel borders painted with `color`."""
    _check_input(vid, "vid")
    _check_input(spix, "spix")
    if not color.is_contiguous():
        raise RuntimeError("color must be contiguous")
    T, H, W, F = vid.shape
    if color.numel() != F:
        raise RuntimeError("color must have one value per channel")
    color = color.to(device=vid.device, dtype=torch.float32).contiguous()
    spix = spix.to(torch.int32).contiguous()
    marked = torch.zeros((T, H, W, F), dtype=torch.float32, device=vid.device)
    ctx = _ctx(vid.device)
    with torch.cuda.device(vid.device):
        st = ctx.lib.stspix_get_marked_video(ctx.handle, _stream(vid.device), vid.data_ptr(),
                                             spix.data_ptr(), color.data_ptr(), T, H, W, F,
                                             marked.data_ptr())
    ctx.check(st)
    return marked


# ---------------------------------------------------------------------------
# Cross-frame parameters (SuperpixelParams, structs.h:13-48).
PARAM_FIELDS = [("mu_app", torch.float32, 3), ("prior_mu_app", torch.float32, 3),
                ("mu_shape", torch.float64, 2), ("sigma_shape", torch.float64, 3),
                ("logdet_sigma_shape", torch.float32, 1), ("prior_mu_shape", torch.float64, 2),
                ("prior_sigma_shape", torch.float64, 3), ("sample_sigma_shape", torch.float64, 3),
                ("counts", torch.int32, 1), ("sm_counts", torch.int32, 1),
                ("prior_counts", torch.float32, 1), ("ids", torch.int32, 1),
                ("invalid_counts", torch.float32, 1)]


class SuperpixelParams:
    """The 13 per-superpixel tensors of the reference's SuperpixelParams, with
    `capacity` rows allocated and the first `n` valid."""

    def __init__(self, capacity: int, device):
        self.capacity = int(capacity)
        self.n = 0
        for name, dt, per in PARAM_FIELDS:
            setattr(self, "_" + name, torch.zeros(self.capacity * per, dtype=dt, device=device))

    def struct(self) -> _lib.ParamsC:
        ps = _lib.ParamsC()
        for name, _, _ in PARAM_FIELDS:
            setattr(ps, name, getattr(self, "_" + name).data_ptr())
        ps.capacity = self.capacity
        return ps

    def field(self, name: str) -> torch.Tensor:
        per = dict((n, p) for n, _, p in PARAM_FIELDS)[name]
        t = getattr(self, "_" + name)[: self.n * per]
        return t.view(self.n, per) if per > 1 else t

    def as_dict(self) -> dict:
        return {name: self.field(name) for name, _, _ in PARAM_FIELDS}


def hex_count(H: int, W: int, sp_size: int) -> int:
    import math
    Hh = math.sqrt(float(sp_size) ** 2 / (1.5 * math.sqrt(3.0)))
    w = math.sqrt(3.0) * Hh
    return (int(math.floor(W / w)) + 2) * (int(math.floor(H / (1.5 * Hh))) + 2)


def run_bass(img: torch.Tensor, **cfg_kw):
    """bass.cu:221 run_bass on one frame f32 [H,W,3] -> (labels i32 [H,W], params)."""
    _check_input(img, "img")
    H, W = img.shape[:2]
    cfg = make_config(**cfg_kw)
    params = SuperpixelParams(30 * hex_count(H, W, cfg.sp_size), img.device)
    labels = torch.zeros((H, W), dtype=torch.int32, device=img.device)
    ps = params.struct()
    n = C.c_int(0)
    ctx = _ctx(img.device)
    st = ctx.lib.stspix_run_bass(ctx.handle, _stream(img.device), img.data_ptr(), H, W,
                                 C.byref(cfg), labels.data_ptr(), C.byref(ps), C.byref(n))
    ctx.check(st)
    params.n = n.value
    return labels, params


def shift_and_fill(labels_prev: torch.Tensor, params: SuperpixelParams, flow: torch.Tensor):
    """shift_and_fill.cu:108: -> (filled, shifted); updates params.prior_counts and
    params.invalid_counts in place."""
    _check_input(labels_prev, "spix")
    _check_input(flow, "flow")
    H, W = labels_prev.shape
    filled = torch.empty((H, W), dtype=torch.int32, device=labels_prev.device)
    shifted = torch.empty_like(filled)
    ps = params.struct()
    ctx = _ctx(labels_prev.device)
    st = ctx.lib.stspix_shift_and_fill(ctx.handle, _stream(labels_prev.device),
                                       labels_prev.data_ptr(), C.byref(ps), params.n,
                                       flow.data_ptr(), H, W, filled.data_ptr(),
                                       shifted.data_ptr())
    ctx.check(st)
    return filled, shifted


def run_prop(img: torch.Tensor, niters: int, filled: torch.Tensor, shifted: torch.Tensor,
             params_prev: SuperpixelParams, **cfg_kw):
    """prop.cu:677 run_prop -> (labels i32 [H,W], params)."""
    _check_input(img, "img")
    H, W = img.shape[:2]
    cfg = make_config(**cfg_kw)
    out = SuperpixelParams(10 * params_prev.n, img.device)
    labels = torch.zeros((H, W), dtype=torch.int32, device=img.device)
    pprev = params_prev.struct()
    ps = out.struct()
    n = C.c_int(0)
    ctx = _ctx(img.device)
    st = ctx.lib.stspix_run_prop(ctx.handle, _stream(img.device), img.data_ptr(), H, W,
                                 C.byref(cfg), int(niters), filled.data_ptr(), shifted.data_ptr(),
                                 C.byref(pprev), params_prev.n, labels.data_ptr(), C.byref(ps),
                                 C.byref(n))
    ctx.check(st)
    out.n = n.value
    return labels, out


def frame_log(device=None) -> _lib.FrameLog:
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    return _ctx(dev).frame_log()


def kernel_launches(device=None) -> int:
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    return _ctx(dev).launches()


# ---------------------------------------------------------------------------
# Colour front end (rgb2lab.cu; the reference's frame pipeline, not bist_forward).
def rgb2lab(img: torch.Tensor) -> torch.Tensor:
    """f32 [...,3] (first channel read as blue, as the reference) -> CIELAB stored as
    (L/-100, a/100, b/100), rgb2lab.cu:51-122."""
    _check_input(img, "img")
    out = img.clone()
    ctx = _ctx(img.device)
    ctx.check(ctx.lib.stspix_rgb2lab(ctx.handle, _stream(img.device), img.data_ptr(),
                                     out.data_ptr(), img.numel() // 3))
    return out


def lab2rgb(lab: torch.Tensor) -> torch.Tensor:
    """The inverse of rgb2lab (rgb2lab.cu:124-181), clamped to [0, 1]."""
    _check_input(lab, "lab")
    out = lab.clone()
    ctx = _ctx(lab.device)
    ctx.check(ctx.lib.stspix_lab2rgb(ctx.handle, _stream(lab.device), lab.data_ptr(),
                                     out.data_ptr(), lab.numel() // 3))
    return out


def rescale_u8(img: torch.Tensor, scale: float = 255.0) -> torch.Tensor:
    """u8 frames -> f32 value / scale (rgb2lab.cu:184 rescale_image_kernel)."""
    _check_input(img, "img")
    if img.dtype != torch.uint8:
        raise RuntimeError("img must be uint8")
    out = torch.empty(img.shape, dtype=torch.float32, device=img.device)
    ctx = _ctx(img.device)
    ctx.check(ctx.lib.stspix_rescale_u8(ctx.handle, _stream(img.device), img.data_ptr(),
                                        out.data_ptr(), img.numel(), float(scale)))
    return out
