"""Batched form of the streaming-BASS path: many frames of uneven size in one pass.

The reference processes one frame per call (st_spix/csrc/bist/pyapi.cu:46
main_loop).  Here a batch mixes

  * independent frames (the reference's run_bass, bass.cu:221), and
  * the next frame of any number of video streams (shift_and_fill + run_prop,
    shift_and_fill.cu:108 / prop.cu:677), whose labels, superpixel parameters and
    superpixel count stay resident on the device between calls (`Video`).

Every kernel of the per-frame path is launched once for the whole batch (the C
ABI's stspix_process_batch), and a frame's result is the same alone and in any
batch.  Work runs on torch's current CUDA stream.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional

import torch

from . import _lib
from .bist_cuda import _check_input, _ctx, _stream, make_config


class Video:
    """Resident device state of one video stream of H x W frames (stspix_video)."""

    def __init__(self, H: int, W: int, device=None):
        idx = None if device is None else torch.device(device).index
        dev = torch.device("cuda", torch.cuda.current_device() if idx is None else idx)
        self.device = dev
        self.H, self.W = int(H), int(W)
        self.ctx = _ctx(dev)
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.stspix_video_create(self.ctx.handle, C.byref(h), self.H,
                                                        self.W))
        self.handle = h

    @property
    def nspix(self) -> int:
        """Superpixels of the stream's last frame (0 before its first frame)."""
        return int(self.ctx.lib.stspix_video_nspix(self.handle))

    @property
    def frames(self) -> int:
        return int(self.ctx.lib.stspix_video_frames(self.handle))

    def reset(self):
        """Forget the history: the next frame starts a new video."""
        self.ctx.lib.stspix_video_reset(self.handle)

    def save(self) -> bytes:
        """Snapshot of the resident state (labels, superpixel count and parameters of
        the last frame) as bytes (stspix_video_save)."""
        n = C.c_longlong(0)
        st = _stream(self.device)
        self.ctx.check(self.ctx.lib.stspix_video_save(self.handle, st, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        self.ctx.check(self.ctx.lib.stspix_video_save(self.handle, st, buf, n.value, C.byref(n)))
        return buf.raw

    def load(self, snapshot: bytes):
        """Restore a snapshot taken by save(): the next frame continues that stream."""
        self.ctx.check(self.ctx.lib.stspix_video_load(self.handle, _stream(self.device),
                                                      snapshot, len(snapshot)))

    def close(self):
        if getattr(self, "handle", None):
            self.ctx.lib.stspix_video_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Frame:
    """One frame of a batch.  img f32 [H,W,3]; flow f32 [H,W,2] (dx,dy) from the
    video's previous frame (needed for every frame of a video after its first);
    sp_size 0 takes the config's."""
    img: torch.Tensor
    flow: Optional[torch.Tensor] = None
    video: Optional[Video] = None
    sp_size: int = 0
    labels: Optional[torch.Tensor] = None   # i32 [H,W] output (allocated if None)
    # filled in by process_batch
    nspix: int = 0
    niters: int = 0
    status: int = 0
    log: Optional[_lib.FrameLog] = None


def process_batch(frames: List[Frame], **cfg_kw) -> List[Frame]:
    """Run one batch; returns `frames` with labels, nspix, niters, status and log set.
    Keyword arguments are config fields (niters, sp_size, potts, sigma2_app, alpha,
    split_alpha, sm_period, prop_niters, ...)."""
    if not frames:
        return frames
    dev = frames[0].img.device
    cfg = make_config(**cfg_kw)
    arr = (_lib.FrameC * len(frames))()
    for i, f in enumerate(frames):
        _check_input(f.img, "img")
        if f.img.dtype != torch.float32 or f.img.dim() != 3 or f.img.shape[2] != 3:
            raise RuntimeError("img must be float32 [H,W,3]")
        if f.img.device != dev:
            raise RuntimeError("all frames of a batch must be on one device")
        H, W = f.img.shape[:2]
        if f.labels is None:
            f.labels = torch.empty((H, W), dtype=torch.int32, device=dev)
        _check_input(f.labels, "labels")
        if f.flow is not None:
            _check_input(f.flow, "flow")
            if tuple(f.flow.shape) != (H, W, 2) or f.flow.dtype != torch.float32:
                raise RuntimeError("flow must be float32 [H,W,2]")
        a = arr[i]
        a.img = f.img.data_ptr()
        a.flow = f.flow.data_ptr() if f.flow is not None else None
        a.H, a.W = H, W
        a.sp_size = int(f.sp_size)
        a.labels_out = f.labels.data_ptr()
        a.video = f.video.handle if f.video is not None else None
    ctx = _ctx(dev)
    with torch.cuda.device(dev):
        st = ctx.lib.stspix_process_batch(ctx.handle, _stream(dev), arr, len(frames),
                                          C.byref(cfg))
    for i, f in enumerate(frames):
        f.nspix, f.niters, f.status = arr[i].nspix, arr[i].niters, arr[i].status
        lg = _lib.FrameLog()
        C.memmove(C.byref(lg), C.byref(arr[i].log), C.sizeof(lg))
        f.log = lg
    ctx.check(st)
    return frames


def last_batch_ms(device=None) -> float:
    """GPU time of the last batch run on torch's current stream (CUDA events)."""
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    return _ctx(dev).last_batch_ms()
