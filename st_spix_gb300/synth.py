"""Seeded synthetic inputs standing in for the DAVIS / SegTrackv2 videos the
reference measures on (those datasets are not available here).

Frames are piecewise-constant Voronoi images with iid Gaussian noise; videos move
every region by its own affine motion (translation + rotation about its seed) and
come with the ground-truth forward flow.  Everything is a pure function of the
seed (numpy PCG64).
"""
from __future__ import annotations

import math

import numpy as np

try:  # scipy is present in both environments; fall back to a chunked scan.
    from scipy.spatial import cKDTree as _KDTree
except Exception:  # pragma: no cover
    _KDTree = None


def _nearest(seeds_xy: np.ndarray, H: int, W: int) -> np.ndarray:
    ys, xs = np.mgrid[0:H, 0:W]
    pts = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.float64)
    if _KDTree is not None:
        _, idx = _KDTree(seeds_xy).query(pts)
        return idx.reshape(H, W).astype(np.int32)
    out = np.empty(pts.shape[0], np.int32)
    for s in range(0, pts.shape[0], 65536):
        d = ((pts[s:s + 65536, None, :] - seeds_xy[None]) ** 2).sum(-1)
        out[s:s + 65536] = d.argmin(1)
    return out.reshape(H, W)


def voronoi_frame(H: int, W: int, nseeds: int, sigma: float, seed: int = 0):
    """One Voronoi frame: f32 [H,W,3] in [0,1] and the region map i32 [H,W]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    seeds = rng.uniform([0, 0], [W, H], size=(nseeds, 2))
    colors = rng.uniform(0, 1, size=(nseeds, 3)).astype(np.float32)
    reg = _nearest(seeds, H, W)
    img = colors[reg] + rng.normal(0, sigma, size=(H, W, 3)).astype(np.float32)
    return np.clip(img, 0, 1).astype(np.float32), reg


def voronoi_video(H: int, W: int, T: int, nseeds: int, sigma: float, seed: int = 0,
                  max_shift: float = 4.0, max_rot_deg: float = 1.0):
    """Video f32 [T,H,W,3], forward flow f32 [T-1,H,W,2] (dx,dy interleaved) and
    region maps i32 [T,H,W].  Region r moves by translation t_r (uniform in
    [-max_shift,max_shift] px/frame) and rotation th_r (uniform in
    [-max_rot_deg,max_rot_deg] deg/frame) about its seed; frame t is the Voronoi
    partition of the moved seeds (ties to the lower region index) and the flow of a
    pixel is its region's motion."""
    rng = np.random.Generator(np.random.PCG64(seed))
    seeds = rng.uniform([0, 0], [W, H], size=(nseeds, 2))
    colors = rng.uniform(0, 1, size=(nseeds, 3)).astype(np.float32)
    trans = rng.uniform(-max_shift, max_shift, size=(nseeds, 2))
    rot = np.deg2rad(rng.uniform(-max_rot_deg, max_rot_deg, size=nseeds))
    vid = np.empty((T, H, W, 3), np.float32)
    flows = np.empty((max(T - 1, 0), H, W, 2), np.float32)
    regs = np.empty((T, H, W), np.int32)
    ys, xs = np.mgrid[0:H, 0:W].astype(np.float64)
    cur = seeds.copy()
    for t in range(T):
        reg = _nearest(cur, H, W)
        regs[t] = reg
        noise = rng.normal(0, sigma, size=(H, W, 3)).astype(np.float32)
        vid[t] = np.clip(colors[reg] + noise, 0, 1)
        if t < T - 1:
            c = cur[reg]
            th = rot[reg]
            dx, dy = xs - c[..., 0], ys - c[..., 1]
            cs, sn = np.cos(th), np.sin(th)
            nx = cs * dx - sn * dy + c[..., 0] + trans[reg, 0]
            ny = sn * dx + cs * dy + c[..., 1] + trans[reg, 1]
            flows[t, ..., 0] = (nx - xs).astype(np.float32)
            flows[t, ..., 1] = (ny - ys).astype(np.float32)
            cur = cur + trans
    return vid, flows, regs


def voronoi_video_device(H: int, W: int, T: int, nseeds: int, sigma: float, seed: int = 0,
                         max_shift: float = 4.0, max_rot_deg: float = 1.0, device="cuda",
                         regions: bool = False):
    """voronoi_video's scene model generated on a torch device (for benchmarks that
    need many large videos): the same seeds, colours and motions drawn from the
    numpy generator of `seed`; region maps as the nearest moved seed (first index
    on ties) and the noise from a torch generator seeded with `seed`.  Returns
    (vid f32 [T,H,W,3], flows f32 [T-1,H,W,2]) on the device, and the region maps
    i32 [T,H,W] as a third item when `regions`."""
    import torch
    rng = np.random.Generator(np.random.PCG64(seed))
    seeds = rng.uniform([0, 0], [W, H], size=(nseeds, 2))
    colors = rng.uniform(0, 1, size=(nseeds, 3)).astype(np.float32)
    trans = rng.uniform(-max_shift, max_shift, size=(nseeds, 2))
    rot = np.deg2rad(rng.uniform(-max_rot_deg, max_rot_deg, size=nseeds))
    dev = torch.device(device)
    g = torch.Generator(device=dev)
    g.manual_seed(int(seed))
    colors_t = torch.from_numpy(colors).to(dev)
    trans_t = torch.from_numpy(trans).to(dev)
    rot_t = torch.from_numpy(rot).to(dev)
    ys, xs = torch.meshgrid(torch.arange(H, device=dev, dtype=torch.float64),
                            torch.arange(W, device=dev, dtype=torch.float64), indexing="ij")
    vid = torch.empty((T, H, W, 3), dtype=torch.float32, device=dev)
    flows = torch.empty((max(T - 1, 0), H, W, 2), dtype=torch.float32, device=dev)
    regs = torch.empty((T, H, W), dtype=torch.int32, device=dev) if regions else None
    cur = torch.from_numpy(seeds).to(dev)
    rows = max(1, (1 << 24) // max(1, W * nseeds))
    for t in range(T):
        reg = torch.empty((H, W), dtype=torch.long, device=dev)
        for y0 in range(0, H, rows):
            y1 = min(H, y0 + rows)
            dx = xs[y0:y1, :, None] - cur[:, 0]
            dy = ys[y0:y1, :, None] - cur[:, 1]
            reg[y0:y1] = (dx * dx + dy * dy).argmin(-1)
        if regions:
            regs[t] = reg
        noise = torch.randn((H, W, 3), generator=g, device=dev, dtype=torch.float32) * sigma
        vid[t] = (colors_t[reg] + noise).clamp_(0, 1)
        if t < T - 1:
            c = cur[reg]
            th = rot_t[reg]
            dx, dy = xs - c[..., 0], ys - c[..., 1]
            cs, sn = torch.cos(th), torch.sin(th)
            nx = cs * dx - sn * dy + c[..., 0] + trans_t[reg, 0]
            ny = sn * dx + cs * dy + c[..., 1] + trans_t[reg, 1]
            flows[t, ..., 0] = (nx - xs).float()
            flows[t, ..., 1] = (ny - ys).float()
            cur = cur + trans_t
    return (vid, flows, regs) if regions else (vid, flows)


# Workloads (shapes and value distributions of the benchmark configurations).
def config0(seed: int = 0):
    """240x320 RGB, 200 Voronoi seeds, noise sigma 0.05."""
    img, reg = voronoi_frame(240, 320, 200, 0.05, seed)
    return img, reg


def config1(seed: int = 0, T: int = 30, H: int = 480, W: int = 854):
    """480x854 RGB video, 400 seeds, affine motion, noise sigma 0.03."""
    return voronoi_video(H, W, T, 400, 0.03, seed)


def stream_resolution_mix(n: int, seed: int = 0):
    """Resolutions of n streams mixed 360p / 720p / 1080p at 0.4 / 0.4 / 0.2."""
    rng = np.random.Generator(np.random.PCG64(seed))
    choice = rng.choice(3, size=n, p=[0.4, 0.4, 0.2])
    table = [(360, 640), (720, 1280), (1080, 1920)]
    return [table[c] for c in choice]


def default_log_alpha() -> float:
    return math.log(0.5)
