"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module.  It builds liboracle_bass.so from bass_oracle.cpp on first use.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle_bass.so")
SRC = os.path.join(HERE, "bass_oracle.cpp")
HDR = os.path.join(HERE, "..", "include", "st_spix_gb300.h")
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle (plain g++, no contraction into FMA)."""
    newest = max(os.path.getmtime(SRC), os.path.getmtime(HDR))
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
               "-fPIC", "-shared", "-o", tmp, SRC]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


class Config(C.Structure):
    _fields_ = [("niters", C.c_int), ("niters_seg", C.c_int), ("sp_size", C.c_int),
                ("sm_start", C.c_int), ("sm_period", C.c_int), ("prop_niters", C.c_int),
                ("sigma2_app", C.c_float), ("potts", C.c_float),
                ("alpha_hastings", C.c_float), ("split_alpha", C.c_float),
                ("merge_alpha", C.c_float), ("sigma2_size", C.c_float),
                ("thresh_relabel", C.c_float), ("thresh_new", C.c_float),
                ("accumulator", C.c_int), ("sweep_schedule", C.c_int),
                ("sweep_tile", C.c_int), ("sweep_queue", C.c_int),
                ("lab_ingest", C.c_int)]


class ParamsC(C.Structure):
    _fields_ = [("mu_app", C.c_void_p), ("prior_mu_app", C.c_void_p),
                ("mu_shape", C.c_void_p), ("sigma_shape", C.c_void_p),
                ("logdet_sigma_shape", C.c_void_p), ("prior_mu_shape", C.c_void_p),
                ("prior_sigma_shape", C.c_void_p), ("sample_sigma_shape", C.c_void_p),
                ("counts", C.c_void_p), ("sm_counts", C.c_void_p),
                ("prior_counts", C.c_void_p), ("ids", C.c_void_p),
                ("invalid_counts", C.c_void_p), ("capacity", C.c_int)]


class DumpC(C.Structure):
    _fields_ = [("count", C.c_void_p), ("valid", C.c_void_p), ("prior_count", C.c_void_p),
                ("mu_app", C.c_void_p), ("mu_shape", C.c_void_p),
                ("sigma_shape", C.c_void_p), ("logdet", C.c_void_p), ("sums", C.c_void_p),
                ("capacity", C.c_int)]


class FrameLog(C.Structure):
    _fields_ = [("nsplits", C.c_int), ("nmerges", C.c_int), ("nrevived", C.c_int),
                ("nminted", C.c_int), ("near_ties", C.c_int), ("fill_iters", C.c_int),
                ("niters", C.c_int), ("nspix", C.c_int)]


# Field name -> (dtype, entries per superpixel), in stspix_params order.
PARAM_FIELDS = [("mu_app", np.float32, 3), ("prior_mu_app", np.float32, 3),
                ("mu_shape", np.float64, 2), ("sigma_shape", np.float64, 3),
                ("logdet_sigma_shape", np.float32, 1), ("prior_mu_shape", np.float64, 2),
                ("prior_sigma_shape", np.float64, 3), ("sample_sigma_shape", np.float64, 3),
                ("counts", np.int32, 1), ("sm_counts", np.int32, 1),
                ("prior_counts", np.float32, 1), ("ids", np.int32, 1),
                ("invalid_counts", np.float32, 1)]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            _lib = C.CDLL(build())
            P = C.c_void_p
            _lib.oracle_run_bass.argtypes = [P, C.c_int, C.c_int, C.POINTER(Config), P,
                                             C.POINTER(ParamsC), C.POINTER(C.c_int)]
            _lib.oracle_bass_partial.argtypes = [P, C.c_int, C.c_int, C.POINTER(Config),
                                                 C.c_int, C.c_int, P, C.POINTER(DumpC),
                                                 C.POINTER(C.c_int), C.POINTER(C.c_int)]
            _lib.oracle_shift_and_fill.argtypes = [P, C.POINTER(ParamsC), C.c_int, P,
                                                   C.c_int, C.c_int, P, P]
            _lib.oracle_run_prop.argtypes = [P, C.c_int, C.c_int, C.POINTER(Config), C.c_int,
                                             P, P, C.POINTER(ParamsC), C.c_int, P,
                                             C.POINTER(ParamsC), C.POINTER(C.c_int)]
            _lib.oracle_legacy_split.argtypes = [P, C.c_int, C.c_int, C.POINTER(Config),
                                                 C.c_int, P, C.POINTER(ParamsC), C.c_int, P,
                                                 C.POINTER(ParamsC), C.POINTER(C.c_int)]
            _lib.oracle_bist_forward.argtypes = [P, P, C.c_int, C.c_int, C.c_int,
                                                 C.POINTER(Config), C.c_int, P, P]
            _lib.oracle_get_marked_video.argtypes = [P, P, P, C.c_int, C.c_int, C.c_int, P]
            _lib.oracle_init_seg.argtypes = [P, C.c_int, C.c_int, C.c_int]
            _lib.oracle_hex_count.argtypes = [C.c_int, C.c_int, C.c_int]
            _lib.oracle_find_border.argtypes = [P, P, C.c_int, C.c_int, C.c_int]
            _lib.oracle_fill_missing.argtypes = [P, P, C.c_int, C.c_int, C.c_int, C.c_int,
                                                 C.POINTER(C.c_int)]
            _lib.oracle_invalidate_disconnected.argtypes = [P, C.c_int, C.c_int, C.c_int]
            _lib.oracle_get_frame_log.argtypes = [C.POINTER(FrameLog)]
            F = C.c_float
            _lib.oracle_update_params_given.argtypes = [P, P, C.c_int, C.c_int, C.c_int, C.c_int,
                                                        F, P, P, P, P, P, P, P, P, P, P, P]
            _lib.oracle_update_seg_given.argtypes = [P, P, C.c_int, C.c_int, C.c_int, C.c_int,
                                                     F, F, P, P, P, P, P]
            _lib.oracle_split_bfs.argtypes = [P, C.c_int, C.c_int, C.c_int, P, P, C.c_int, P]
            _lib.oracle_cc_roots.argtypes = [P, C.c_int, C.c_int, P]
            _lib.oracle_default_config.argtypes = [C.POINTER(Config)]
            _lib.oracle_sm_step.argtypes = [P, P, C.c_int, C.c_int, C.POINTER(Config), C.c_int,
                                            P, P, P, P, C.c_int, C.c_int, C.c_int, P, P, P, P,
                                            P, P, C.POINTER(C.c_int)]
            _lib.oracle_sm_step_ex.argtypes = [
                P, P, C.c_int, C.c_int, C.POINTER(Config), C.c_int, P, P, P, P, C.c_int,
                C.c_int, C.c_int, P, P, P, C.c_int, C.c_int, P, P, P, P, P, C.POINTER(C.c_int)]
    return _lib


def default_config(**kw) -> Config:
    c = Config()
    lib().oracle_default_config(C.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def alloc_params(cap: int) -> dict:
    return {name: np.zeros(cap * per, dt) for name, dt, per in PARAM_FIELDS}


def params_struct(arrs: dict, cap: int) -> ParamsC:
    ps = ParamsC()
    for name, _, _ in PARAM_FIELDS:
        setattr(ps, name, arrs[name].ctypes.data)
    ps.capacity = cap
    return ps


def hex_count(H, W, sp_size):
    return lib().oracle_hex_count(H, W, sp_size)


def init_seg(H, W, sp_size):
    lab = np.zeros((H, W), np.int32)
    n = lib().oracle_init_seg(_p(lab), H, W, sp_size)
    return lab, n


def find_border(labels: np.ndarray, mode: int = 0):
    labels = np.ascontiguousarray(labels, np.int32)
    H, W = labels.shape
    b = np.zeros((H, W), np.uint8)
    lib().oracle_find_border(_p(labels), _p(b), H, W, mode)
    return b


def run_bass(img: np.ndarray, cfg: Config):
    img = np.ascontiguousarray(img, np.float32)
    H, W = img.shape[:2]
    cap = 30 * hex_count(H, W, cfg.sp_size)
    lab = np.zeros((H, W), np.int32)
    arrs = alloc_params(cap)
    ps = params_struct(arrs, cap)
    n = C.c_int(0)
    st = lib().oracle_run_bass(_p(img), H, W, C.byref(cfg), _p(lab), C.byref(ps), C.byref(n))
    out = {k: v[: n.value * per] for (k, _, per), v in zip(PARAM_FIELDS, [arrs[f[0]] for f in PARAM_FIELDS])}
    return st, lab, out, n.value


def bass_partial(img: np.ndarray, cfg: Config, iters: int, extra_update: int = 0):
    img = np.ascontiguousarray(img, np.float32)
    H, W = img.shape[:2]
    cap = 30 * hex_count(H, W, cfg.sp_size)
    lab = np.zeros((H, W), np.int32)
    d = {"count": np.zeros(cap, np.int32), "valid": np.zeros(cap, np.uint8),
         "prior_count": np.zeros(cap, np.float32), "mu_app": np.zeros(cap * 3, np.float32),
         "mu_shape": np.zeros(cap * 2, np.float64), "sigma_shape": np.zeros(cap * 3, np.float64),
         "logdet": np.zeros(cap, np.float64), "sums": np.zeros(cap * 8, np.int64)}
    ds = DumpC()
    for k, v in d.items():
        setattr(ds, k, v.ctypes.data)
    ds.capacity = cap
    nbuf, mx = C.c_int(0), C.c_int(0)
    st = lib().oracle_bass_partial(_p(img), H, W, C.byref(cfg), iters, extra_update, _p(lab),
                                   C.byref(ds), C.byref(nbuf), C.byref(mx))
    return st, lab, d, nbuf.value, mx.value


def shift_and_fill(labels_prev, params_prev: dict, n_prev: int, flow):
    labels_prev = np.ascontiguousarray(labels_prev, np.int32)
    flow = np.ascontiguousarray(flow, np.float32)
    H, W = labels_prev.shape
    arrs = {k: np.array(v, copy=True) for k, v in params_prev.items()}
    ps = params_struct(arrs, n_prev)
    filled = np.zeros((H, W), np.int32)
    shifted = np.zeros((H, W), np.int32)
    st = lib().oracle_shift_and_fill(_p(labels_prev), C.byref(ps), n_prev, _p(flow), H, W,
                                     _p(filled), _p(shifted))
    return st, filled, shifted, arrs


def run_prop(img, cfg: Config, niters: int, filled, shifted, params_prev: dict, n_prev: int):
    img = np.ascontiguousarray(img, np.float32)
    H, W = img.shape[:2]
    cap = 10 * n_prev
    arrs_prev = {k: np.ascontiguousarray(v) for k, v in params_prev.items()}
    pprev = params_struct(arrs_prev, n_prev)
    arrs = alloc_params(cap)
    ps = params_struct(arrs, cap)
    lab = np.zeros((H, W), np.int32)
    n = C.c_int(0)
    filled = np.ascontiguousarray(filled, np.int32)
    shifted = np.ascontiguousarray(shifted, np.int32)
    st = lib().oracle_run_prop(_p(img), H, W, C.byref(cfg), niters, _p(filled), _p(shifted),
                               C.byref(pprev), n_prev, _p(lab), C.byref(ps), C.byref(n))
    out = {name: arrs[name][: n.value * per] for name, _, per in PARAM_FIELDS}
    return st, lab, out, n.value


def legacy_split(img, cfg: Config, direction: int, spix, params_prev: dict, n_prev: int):
    """prop/bass.cu:389 run_split_py restated on the propagated model: one split step
    in `direction` on the labels spix with the previous params."""
    img = np.ascontiguousarray(img, np.float32)
    H, W = img.shape[:2]
    cap = 10 * n_prev
    pprev = params_struct({k: np.ascontiguousarray(v) for k, v in params_prev.items()}, n_prev)
    arrs = alloc_params(cap)
    ps = params_struct(arrs, cap)
    lab = np.zeros((H, W), np.int32)
    n = C.c_int(0)
    spix = np.ascontiguousarray(spix, np.int32)
    st = lib().oracle_legacy_split(_p(img), H, W, C.byref(cfg), int(direction), _p(spix),
                                   C.byref(pprev), n_prev, _p(lab), C.byref(ps), C.byref(n))
    out = {name: arrs[name][: n.value * per] for name, _, per in PARAM_FIELDS}
    return st, lab, out, n.value


def bist_forward(vid, flows, cfg: Config, video_mode: bool):
    vid = np.ascontiguousarray(vid, np.float32)
    T, H, W = vid.shape[:3]
    if flows is None:
        flows = np.zeros((max(T - 1, 1), H, W, 2), np.float32)
    flows = np.ascontiguousarray(flows, np.float32)
    out = np.zeros((T, H, W), np.int32)
    used = np.zeros(T, np.int32)
    st = lib().oracle_bist_forward(_p(vid), _p(flows), T, H, W, C.byref(cfg),
                                   int(bool(video_mode)), _p(out), _p(used))
    return st, out, used


def get_marked_video(vid, spix, color):
    vid = np.ascontiguousarray(vid, np.float32)
    spix = np.ascontiguousarray(spix, np.int32)
    color = np.ascontiguousarray(color, np.float32)
    T, H, W = vid.shape[:3]
    out = np.zeros_like(vid)
    lib().oracle_get_marked_video(_p(vid), _p(spix), _p(color), T, H, W, _p(out))
    return out


def fill_missing(seg, centers, break_iter=1000):
    seg = np.array(seg, np.int32, copy=True)
    centers = np.ascontiguousarray(centers, np.float64)
    H, W = seg.shape
    it = C.c_int(0)
    st = lib().oracle_fill_missing(_p(seg), _p(centers), centers.shape[0], H, W, break_iter,
                                   C.byref(it))
    return st, seg, it.value


def invalidate_disconnected(seg, nspix):
    seg = np.array(seg, np.int32, copy=True)
    H, W = seg.shape
    lib().oracle_invalidate_disconnected(_p(seg), H, W, nspix)
    return seg


def last_log() -> FrameLog:
    lg = FrameLog()
    lib().oracle_get_frame_log(C.byref(lg))
    return lg


# Stage functions on caller-supplied state (pinned against the reference's kernels).
def update_params_given(img, labels, nbuf, sp_size, sigma2_app, valid, prop, prior_count,
                        prior_icov, sample_sigma):
    img = np.ascontiguousarray(img, np.float32)
    labels = np.ascontiguousarray(labels, np.int32)
    args = [np.ascontiguousarray(valid, np.int32), np.ascontiguousarray(prop, np.int32),
            np.ascontiguousarray(prior_count, np.float32),
            np.ascontiguousarray(prior_icov, np.float64),
            np.ascontiguousarray(sample_sigma, np.float64)]
    out = dict(count=np.zeros(nbuf, np.int32), mu_app=np.zeros(3 * nbuf, np.float32),
               mu_shape=np.zeros(2 * nbuf, np.float64),
               sigma_shape=np.zeros(3 * nbuf, np.float64), logdet=np.zeros(nbuf, np.float64),
               valid=np.zeros(nbuf, np.int32))
    H, W = labels.shape
    lib().oracle_update_params_given(_p(img), _p(labels), H, W, nbuf, sp_size, sigma2_app,
                                     *[_p(a) for a in args], _p(out["count"]), _p(out["mu_app"]),
                                     _p(out["mu_shape"]), _p(out["sigma_shape"]),
                                     _p(out["logdet"]), _p(out["valid"]))
    return out


def update_seg_given(img, labels, nbuf, niters_seg, sigma2_app, potts, count, mu_app, mu_shape,
                     sigma_shape, logdet):
    img = np.ascontiguousarray(img, np.float32)
    lab = np.array(labels, np.int32, copy=True)
    a = [np.ascontiguousarray(count, np.int32), np.ascontiguousarray(mu_app, np.float32),
         np.ascontiguousarray(mu_shape, np.float64), np.ascontiguousarray(sigma_shape, np.float64),
         np.ascontiguousarray(logdet, np.float64)]
    H, W = lab.shape
    lib().oracle_update_seg_given(_p(img), _p(lab), H, W, nbuf, niters_seg, sigma2_app, potts,
                                  *[_p(x) for x in a])
    return lab


def split_bfs(labels, nbuf, valid, mu_shape, direction):
    labels = np.ascontiguousarray(labels, np.int32)
    out = np.zeros(labels.shape, np.int32)
    H, W = labels.shape
    lib().oracle_split_bfs(_p(labels), H, W, nbuf, _p(np.ascontiguousarray(valid, np.int32)),
                           _p(np.ascontiguousarray(mu_shape, np.float64)), direction, _p(out))
    return out


def cc_roots(seg):
    seg = np.ascontiguousarray(seg, np.int32)
    out = np.zeros(seg.shape, np.int32)
    lib().oracle_cc_roots(_p(seg), seg.shape[0], seg.shape[1], _p(out))
    return out


def rgb2lab(rgb):
    """rgb2lab.cu:51-122 restated (first channel read as blue; L/-100, a/100, b/100)."""
    rgb = np.ascontiguousarray(rgb, np.float32)
    out = rgb.copy()
    lib().oracle_rgb2lab(_p(rgb), _p(out), C.c_longlong(rgb.size // 3))
    return out


def lab2rgb(lab):
    lab = np.ascontiguousarray(lab, np.float32)
    out = lab.copy()
    lib().oracle_lab2rgb(_p(lab), _p(out), C.c_longlong(lab.size // 3))
    return out


def rescale_u8(img, scale=255.0):
    img = np.ascontiguousarray(img, np.uint8)
    out = np.empty(img.shape, np.float32)
    lib().oracle_rescale_u8(_p(img), _p(out), C.c_longlong(img.size), C.c_float(scale))
    return out


def sm_step(img, labels, cfg: Config, nbuf, valid, prior_count, prop, sample_sigma, max_spix,
            kind, direction, shifted=None, relabel=None, border=None):
    """One split (kind 0 BASS / 2 propagated) or merge (kind 1 / 3) step on a given
    state (oracle_sm_step): per id the Hastings log-ratio (NaN where none is scored),
    merge candidate, threshold test and decision, and the labels after the step.
    relabel=(rid, nspix_prev): `labels` are those update_params saw and rid[s] the id a
    propagated frame's relabel_spix gave s (-1: kept), applied before the step
    (oracle_sm_step_ex).  The step keeps the relabelled labels.  border: the border
    mask to use in place of the border of `labels` (the one a running loop holds)."""
    img = np.ascontiguousarray(img, np.float32)
    labels = np.ascontiguousarray(labels, np.int32)
    H, W = labels.shape
    valid = np.ascontiguousarray(valid, np.uint8)
    prior_count = np.ascontiguousarray(prior_count, np.float32)
    prop = np.ascontiguousarray(prop, np.uint8)
    sample_sigma = np.ascontiguousarray(sample_sigma, np.float64)
    shifted = (np.ascontiguousarray(shifted, np.int32) if shifted is not None
               else np.zeros((H, W), np.int32))
    out = dict(h=np.zeros(nbuf, np.float64), pair=np.zeros(nbuf, np.int32),
               want=np.zeros(nbuf, np.uint8), accept=np.zeros(nbuf, np.uint8),
               labels=np.zeros((H, W), np.int32))
    mx = C.c_int(0)
    tail = (_p(out["h"]), _p(out["pair"]), _p(out["want"]), _p(out["accept"]),
            _p(out["labels"]), C.byref(mx))
    head = (_p(img), _p(labels), H, W, C.byref(cfg), nbuf, _p(valid), _p(prior_count), _p(prop),
            _p(sample_sigma), int(max_spix), int(kind), int(direction), _p(shifted))
    if relabel is None and border is None:
        st = lib().oracle_sm_step(*head, *tail)
    else:
        rid, nspix_prev = relabel if relabel is not None else (None, 0)
        rid = np.ascontiguousarray(rid, np.int32) if rid is not None else None
        border = np.ascontiguousarray(border, np.uint8) if border is not None else None
        st = lib().oracle_sm_step_ex(*head, _p(border) if border is not None else None,
                                     _p(rid) if rid is not None else None,
                                     len(rid) if rid is not None else 0, int(nspix_prev), *tail)
    out["max_spix"] = mx.value
    out["status"] = st
    return out
