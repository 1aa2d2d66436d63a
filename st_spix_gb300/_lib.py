"""ctypes binding of libstspix_gb300.so (the C ABI in include/st_spix_gb300.h).

The library is the only compute path: if it is missing or fails to load this module
raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None


class Config(C.Structure):
    """stspix_config."""
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
    """stspix_params (device pointers)."""
    _fields_ = [("mu_app", C.c_void_p), ("prior_mu_app", C.c_void_p),
                ("mu_shape", C.c_void_p), ("sigma_shape", C.c_void_p),
                ("logdet_sigma_shape", C.c_void_p), ("prior_mu_shape", C.c_void_p),
                ("prior_sigma_shape", C.c_void_p), ("sample_sigma_shape", C.c_void_p),
                ("counts", C.c_void_p), ("sm_counts", C.c_void_p),
                ("prior_counts", C.c_void_p), ("ids", C.c_void_p),
                ("invalid_counts", C.c_void_p), ("capacity", C.c_int)]


class DumpC(C.Structure):
    """stspix_state_dump (device pointers)."""
    _fields_ = [("count", C.c_void_p), ("valid", C.c_void_p), ("prior_count", C.c_void_p),
                ("mu_app", C.c_void_p), ("mu_shape", C.c_void_p),
                ("sigma_shape", C.c_void_p), ("logdet", C.c_void_p), ("sums", C.c_void_p),
                ("capacity", C.c_int)]


class FrameLog(C.Structure):
    """stspix_frame_log."""
    _fields_ = [("nsplits", C.c_int), ("nmerges", C.c_int), ("nrevived", C.c_int),
                ("nminted", C.c_int), ("near_ties", C.c_int), ("fill_iters", C.c_int),
                ("niters", C.c_int), ("nspix", C.c_int)]


class FrameC(C.Structure):
    """stspix_frame (device pointers; the last four fields are outputs)."""
    _fields_ = [("img", C.c_void_p), ("flow", C.c_void_p), ("H", C.c_int), ("W", C.c_int),
                ("sp_size", C.c_int), ("labels_out", C.c_void_p), ("video", C.c_void_p),
                ("nspix", C.c_int), ("niters", C.c_int), ("status", C.c_int),
                ("log", FrameLog)]


class QualityC(C.Structure):
    """stspix_quality (host)."""
    _fields_ = [(n, C.c_double) for n in ("tex", "szv", "ev", "ev3d", "psnr", "ave_nsp",
                                          "ue2d", "sa2d", "ue3d", "sa3d")] + \
               [("spnum", C.c_int), ("has_gt", C.c_int)]


# Every symbol declared in include/st_spix_gb300.h.
EXPORTS = ["stspix_default_config", "stspix_create", "stspix_destroy", "stspix_last_error",
           "stspix_version", "stspix_kernel_launches", "stspix_get_frame_log",
           "stspix_bist_forward", "stspix_get_marked_video", "stspix_run_bass",
           "stspix_shift_and_fill", "stspix_run_prop", "stspix_init_seg",
           "stspix_find_border", "stspix_bass_partial", "stspix_profile_enable",
           "stspix_profile_get", "stspix_frame_times", "stspix_get_marked_video_noalloc",
           "stspix_video_create", "stspix_video_destroy", "stspix_video_reset",
           "stspix_video_nspix", "stspix_video_frames", "stspix_process_batch",
           "stspix_footprint", "stspix_last_batch_ms", "stspix_profile_kernels",
           "stspix_label_stats", "stspix_rgb2lab", "stspix_lab2rgb", "stspix_rescale_u8",
           "stspix_video_save", "stspix_video_load", "stspix_evaluate", "stspix_label_range",
           "stspix_count_spix", "stspix_size_variation", "stspix_sp_pooling",
           "stspix_legacy_shift_labels", "stspix_legacy_fill_missing", "stspix_legacy_split",
           "stspix_legacy_rgb_to_lab",
           "stspix_sp_video_pooling", "stspix_downsampled_video_to_pooled",
           "stspix_graph_replays", "stspix_set_batch_graphs", "stspix_sweep_choice",
           "stspix_legacy_update_prior", "stspix_legacy_shift_tensor",
           "stspix_legacy_shift_order", "stspix_legacy_split_disconnected"]

FAMILIES = ["sweep", "stats", "posterior", "split", "merge", "prop", "other"]

# status codes (include/st_spix_gb300.h)
STSPIX_OK, STSPIX_ERR_ARG, STSPIX_ERR_CUDA, STSPIX_ERR_NOMEM = 0, 1, 2, 3
STSPIX_ERR_NOPROGRESS, STSPIX_ERR_ITER_LIMIT, STSPIX_ERR_CAPACITY = 4, 5, 6
STSPIX_ERR_BARRIER, STSPIX_ERR_DEGENERATE, STSPIX_ERR_TOO_LARGE = 7, 8, 9


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first when needed and allowed) the engine library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path) or not _build.up_to_date():
            if not build_if_missing:
                raise RuntimeError(f"st_spix_gb300 CUDA library not built: {path}")
            _build.build()
        lib = C.CDLL(path)
        P, I = C.c_void_p, C.c_int
        sig = {
            "stspix_default_config": (None, [C.POINTER(Config)]),
            "stspix_create": (I, [C.POINTER(C.c_void_p), I]),
            "stspix_destroy": (I, [P]),
            "stspix_last_error": (C.c_char_p, [P]),
            "stspix_version": (I, []),
            "stspix_kernel_launches": (C.c_longlong, [P]),
            "stspix_get_frame_log": (I, [P, C.POINTER(FrameLog)]),
            "stspix_bist_forward": (I, [P, P, P, P, I, I, I, I, C.POINTER(Config), I, I, P]),
            "stspix_get_marked_video": (I, [P, P, P, P, P, I, I, I, I, P]),
            "stspix_run_bass": (I, [P, P, P, I, I, C.POINTER(Config), P, C.POINTER(ParamsC),
                                    C.POINTER(I)]),
            "stspix_shift_and_fill": (I, [P, P, P, C.POINTER(ParamsC), I, P, I, I, P, P]),
            "stspix_run_prop": (I, [P, P, P, I, I, C.POINTER(Config), I, P, P,
                                    C.POINTER(ParamsC), I, P, C.POINTER(ParamsC),
                                    C.POINTER(I)]),
            "stspix_init_seg": (I, [P, P, P, I, I, I, C.POINTER(I)]),
            "stspix_find_border": (I, [P, P, P, P, I, I, I]),
            "stspix_bass_partial": (I, [P, P, P, I, I, C.POINTER(Config), I, I, P,
                                        C.POINTER(DumpC), C.POINTER(I), C.POINTER(I)]),
            "stspix_profile_enable": (I, [P, I]),
            "stspix_profile_get": (I, [P, I, C.POINTER(C.c_longlong), C.POINTER(C.c_double)]),
            "stspix_frame_times": (I, [P, C.POINTER(C.c_double), I]),
            "stspix_get_marked_video_noalloc": (I, [P, P, P, P, I, I, I, I, P]),
            "stspix_video_create": (I, [P, C.POINTER(C.c_void_p), I, I]),
            "stspix_video_destroy": (I, [P]),
            "stspix_video_reset": (I, [P]),
            "stspix_video_nspix": (I, [P]),
            "stspix_video_frames": (C.c_longlong, [P]),
            "stspix_process_batch": (I, [P, P, C.POINTER(FrameC), I, C.POINTER(Config)]),
            "stspix_footprint": (I, [I, I, I, C.POINTER(C.c_longlong),
                                     C.POINTER(C.c_longlong)]),
            "stspix_last_batch_ms": (C.c_double, [P]),
            "stspix_profile_kernels": (I, [P, C.c_char_p, I]),
            "stspix_label_stats": (I, [P, P, P, P, I, I, I, I, P]),
            "stspix_rgb2lab": (I, [P, P, P, P, C.c_longlong]),
            "stspix_video_save": (I, [P, P, P, C.c_longlong, C.POINTER(C.c_longlong)]),
            "stspix_video_load": (I, [P, P, P, C.c_longlong]),
            "stspix_lab2rgb": (I, [P, P, P, P, C.c_longlong]),
            "stspix_rescale_u8": (I, [P, P, P, P, C.c_longlong, C.c_float]),
            "stspix_evaluate": (I, [P, P, P, P, P, I, I, I, C.POINTER(QualityC)]),
            "stspix_label_range": (I, [P, P, P, C.c_longlong, C.POINTER(C.c_int32)]),
            "stspix_count_spix": (I, [P, P, P, I, C.c_longlong, C.c_int32, I, P]),
            "stspix_size_variation": (I, [P, P, P, I, I, C.POINTER(C.c_double),
                                          C.POINTER(C.c_double), C.POINTER(C.c_double)]),
            "stspix_sp_pooling": (I, [P, P, P, P, I, I, I, I, P, P]),
            "stspix_legacy_shift_labels": (I, [P, P, P, P, I, I, I, P, P]),
            "stspix_legacy_fill_missing": (I, [P, P, P, P, I, P, I, I, I, I, C.POINTER(I),
                                               C.POINTER(I)]),
            "stspix_legacy_split": (I, [P, P, P, I, I, C.POINTER(Config), I, P,
                                        C.POINTER(ParamsC), I, P, C.POINTER(ParamsC),
                                        C.POINTER(I)]),
            "stspix_legacy_rgb_to_lab": (I, [P, P, P, P, C.c_longlong]),
            "stspix_sp_video_pooling": (I, [P, P, P, P, I, I, I, I, I, I, P, P, P]),
            "stspix_downsampled_video_to_pooled": (I, [P, P, P, P, I, I, I, I, I, I, P]),
            "stspix_graph_replays": (C.c_longlong, [P]),
            "stspix_set_batch_graphs": (I, [P, I]),
            "stspix_sweep_choice": (I, [P, I, C.POINTER(I), C.POINTER(I), C.POINTER(I)]),
            "stspix_legacy_update_prior": (I, [P, P, P, C.c_longlong, I, P, P, P, P, P, P, I,
                                               I]),
            "stspix_legacy_shift_tensor": (I, [P, P, P, P, P, I, I, I, I, I, P, P, P, P]),
            "stspix_legacy_shift_order": (I, [P, P, P, I, I, I, I, P]),
            "stspix_legacy_split_disconnected": (I, [P, P, P, I, I, I, P, P, C.c_longlong,
                                                     C.POINTER(I)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return _lib


class StspixError(RuntimeError):
    """A non-zero status returned by the engine."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"st_spix_gb300 error {code}: {msg}")
        self.code = code


class Context:
    """One engine context (device workspace) bound to a CUDA device."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        st = self.lib.stspix_create(C.byref(h), int(device))
        if st != 0:
            raise StspixError(st, f"stspix_create(device={device}) failed")
        self.handle = h
        self.device = device

    def check(self, st: int):
        if st != 0:
            msg = self.lib.stspix_last_error(self.handle)
            raise StspixError(st, msg.decode() if msg else "")

    def launches(self) -> int:
        return int(self.lib.stspix_kernel_launches(self.handle))

    def graph_replays(self) -> int:
        return int(self.lib.stspix_graph_replays(self.handle))

    def sweep_choices(self) -> list:
        """The autotuner's (tile-count class, single width, pair width or 0) entries."""
        out, i = [], 0
        a, b, c = C.c_int(0), C.c_int(0), C.c_int(0)
        while self.lib.stspix_sweep_choice(self.handle, i, C.byref(a), C.byref(b), C.byref(c)):
            out.append((a.value, b.value, c.value))
            i += 1
        return out

    def set_batch_graphs(self, enable: bool) -> None:
        self.check(self.lib.stspix_set_batch_graphs(self.handle, int(bool(enable))))

    def frame_log(self) -> FrameLog:
        lg = FrameLog()
        self.check(self.lib.stspix_get_frame_log(self.handle, C.byref(lg)))
        return lg

    def profile(self, enable: bool = True):
        self.check(self.lib.stspix_profile_enable(self.handle, int(bool(enable))))

    def profile_get(self) -> dict:
        out = {}
        for i, name in enumerate(FAMILIES):
            n, ms = C.c_longlong(0), C.c_double(0)
            self.check(self.lib.stspix_profile_get(self.handle, i, C.byref(n), C.byref(ms)))
            out[name] = (int(n.value), float(ms.value))
        return out

    def profile_kernels(self) -> dict:
        """Per-kernel (launches, total ms) of the profiled launches."""
        n = self.lib.stspix_profile_kernels(self.handle, None, 0)
        buf = C.create_string_buffer(max(n, 1))
        self.lib.stspix_profile_kernels(self.handle, buf, n)
        out = {}
        for ln in buf.value.decode().splitlines():
            name, cnt, ms = ln.split()
            out[name] = (int(cnt), float(ms))
        return out

    def frame_times(self) -> list:
        n = self.lib.stspix_frame_times(self.handle, None, 0)
        buf = (C.c_double * max(n, 1))()
        self.lib.stspix_frame_times(self.handle, buf, n)
        return [buf[i] for i in range(n)]

    def last_batch_ms(self) -> float:
        return float(self.lib.stspix_last_batch_ms(self.handle))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.stspix_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass


def default_config(**kw) -> Config:
    c = Config()
    load().stspix_default_config(C.byref(c))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise KeyError(k)
        setattr(c, k, v)
    return c


def footprint(H: int, W: int, sp_size: int) -> tuple:
    """(bytes resident per video stream, bytes per batch slot) on the device."""
    vb, sb = C.c_longlong(0), C.c_longlong(0)
    st = load().stspix_footprint(int(H), int(W), int(sp_size), C.byref(vb), C.byref(sb))
    if st != 0:
        raise StspixError(st, "stspix_footprint: bad size")
    return int(vb.value), int(sb.value)
