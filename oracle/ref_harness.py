"""ctypes binding of oracle/ref_harness.cpp (test infrastructure only): the
reference's own kernels, from the cubins in oracle/_ref, run on the GPU through the
CUDA driver API.  Available only where oracle/_ref was built (oracle/ref_build.py)
and a GPU is present."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
SRC = os.path.join(HERE, "ref_harness.cpp")
LIB = os.path.join(REF_DIR, "libref_harness.so")
_lib = None


def cubins_present() -> bool:
    need = ["update_seg", "seg_utils", "update_params", "init_seg", "split_merge",
            "fill_missing", "split_disconnected"]
    return (os.path.exists(os.path.join(REF_DIR, "spix_layout.h")) and
            all(os.path.exists(os.path.join(REF_DIR, n + ".cubin")) for n in need))


def build() -> str:
    """Compile the harness host code (needs the generated spix_layout.h)."""
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cuda = "/usr/local/cuda"
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + cuda + "/include",
                        "-I" + HERE, "-o", tmp, SRC, "-L" + cuda + "/lib64/stubs", "-lcuda"],
                       check=True)
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        P, I, F = C.c_void_p, C.c_int, C.c_float
        L.refh_error.restype = C.c_char_p
        L.refh_init.argtypes = [C.c_char_p]
        L.refh_find_border.argtypes = [P, P, I, I, I]
        L.refh_init_seg.argtypes = [I, I, I, P]
        L.refh_update_params.argtypes = [P, P, I, I, I, I, F, P, P, P, P, P, P, P, P, P, P, P]
        L.refh_update_seg.argtypes = [P, P, I, I, I, I, F, F, P, P, P, P, P]
        L.refh_split_bfs.argtypes = [P, I, I, I, P, P, I, I, P]
        L.refh_fill.argtypes = [P, P, I, I, I, I]
        L.refh_cc_roots.argtypes = [P, I, I, P]
        if L.refh_init(REF_DIR.encode()) != 0:
            raise RuntimeError("reference harness init failed: " + L.refh_error().decode())
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _check(r):
    if r < 0 and r != -2:
        raise RuntimeError(lib().refh_error().decode())
    return r


def find_border(labels, mode):
    labels = np.ascontiguousarray(labels, np.int32)
    out = np.zeros(labels.shape, np.uint8)
    _check(lib().refh_find_border(_p(labels), _p(out), labels.shape[0], labels.shape[1], mode))
    return out


def init_seg(H, W, sp_size):
    out = np.zeros((H, W), np.int32)
    n = _check(lib().refh_init_seg(H, W, sp_size, _p(out)))
    return out, n


def update_params(img, labels, nbuf, sp_size, sigma2_app, valid, prop, prior_count, prior_icov,
                  sample_sigma):
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
    _check(lib().refh_update_params(_p(img), _p(labels), H, W, nbuf, sp_size, sigma2_app,
                                    *[_p(a) for a in args], _p(out["count"]), _p(out["mu_app"]),
                                    _p(out["mu_shape"]), _p(out["sigma_shape"]),
                                    _p(out["logdet"]), _p(out["valid"])))
    return out


def update_seg(img, labels, nbuf, niters_seg, sigma2_app, potts, count, mu_app, mu_shape,
               sigma_shape, logdet):
    img = np.ascontiguousarray(img, np.float32)
    lab = np.array(labels, np.int32, copy=True)
    a = [np.ascontiguousarray(count, np.int32), np.ascontiguousarray(mu_app, np.float32),
         np.ascontiguousarray(mu_shape, np.float64), np.ascontiguousarray(sigma_shape, np.float64),
         np.ascontiguousarray(logdet, np.float64)]
    H, W = lab.shape
    _check(lib().refh_update_seg(_p(img), _p(lab), H, W, nbuf, niters_seg, sigma2_app, potts,
                                 *[_p(x) for x in a]))
    return lab


def split_bfs(labels, nbuf, valid, mu_shape, direction, max_spix):
    labels = np.ascontiguousarray(labels, np.int32)
    out = np.zeros(labels.shape, np.int32)
    H, W = labels.shape
    _check(lib().refh_split_bfs(_p(labels), H, W, nbuf, _p(np.ascontiguousarray(valid, np.int32)),
                                _p(np.ascontiguousarray(mu_shape, np.float64)), direction,
                                max_spix, _p(out)))
    return out


def fill(seg, centers, break_iter=1000):
    seg = np.array(seg, np.int32, copy=True)
    centers = np.ascontiguousarray(centers, np.float64)
    r = _check(lib().refh_fill(_p(seg), _p(centers), centers.shape[0], seg.shape[0], seg.shape[1],
                               break_iter))
    return r, seg


def cc_roots(seg):
    seg = np.ascontiguousarray(seg, np.int32)
    out = np.zeros(seg.shape, np.int32)
    _check(lib().refh_cc_roots(_p(seg), seg.shape[0], seg.shape[1], _p(out)))
    return out


def rgb2lab(rgb):
    """The reference's rgb_to_lab kernel on a copy of `rgb` (f32 [...,3])."""
    rgb = np.ascontiguousarray(rgb, np.float32)
    out = np.empty_like(rgb)
    _check(lib().refh_color(0, _p(rgb), _p(out), rgb.size // 3))
    return out


def lab2rgb(lab):
    """The reference's lab_to_rgb kernel (writes the RGB image from a LAB image)."""
    lab = np.ascontiguousarray(lab, np.float32)
    out = np.empty_like(lab)
    _check(lib().refh_color(1, _p(lab), _p(out), lab.size // 3))
    return out


def rescale_u8(img, mval=255.0):
    img = np.ascontiguousarray(img, np.uint8)
    out = np.empty(img.shape, np.float32)
    _check(lib().refh_rescale(_p(img), _p(out), img.size // 3, C.c_float(mval)))
    return out
