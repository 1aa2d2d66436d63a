"""ORACLE -- test infrastructure only: the reference's whole bist_forward path, run on
the GPU host with the reference's OWN kernels.

The kernels are the cubins oracle/ref_build.py compiles from the unmodified reference
sources (oracle/_ref: -fmad=false; oracle/_ref/stock: nvcc's default contraction, as
the reference's setup.py builds them), launched through oracle/ref_harness.cpp's
generic layer.  The reference's host drivers cannot be compiled for the GPU host (its
sources are not there), so this module restates them in Python, launch for launch,
with the same grids (512-thread blocks), arguments, memsets and host loops:

  bist_forward / main_loop       st_spix/csrc/bist/pyapi.cu:46-215
  run_bass / bass                bass.cu:221-345 / bass.cu:46-181
  shift_and_fill                 shift_and_fill.cu:108-339
  run_prop / prop_bass_v3        prop.cu:677-865 / prop.cu:326-468
  split / merge (BASS)           split_merge_orig.cu:26-414
  split / merge (propagated)     split_merge_prop.cu:31-395
  relabel_spix                   relabel.cu:279-409
  compactify / unique ids        compact_spix.cu:41-138, seg_utils.cu:22-43
  update_params, summaries       update_params.cu:12-52, 385-395
  init_sp_params, mark_active    init_sparams.cu:25-43, 225-290
  parameter I/O, prior update    sparams_io.cu:65-79, 123-326, 642-688
  update_seg, borders            update_seg.cu:281-311, seg_utils.cu:156-216
  init_seg                       init_seg.cu:20-46
  run_sp_downsample              sp_pooling.cu:121-147
  run_shift_labels               shift_labels.cu:175-239
  run_fill_missing               fill_missing.cu:35-130, 656-669
  run_invalidate_disconnected    split_disconnected.cu:33-185
  get_spix_counts                seg_utils.cu:104-135

Thrust steps (sort, unique, copy_if, count, transform, scatter, gather) run on the
host with numpy: they only order, select and combine values (the one arithmetic
transform, shift_and_fill.cu:147-149 and :277-316, is restated with the same IEEE
operations), so every kernel sees the inputs the reference's would.  Where the
reference reads memory it never wrote (easy_allocate, init_utils.cu:26, does not
clear), the allocation starts zeroed here; run_update_prior's id list, which the
reference reads past its size (prop.cu:839-841), is padded with -1.  The reference's
exit(1) paths (fill_missing.cu:97-111, split_merge_orig.cu:334) raise RefError.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
import struct

import numpy as np

from oracle import ref_harness as RH

UNITS = ["update_seg", "seg_utils", "update_params", "init_seg", "split_merge",
         "fill_missing", "split_disconnected", "split_merge_orig", "split_merge_prop",
         "relabel", "shift_labels", "sp_pooling", "init_sparams", "sparams_io",
         "compact_spix"]
TPB = 512  # THREADS_PER_BLOCK in every reference unit
_libm = C.CDLL(None)
_libm.expf.restype = C.c_float
_libm.expf.argtypes = [C.c_float]
_libm.sqrtf.restype = C.c_float
_libm.sqrtf.argtypes = [C.c_float]


class RefError(RuntimeError):
    pass


def nblk(n: int) -> int:
    return (int(n) + TPB - 1) // TPB


def f32(x) -> float:
    return float(np.float32(x))


def variant_dir(variant: str) -> str:
    return RH.REF_DIR if variant == "nofma" else os.path.join(RH.REF_DIR, variant)


def available(variant: str = "nofma") -> bool:
    d = variant_dir(variant)
    return (RH.cubins_present() and os.path.exists(os.path.join(RH.REF_DIR, "spix_layout.json"))
            and all(os.path.exists(os.path.join(d, u + ".cubin")) for u in UNITS))


# kernel argument kinds: each occupies one 8-byte slot
def P(x):
    return ("Q", x.p if isinstance(x, Buf) else int(x))


def I(x):
    return ("i", int(x))


def F(x):
    return ("f", float(x))


def B(x):
    return ("?", bool(x))


class Buf:
    __slots__ = ("p", "n")

    def __init__(self, p, n):
        self.p, self.n = p, n


class Params:
    """SuperpixelParams (structs.h:13-48) as device arrays of `size` entries."""
    FIELDS = [("mu_app", np.float32, 3), ("prior_mu_app", np.float32, 3),
              ("mu_shape", np.float64, 2), ("sigma_shape", np.float64, 3),
              ("logdet_sigma_shape", np.float32, 1), ("prior_mu_shape", np.float64, 2),
              ("prior_sigma_shape", np.float64, 3), ("sample_sigma_shape", np.float64, 3),
              ("counts", np.int32, 1), ("sm_counts", np.int32, 1),
              ("prior_counts", np.float32, 1), ("ids", np.int32, 1),
              ("invalid_counts", np.float32, 1)]

    def __init__(self, ref: "Ref", size: int):
        self.size = size
        for name, dt, k in self.FIELDS:
            setattr(self, name, ref.zeros(size * k * np.dtype(dt).itemsize))

    def host(self, ref: "Ref") -> dict:
        return {name: ref.d2h(getattr(self, name), dt, self.size * k)
                for name, dt, k in self.FIELDS}

    def free(self, ref: "Ref"):
        for name, _, _ in self.FIELDS:
            ref.free(getattr(self, name))


class Ref:
    """One build variant of the reference kernels ("nofma" or "stock")."""

    def __init__(self, variant: str = "nofma"):
        if not available(variant):
            raise RefError("oracle/_ref cubins for variant %r not built" % variant)
        L = RH.lib()
        V, P_, U64 = C.c_void_p, C.c_char_p, C.c_ulonglong
        L.refh_variant_load.argtypes = [P_, P_]
        L.refh_fn.argtypes = [C.c_int, P_, P_, P_]
        L.refh_fn_name.restype = C.c_char_p
        L.refh_malloc.restype = U64
        L.refh_malloc.argtypes = [U64]
        L.refh_free.argtypes = [U64]
        L.refh_memset8.argtypes = [U64, C.c_uint, U64]
        L.refh_memset32.argtypes = [U64, C.c_uint, U64]
        L.refh_h2d.argtypes = [U64, V, U64]
        L.refh_d2h.argtypes = [V, U64, U64]
        L.refh_d2d.argtypes = [U64, U64, U64]
        L.refh_launch.argtypes = [C.c_int, C.c_uint, C.c_uint, C.c_uint, V, C.c_int]
        L.refh_event_record.argtypes = [C.c_int]
        L.refh_event_ms.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_float)]
        self.L = L
        self.variant = variant
        self.var = self._ck(L.refh_variant_load(variant_dir(variant).encode(),
                                                ",".join(UNITS).encode()))
        lay = json.load(open(os.path.join(RH.REF_DIR, "spix_layout.json")))
        self.lay = lay
        self.SP, self.HELPER = lay["REF_SP_SIZE"], lay["REF_HELPER_SIZE"]
        self.SM, self.SM2 = lay["REF_SM_SIZE"], lay["REF_SM2_SIZE"]
        self._fns = {}
        self.log = []        # (event, value) records of the last run

    # -- plumbing ---------------------------------------------------------------
    def _ck(self, r):
        if r < 0:
            raise RefError(self.L.refh_error().decode())
        return r

    def fn(self, module, name, mangled=""):
        key = (module, name, mangled)
        if key not in self._fns:
            self._fns[key] = self._ck(self.L.refh_fn(self.var, module.encode(), name.encode(),
                                                     mangled.encode()))
        return self._fns[key]

    def launch(self, module, name, grid, args, mangled=""):
        h = self.fn(module, name, mangled)
        slots = (C.c_ulonglong * max(1, len(args)))()
        for i, (fmt, v) in enumerate(args):
            struct.pack_into("<" + fmt, slots, 8 * i, v)
        self._ck(self.L.refh_launch(h, grid, 1, TPB, slots, len(args)))

    def alloc(self, nbytes: int) -> Buf:
        p = self.L.refh_malloc(max(16, int(nbytes)))
        if not p:
            raise RefError("device allocation of %d bytes failed" % nbytes)
        return Buf(p, int(nbytes))

    def zeros(self, nbytes: int) -> Buf:
        b = self.alloc(nbytes)
        self._ck(self.L.refh_memset8(b.p, 0, max(16, int(nbytes))))
        return b

    def free(self, b: Buf):
        if b is not None and b.p:
            self._ck(self.L.refh_free(b.p))
            b.p = 0

    def memset8(self, b: Buf, v: int, n: int):
        self._ck(self.L.refh_memset8(b.p, v & 0xFF, n))

    def memset32(self, b: Buf, v: int, n: int):
        self._ck(self.L.refh_memset32(b.p, v & 0xFFFFFFFF, n))

    def h2d(self, a: np.ndarray) -> Buf:
        a = np.ascontiguousarray(a)
        b = self.alloc(a.nbytes)
        if a.nbytes:
            self._ck(self.L.refh_h2d(b.p, a.ctypes.data_as(C.c_void_p), a.nbytes))
        return b

    def upload(self, b: Buf, a: np.ndarray):
        a = np.ascontiguousarray(a)
        if a.nbytes:
            self._ck(self.L.refh_h2d(b.p, a.ctypes.data_as(C.c_void_p), a.nbytes))

    def d2h(self, b: Buf, dtype, count: int) -> np.ndarray:
        out = np.empty(int(count), dtype)
        if out.nbytes:
            self._ck(self.L.refh_d2h(out.ctypes.data_as(C.c_void_p), b.p, out.nbytes))
        return out

    def d2d(self, dst: Buf, src: Buf, nbytes: int):
        self._ck(self.L.refh_d2d(dst.p, src.p, nbytes))

    def int_at(self, b: Buf) -> int:
        return int(self.d2h(b, np.int32, 1)[0])

    def sync(self):
        self._ck(self.L.refh_sync())

    # -- thrust steps on the host ----------------------------------------------------
    def labels(self, seg: Buf, npix: int) -> np.ndarray:
        return self.d2h(seg, np.int32, npix)

    def get_unique(self, seg, npix):                      # seg_utils.cu:22-36
        return np.unique(self.labels(seg, npix)).astype(np.int32)

    def extract_unique_ids(self, seg, npix, prev_nspix):  # compact_spix.cu:93-122
        u = self.get_unique(seg, npix)
        return u[u >= prev_nspix]

    # -- seg_utils / update_params / init ---------------------------------------------
    def find_border(self, seg, border, npix, W, H):       # seg_utils.cu:156-163
        self.launch("seg_utils", "find_border_pixels", nblk(npix),
                    [P(seg), P(border), I(npix), I(W), I(H)])

    def find_border_end(self, seg, border, npix, W, H):   # seg_utils.cu:209-216
        self.launch("seg_utils", "find_border_pixels_end", nblk(npix),
                    [P(seg), P(border), I(npix), I(W), I(H)])

    def update_params(self, img, seg, sp, helper, sigma2_app, npix, sp_size, nbuf, W):
        # update_params.cu:12-31
        self.launch("update_params", "clear_fields", nblk(nbuf), [P(sp), P(helper), I(nbuf), I(3)])
        self.memset8(helper, 0, nbuf * self.HELPER)
        self.launch("update_params", "sum_by_label", nblk(npix),
                    [P(img), P(seg), P(sp), P(helper), I(npix), I(1), I(W), I(3)])
        self.launch("update_params", "calc_simple_update", nblk(nbuf),
                    [P(sp), P(helper), F(sigma2_app), I(sp_size), I(nbuf)])

    def update_params_summ(self, img, seg, sp, helper, sigma_app, npix, nbuf, W):
        # update_params.cu:34-52
        self.launch("update_params", "clear_fields", nblk(nbuf), [P(sp), P(helper), I(nbuf), I(3)])
        self.memset8(helper, 0, nbuf * self.HELPER)
        self.launch("update_params", "sum_by_label", nblk(npix),
                    [P(img), P(seg), P(sp), P(helper), I(npix), I(1), I(W), I(3)])
        self.launch("update_params", "calc_summ_stats", nblk(nbuf),
                    [P(sp), P(helper), F(sigma_app), I(nbuf)])

    def store_sample_sigma_shape(self, sp, helper, sp_size, nbuf):
        # update_params.cu:385-395 (sp_size is passed to the kernel's float parameter)
        self.launch("update_params", "store_sample_sigma_shape_k", nblk(nbuf),
                    [P(sp), P(helper), F(float(sp_size)), I(nbuf)])

    def init_sp_params(self, sp, sigma2_app, img, seg, helper, npix, nspix, nbuf, W, sp_size):
        # init_sparams.cu:25-43
        self.update_params_summ(img, seg, sp, helper, sigma2_app, npix, nbuf, W)
        self.launch("init_sparams", "init_sp_params_kernel", nblk(nbuf),
                    [P(sp), F(sigma2_app), I(nspix), I(nbuf), I(npix), I(sp_size)])

    def mark_active(self, sp, ids: np.ndarray, nspix, nbuf, sp_size):
        # init_sparams.cu:234-290
        nvalid = self.zeros(4)
        self.launch("init_sparams", "mark_inactive_kernel", nblk(nbuf),
                    [P(sp), I(nbuf), P(nvalid), I(nspix), I(sp_size)])
        self.memset8(nvalid, 0, 4)
        dids = self.h2d(ids.astype(np.int32))
        self.launch("init_sparams", "mark_active_kernel", nblk(len(ids)),
                    [P(sp), P(dids), I(len(ids)), I(nspix), I(nbuf), P(nvalid)])
        self.free(dids)
        self.free(nvalid)

    def init_seg(self, seg, sp_size, W, H):
        # init_seg.cu:20-46
        npix = H * W
        hh = math.sqrt(float(sp_size) ** 2 / (1.5 * math.sqrt(3.0)))
        w = math.sqrt(3.0) * hh
        nx = int(math.floor(W / w)) + 2
        ny = int(math.floor(H / (1.5 * hh))) + 2
        nspix = nx * ny
        centers = self.zeros(16 * nspix)
        self.launch("init_seg", "InitHexCenter", nblk(nspix),
                    [P(centers), ("d", hh), ("d", w), I(nspix), I(nx), I(W), I(H)])
        self.launch("init_seg", "InitHexSeg", nblk(npix),
                    [P(seg), P(centers), I(nspix), I(npix), I(W)])
        self.free(centers)
        return nspix

    def update_seg(self, img, seg, border, sp, niters, sigma2_app, potts, npix, W, H):
        # update_seg.cu:281-311
        for _ in range(niters):
            self.memset8(border, 0, npix)
            self.find_border(seg, border, npix, W, H)
            for xm in range(2):
                for ym in range(2):
                    self.launch("update_seg", "update_seg_subset", nblk(npix),
                                [P(img), P(seg), P(border), P(sp), F(sigma2_app), F(potts),
                                 I(npix), I(1), I(W), I(H), I(3), I(xm), I(ym)])
        self.memset8(border, 0, npix)
        self.find_border(seg, border, npix, W, H)

    # -- compaction and parameter I/O ------------------------------------------------
    def compactify(self, seg, sp, prop_ids: np.ndarray, prev_nspix, npix):
        # compact_spix.cu:41-89
        num_new = int(len(prop_ids))
        if num_new == 0:
            return prev_nspix
        new_params = self.zeros(num_new * self.SP)
        cmap = self.zeros(4 * num_new)
        pid = self.h2d(prop_ids.astype(np.int32))
        self.launch("compact_spix", "compact_new_spix", nblk(npix),
                    [P(seg), P(cmap), P(pid), I(num_new), I(prev_nspix), I(npix)])
        self.launch("compact_spix", "fill_new_params_from_old", nblk(num_new),
                    [P(sp), P(new_params), P(cmap), I(num_new)])
        self.launch("compact_spix", "fill_old_params_from_new", nblk(num_new),
                    [P(sp), P(new_params), I(prev_nspix), I(num_new)])
        for b in (new_params, cmap, pid):
            self.free(b)
        return prev_nspix + num_new

    def get_params_as_vectors(self, sp, num_ids, nspix) -> Params:
        # sparams_io.cu:65-79 + params_to_vectors :142-187 (read_params ignores `ids`)
        pr = Params(self, nspix)
        self.upload(pr.ids, np.arange(num_ids, dtype=np.int32)[:nspix])
        self.launch("sparams_io", "read_params", nblk(num_ids),
                    [P(pr.mu_app), P(pr.prior_mu_app), P(pr.mu_shape), P(pr.sigma_shape),
                     P(pr.logdet_sigma_shape), P(pr.prior_mu_shape), P(pr.prior_sigma_shape),
                     P(pr.sample_sigma_shape), P(pr.counts), P(pr.invalid_counts),
                     P(pr.sm_counts), P(pr.prior_counts), P(sp), P(pr.ids), I(num_ids)])
        return pr

    def run_update_prior(self, pr: Params, uniq: np.ndarray, nspix, prev_nspix):
        # sparams_io.cu:642-688, invert = false
        ids = np.full(max(nspix, len(uniq)), -1, np.int32)
        ids[:len(uniq)] = uniq
        dids = self.h2d(ids)
        self.launch("sparams_io", "update_prior_kernel", nblk(nspix),
                    [P(pr.mu_app), P(pr.prior_mu_app), P(pr.mu_shape), P(pr.prior_mu_shape),
                     P(pr.sigma_shape), P(pr.prior_sigma_shape), P(pr.sample_sigma_shape),
                     P(pr.counts), P(dids), I(nspix), I(prev_nspix), B(False)])
        self.free(dids)

    def get_vectors_as_params(self, pr: Params, nbuf):
        # sparams_io.cu:123-140 + vectors_to_params :289-326
        sp = self.zeros(nbuf * self.SP)
        self.launch("sparams_io", "write_params", nblk(pr.size),
                    [P(pr.mu_app), P(pr.prior_mu_app), P(pr.mu_shape), P(pr.sigma_shape),
                     P(pr.logdet_sigma_shape), P(pr.prior_mu_shape), P(pr.prior_sigma_shape),
                     P(pr.sample_sigma_shape), P(pr.counts), P(pr.invalid_counts),
                     P(pr.sm_counts), P(pr.prior_counts), P(sp), I(pr.size)])
        return sp

    # -- split / merge ----------------------------------------------------------------
    def _sm_consts(self, sigma2_app):
        # a_0 = 1e4, i_std = sqrt(sigma2_app)*2, b_0 = i_std*a_0, all FP32 host floats
        a_0 = f32(1e4)
        i_std = f32(_libm.sqrtf(f32(sigma2_app)) * np.float32(2))
        b_0 = f32(np.float32(i_std) * np.float32(a_0))
        return a_0, b_0

    def _bfs(self, module, name, dist, seg, border, done, npix, W, H, read_first):
        distance, flag, steps = 1, 1, 0
        while flag:
            self.memset8(done, 0, 4)
            if read_first:
                flag = self.int_at(done)
            self.launch(module, name, nblk(npix),
                        [P(dist), P(seg), P(border), I(distance), P(done), I(npix), I(1),
                         I(W), I(H)])
            distance += 1
            flag = self.int_at(done)
            steps += 1
            if distance > 5005:                        # split_merge_orig.cu:333-335
                raise RefError("split BFS did not finish")
        return steps

    def split_orig(self, S, max_spix, direction, log_alpha, split_alpha):
        # CudaCalcSplitCandidate_orig, split_merge_orig.cu:202-414
        nbuf, npix, W, H = S["nbuf"], S["npix"], S["W"], S["H"]
        if max_spix > nbuf // 2:
            return max_spix
        a_0, b_0 = self._sm_consts(S["sigma2_app"])
        alpha = f32(_libm.expf(f32(log_alpha)))
        nvalid, max_sp, done = self.zeros(4), self.zeros(4), self.zeros(4)
        img, seg, border, sp = S["img"], S["seg"], S["border"], S["sp"]
        helper, smh, seg1, seg2, pairs = S["helper"], S["smh"], S["seg1"], S["seg2"], S["pairs"]
        self.memset8(seg1, 0xFF, 4 * npix)
        self.memset8(seg2, 0xFF, 4 * npix)
        self.launch("split_merge", "init_sm", nblk(nbuf),
                    [P(img), P(seg), P(sp), P(smh), I(nbuf), I(1), I(W), I(3), I(npix), P(pairs),
                     P(nvalid)])
        self.int_at(nvalid)
        for d, tgt in ((direction, seg1), (-direction, seg2)):
            self.launch("split_merge", "init_split", nblk(nbuf),
                        [P(border), P(tgt), P(sp), I(nbuf), I(1), I(W), I(H), I(d), P(seg),
                         P(max_sp), I(max_spix)])
        split_sp = [P(seg), P(seg1), P(pairs), P(sp), P(smh), I(npix), I(1), I(W), I(H),
                    I(max_spix)]
        self.launch("split_merge", "split_sp", nblk(npix), split_sp)
        self._bfs("split_merge", "calc_split_candidate", seg1, seg, border, done, npix, W, H, False)
        self._bfs("split_merge", "calc_split_candidate", seg2, seg, border, done, npix, W, H, True)
        self.launch("split_merge", "calc_seg_split", nblk(npix),
                    [P(seg1), P(seg2), P(seg), I(npix), I(1), I(max_spix)])
        self.launch("split_merge", "sum_by_label", nblk(npix),
                    [P(img), P(seg1), P(sp), P(smh), I(npix), I(1), I(W), I(3)])
        self.launch("split_merge_orig", "calc_split_stats_step0", nblk(nbuf),
                    [P(sp), P(helper), P(smh), I(nbuf), F(b_0), I(max_spix)])
        self.launch("split_merge_orig", "calc_split_stats_step1", nblk(nbuf),
                    [P(sp), P(helper), P(smh), I(nbuf), F(a_0), F(b_0), I(max_spix)])
        self.launch("split_merge_orig", "update_split_flag", nblk(nbuf),
                    [P(pairs), P(sp), P(smh), I(nbuf), F(alpha), F(split_alpha), I(max_spix),
                     P(max_sp)])
        if S.get("decision_hook"):
            S["decision_hook"]("split", max_spix)
        self.launch("split_merge", "split_sp", nblk(npix), split_sp)
        new_max = self.int_at(max_sp)
        for b in (nvalid, max_sp, done):
            self.free(b)
        self.log.append(("split", new_max - max_spix))
        return new_max

    def merge_orig(self, S, direction, log_alpha, alpha_merge):
        # CudaCalcMergeCandidate_orig, split_merge_orig.cu:79-199
        nbuf, npix, W, H = S["nbuf"], S["npix"], S["W"], S["H"]
        a_0, b_0 = self._sm_consts(S["sigma2_app"])
        alpha = f32(_libm.expf(f32(log_alpha)))
        nvalid, nmerges = self.zeros(4), self.zeros(4)
        img, seg, border, sp = S["img"], S["seg"], S["border"], S["sp"]
        helper, smh, pairs = S["helper"], S["smh"], S["pairs"]
        self.launch("split_merge", "init_sm", nblk(nbuf),
                    [P(img), P(seg), P(sp), P(smh), I(nbuf), I(1), I(W), I(3), I(npix), P(pairs),
                     P(nvalid)])
        self.launch("split_merge", "calc_merge_candidate", nblk(npix),
                    [P(seg), P(border), P(pairs), I(npix), I(1), I(W), I(H), I(direction)])
        self.launch("split_merge", "sum_by_label", nblk(npix),
                    [P(img), P(seg), P(sp), P(smh), I(npix), I(1), I(W), I(3)])
        self.launch("split_merge_orig", "calc_merge_stats_step0", nblk(nbuf),
                    [P(pairs), P(sp), P(helper), P(smh), I(nbuf), F(b_0)])
        self.launch("split_merge_orig", "calc_merge_stats_step1", nblk(nbuf),
                    [P(sp), P(smh), I(nbuf), F(a_0), F(b_0)])
        self.launch("split_merge_orig", "calc_merge_stats_step2", nblk(nbuf),
                    [P(pairs), P(sp), P(smh), I(nbuf), F(alpha), F(alpha_merge)])
        self.launch("split_merge_orig", "update_merge_flag", nblk(nbuf),
                    [P(pairs), P(sp), P(smh), I(nbuf), P(nmerges)])
        if S.get("decision_hook"):
            S["decision_hook"]("merge", None)
        self.launch("split_merge", "remove_sp", nblk(nbuf), [P(pairs), P(sp), P(smh), I(nbuf)])
        self.launch("split_merge", "merge_sp", nblk(npix),
                    [P(seg), P(border), P(pairs), P(sp), P(smh), I(npix), I(1), I(W), I(H)])
        self.free(nvalid)
        self.free(nmerges)

    def split_p(self, S, max_spix, direction, alpha, split_alpha):
        # CudaCalcSplitCandidate_p, split_merge_prop.cu:184-395 (alpha = log alpha as passed)
        nbuf, npix, W, H = S["nbuf"], S["npix"], S["W"], S["H"]
        if max_spix > nbuf // 2:
            return max_spix
        a_0, b_0 = self._sm_consts(S["sigma2_app"])
        done, max_sp, nvalid = self.zeros(4), self.zeros(4), self.zeros(4)
        count_rules = self.zeros(40)
        img, seg, border, sp, shifted = S["img"], S["seg"], S["border"], S["sp"], S["shifted"]
        helper, smh, seg1, seg2, pairs = S["helper"], S["smh"], S["seg1"], S["seg2"], S["pairs"]
        self.memset8(seg1, 0xFF, 4 * npix)
        self.memset8(seg2, 0xFF, 4 * npix)
        self.memset8(nvalid, 0, 4)
        self.launch("split_merge_prop", "init_sm_p", nblk(nbuf),
                    [P(img), P(seg), P(sp), P(smh), I(nbuf), I(1), I(H), I(W), I(3), I(npix),
                     P(pairs), P(nvalid)])
        for d, tgt in ((direction, seg1), (-direction, seg2)):
            self.launch("split_merge_prop", "init_split_p", nblk(nbuf),
                        [P(border), P(tgt), P(sp), P(smh), I(nbuf), I(1), I(W), I(H), I(d),
                         P(seg), P(max_sp), I(max_spix)])
        split_sp = [P(seg), P(seg1), P(pairs), P(sp), P(smh), I(npix), I(1), I(W), I(H),
                    I(max_spix)]
        self.launch("split_merge_prop", "split_sp_p", nblk(npix), split_sp)
        self._bfs("split_merge_prop", "calc_split_candidate_p", seg1, seg, border, done, npix, W,
                  H, True)
        self._bfs("split_merge_prop", "calc_split_candidate_p", seg2, seg, border, done, npix, W,
                  H, True)
        self.launch("split_merge_prop", "calc_seg_split_p", nblk(npix),
                    [P(seg1), P(seg2), P(seg), I(npix), I(1), I(max_spix)])
        self.launch("split_merge_prop", "sum_by_label_split_p", nblk(npix),
                    [P(img), P(seg1), P(shifted), P(sp), P(smh), I(npix), I(1), I(H), I(W), I(3),
                     I(max_spix)])
        self.launch("split_merge_prop", "calc_split_stats_step0_p", nblk(nbuf),
                    [P(sp), P(helper), P(smh), I(nbuf), F(b_0), I(max_spix)])
        self.launch("split_merge_prop", "calc_split_stats_step1_p", nblk(nbuf),
                    [P(sp), P(helper), P(smh), I(nbuf), F(a_0), F(b_0), I(max_spix)])
        self.launch("split_merge_prop", "update_split_flag_p", nblk(nbuf),
                    [P(pairs), P(sp), P(smh), I(nbuf), F(alpha), F(split_alpha), I(S["sp_size"]),
                     I(max_spix), P(max_sp)])
        if S.get("decision_hook"):
            S["decision_hook"]("split_p", max_spix)
        self.launch("split_merge_prop", "split_sp_p", nblk(npix), split_sp)
        new_max = self.int_at(max_sp)
        for b in (done, max_sp, nvalid, count_rules):
            self.free(b)
        self.log.append(("split", new_max - max_spix))
        return new_max

    def merge_p(self, S, direction, log_alpha, merge_alpha):
        # CudaCalcMergeCandidate_p, split_merge_prop.cu:87-181
        nbuf, npix, W, H = S["nbuf"], S["npix"], S["W"], S["H"]
        a_0, b_0 = self._sm_consts(S["sigma2_app"])
        alpha = f32(_libm.expf(f32(log_alpha)))
        nvalid, nmerges = self.zeros(4), self.zeros(4)
        img, seg, border, sp = S["img"], S["seg"], S["border"], S["sp"]
        helper, smh, pairs = S["helper"], S["smh"], S["pairs"]
        self.launch("split_merge_prop", "init_sm_p", nblk(nbuf),
                    [P(img), P(seg), P(sp), P(smh), I(nbuf), I(1), I(H), I(W), I(3), I(npix),
                     P(pairs), P(nvalid)])
        self.launch("split_merge_prop", "calc_merge_candidate_p", nblk(npix),
                    [P(seg), P(border), P(pairs), P(sp), I(npix), I(1), I(W), I(H), I(direction)])
        self.launch("split_merge_prop", "sum_by_label_merge_p", nblk(npix),
                    [P(img), P(seg), P(sp), P(smh), I(npix), I(1), I(W), I(3)])
        self.launch("split_merge_prop", "calc_merge_stats_step0_p", nblk(nbuf),
                    [P(pairs), P(sp), P(helper), P(smh), I(nbuf), F(b_0)])
        self.launch("split_merge_prop", "calc_merge_stats_step1_p", nblk(nbuf),
                    [P(sp), P(smh), I(nbuf), F(a_0), F(b_0)])
        self.launch("split_merge_prop", "calc_merge_stats_step2_p", nblk(nbuf),
                    [P(pairs), P(sp), P(smh), I(nbuf), F(alpha), F(merge_alpha)])
        self.launch("split_merge_prop", "update_merge_flag_p", nblk(nbuf),
                    [P(pairs), P(sp), P(smh), I(nbuf), P(nmerges)])
        if S.get("decision_hook"):
            S["decision_hook"]("merge_p", None)
        self.launch("split_merge_prop", "remove_sp_p", nblk(nbuf),
                    [P(pairs), P(sp), P(smh), I(nbuf), P(nmerges)])
        self.launch("split_merge_prop", "merge_sp_p", nblk(npix),
                    [P(seg), P(border), P(pairs), P(sp), P(smh), I(npix), I(1), I(W), I(H)])
        self.free(nvalid)
        self.free(nmerges)

    # -- relabel ----------------------------------------------------------------------
    def relabel_spix(self, S, prev: Params, living: np.ndarray, thresh_replace, thresh_new,
                     nspix_prev, max_spix_in):
        # relabel.cu:279-409
        seg, sp, npix, W, H = S["seg"], S["sp"], S["npix"], S["W"], S["H"]
        nspix = max_spix_in + 1
        mx = self.h2d(np.array([max_spix_in], np.int32))
        is_living = np.zeros(nspix, np.uint8)
        is_living[living] = 1
        dliving = self.h2d(is_living)
        ss = self.zeros(4 * nspix)
        comps = self.zeros(8 * nspix)
        self.memset32(comps, struct.unpack("<I", struct.pack("<f", 10000.0))[0], 2 * nspix)
        ntotal = nspix * nspix_prev
        self.launch("relabel", "find_most_similar_spix", nblk(ntotal),
                    [P(comps), P(ss), P(sp), P(prev.prior_mu_app), P(prev.prior_mu_shape),
                     P(dliving), I(H), I(W), I(nspix), I(nspix_prev), I(ntotal)])
        relabel = self.zeros(nspix)
        relabel_id = self.zeros(4 * nspix)
        self.launch("relabel", "mark_for_relabel", nblk(nspix),
                    [P(relabel), P(relabel_id), P(comps), P(ss), P(dliving), P(mx), I(nspix),
                     I(nspix_prev), F(thresh_replace), F(thresh_new)])
        max_spix = self.int_at(mx)
        flags = self.d2h(relabel, np.uint8, nspix)
        self.log.append(("relabel", int(flags.sum()), max_spix - max_spix_in))
        if S.get("relabel_hook"):
            rid = self.d2h(relabel_id, np.int32, nspix)
            S["relabel_hook"](self.labels(seg, npix).reshape(H, W),
                              np.where(flags > 0, rid, -1).astype(np.int32), nspix_prev)
        self.launch("relabel", "relabel_spix_kernel", nblk(npix),
                    [P(seg), P(sp), P(relabel), P(relabel_id), I(npix), I(nspix), I(nspix_prev)])
        dl = self.h2d(living.astype(np.int32))
        self.launch("relabel", "relabel_living_kernel", nblk(len(living)),
                    [P(dl), P(relabel), P(relabel_id), I(len(living))])
        for b in (mx, dliving, ss, comps, relabel, relabel_id, dl):
            self.free(b)
        return max_spix

    # -- decision stages on a given state ------------------------------------------------
    def pack_sp(self, nbuf, **fields) -> np.ndarray:
        """Host image of nbuf spix_params (structs.h:71-106) with the named fields set
        (valid int, prior_count float, prop bool, prior_icov / prior_sigma_shape /
        sample_sigma_shape 3 doubles each); every other byte zero."""
        kinds = {"valid": (np.int32, 1), "prior_count": (np.float32, 1), "prop": (np.bool_, 1),
                 "prior_icov": (np.float64, 3), "prior_sigma_shape": (np.float64, 3),
                 "sample_sigma_shape": (np.float64, 3), "count": (np.int32, 1)}
        buf = np.zeros(nbuf * self.SP, np.uint8)
        for name, val in fields.items():
            dt, k = kinds[name]
            dt = np.dtype(dt)
            view = np.ndarray((nbuf, k), dt, buffer=buf, offset=self.lay["REF_OFF_" + name],
                              strides=(self.SP, dt.itemsize))
            view[...] = np.asarray(val, dt).reshape(nbuf, k)
        return buf

    def sm_step(self, img, labels, nbuf, valid, prior_count, prop, sample_sigma, max_spix, kind,
                direction, shifted, sp_size, sigma2_app, log_alpha, split_alpha, merge_alpha):
        """One split (kind 0: BASS, 2: propagated) or merge (kind 1 / 3) step of the
        reference on a given state, preceded by its update_params and the border pass
        update_seg leaves (update_seg.cu:309-310).  Returns per id the FP32 Hastings
        log-ratio as the reference stores it (its init value where it scores none),
        the merge flag after the decision kernel, the merge candidates and the labels
        after the step."""
        H, W = labels.shape
        npix = H * W
        dimg = self.h2d(np.ascontiguousarray(img, np.float32))
        seg = self.h2d(np.ascontiguousarray(labels, np.int32))
        icov = np.tile(np.array([1.0, 0.0, 1.0]), nbuf)
        psig = np.tile(np.array([1.0 / sp_size, 0.0, 1.0 / sp_size]), nbuf)
        host = self.pack_sp(nbuf, valid=valid, prior_count=prior_count, prop=prop,
                            prior_icov=icov, prior_sigma_shape=psig,
                            sample_sigma_shape=sample_sigma)
        smsize = self.SM if kind in (0, 1) else self.SM2
        S = self._state(dimg, seg, npix, W, H, nbuf, sigma2_app, sp_size, 2 * max(npix, nbuf),
                        smsize)
        S["sp"] = self.h2d(host)
        S["shifted"] = self.h2d(np.ascontiguousarray(
            shifted if shifted is not None else np.zeros((H, W)), np.int32))
        self.update_params(dimg, seg, S["sp"], S["helper"], sigma2_app, npix, sp_size, nbuf, W)
        self.memset8(S["border"], 0, npix)
        self.find_border(seg, S["border"], npix, W, H)
        got = {}

        def hook(_event, _mx):
            raw = self.d2h(S["smh"], np.uint8, nbuf * smsize)
            pre = "REF_SMOFF_" if smsize == self.SM else "REF_SM2OFF_"
            got["h"] = np.ndarray((nbuf,), np.float32, buffer=raw,
                                  offset=self.lay[pre + "hasting"], strides=(smsize,)).copy()
            got["merge"] = np.ndarray((nbuf,), np.uint8, buffer=raw,
                                      offset=self.lay[pre + "merge"], strides=(smsize,)).copy()
            got["pair"] = self.d2h(S["pairs"], np.int32, 2 * nbuf)[1::2].copy()
        S["decision_hook"] = hook
        if kind == 0:
            mx = self.split_orig(S, max_spix, direction, log_alpha, split_alpha)
        elif kind == 1:
            self.merge_orig(S, direction, log_alpha, merge_alpha)
            mx = max_spix
        elif kind == 2:
            mx = self.split_p(S, max_spix, direction, log_alpha, split_alpha)
        else:
            self.merge_p(S, direction, log_alpha, merge_alpha)
            mx = max_spix
        got["labels"] = self.labels(seg, npix).reshape(H, W)
        got["max_spix"] = mx
        self._free_state(S, keep=())
        for b in (S["border"], S["shifted"], dimg, seg):
            self.free(b)
        return got

    def _ev_ms(self, fn, reps):
        """Mean GPU time (CUDA events on the default stream) and host wall of fn()."""
        import time
        ms = C.c_float(0)
        tot_gpu = tot_wall = 0.0
        for _ in range(reps):
            self.sync()
            t0 = time.perf_counter()
            self._ck(self.L.refh_event_record(0))
            fn()
            self._ck(self.L.refh_event_record(1))
            self._ck(self.L.refh_event_ms(0, 1, C.byref(ms)))
            tot_wall += time.perf_counter() - t0
            tot_gpu += ms.value
        return tot_gpu / reps, 1000 * tot_wall / reps

    def time_stages(self, img, labels, nbuf, valid, prior_count, max_spix, sp_size, sigma2_app,
                    potts, log_alpha, reps=10):
        """Per-stage times of the reference's own kernels on one frame and a given BASS
        state, each stage restarted from the same labels and parameters every rep:
        update_params (update_params.cu:12-31), update_seg with its 4 sweeps
        (update_seg.cu:281-311), one split step with its host BFS loop
        (split_merge_orig.cu:202-414) and one merge step (:79-199).  Returns
        {stage: (gpu_ms, wall_ms)}; the wall includes the reference's host round trips."""
        H, W = labels.shape
        npix = H * W
        dimg = self.h2d(np.ascontiguousarray(img, np.float32))
        seg = self.h2d(np.ascontiguousarray(labels, np.int32))
        seg0 = self.h2d(np.ascontiguousarray(labels, np.int32))
        icov = np.tile(np.array([1.0, 0.0, 1.0]), nbuf)
        psig = np.tile(np.array([1.0 / sp_size, 0.0, 1.0 / sp_size]), nbuf)
        host = self.pack_sp(nbuf, valid=valid, prior_count=prior_count, prior_icov=icov,
                            prior_sigma_shape=psig)
        S = self._state(dimg, seg, npix, W, H, nbuf, sigma2_app, sp_size, 2 * npix, self.SM)
        S["sp"] = self.h2d(host)
        sp0 = self.h2d(host)
        up = (dimg, seg, S["sp"], S["helper"], sigma2_app, npix, sp_size, nbuf, W)

        def restore():
            self.d2d(seg, seg0, 4 * npix)
            self.d2d(S["sp"], sp0, nbuf * self.SP)
            self.update_params(*up)
            self.memset8(S["border"], 0, npix)
            self.find_border(seg, S["border"], npix, W, H)
            self.sync()
        out = {}
        restore()
        out["update_params"] = self._ev_ms(lambda: self.update_params(*up), reps)
        gpu = wall = 0.0
        for _ in range(reps):
            restore()
            g, w_ = self._ev_ms(lambda: self.update_seg(dimg, seg, S["border"], S["sp"], 4,
                                                        sigma2_app, potts, npix, W, H), 1)
            gpu += g
            wall += w_
        out["update_seg_4_sweeps"] = (gpu / reps, wall / reps)
        gpu = wall = 0.0
        for _ in range(reps):
            restore()
            g, w_ = self._ev_ms(lambda: self.split_orig(S, max_spix, 2, log_alpha, 0.0), 1)
            gpu += g
            wall += w_
        out["split_step"] = (gpu / reps, wall / reps)
        gpu = wall = 0.0
        for _ in range(reps):
            restore()
            g, w_ = self._ev_ms(lambda: self.merge_orig(S, 1, log_alpha, 0.0), 1)
            gpu += g
            wall += w_
        out["merge_step"] = (gpu / reps, wall / reps)
        self._free_state(S, keep=())
        for b in (S["border"], dimg, seg, seg0, sp0):
            self.free(b)
        return out

    # -- drivers ------------------------------------------------------------------------
    def _state(self, img, seg, npix, W, H, nbuf, sigma2_app, sp_size, pairs_entries, sm_size):
        return dict(img=img, seg=seg, npix=npix, W=W, H=H, nbuf=nbuf, sigma2_app=sigma2_app,
                    sp_size=sp_size, border=self.zeros(npix), sp=None,
                    helper=self.zeros(nbuf * self.HELPER), smh=self.zeros(nbuf * sm_size),
                    seg1=self.zeros(4 * npix), seg2=self.zeros(4 * npix),
                    pairs=self.zeros(4 * pairs_entries))

    def _free_state(self, S, keep=("img", "seg", "border")):
        for k in ("helper", "smh", "seg1", "seg2", "pairs", "sp", "shifted_own"):
            if k not in keep and S.get(k) is not None:
                self.free(S[k])

    def bass(self, S, niters, niters_seg, sm_start, potts, alpha_hastings, split_alpha, nspix):
        # bass.cu:46-181 (target_nspix = 0, merge_alpha = 0)
        count, max_spix, merge_alpha = 1, nspix - 1, 0.0
        a = (S["img"], S["seg"], S["sp"], S["helper"], S["sigma2_app"], S["npix"], S["sp_size"],
             S["nbuf"], S["W"])
        for idx in range(niters):
            self.update_params(*a)
            if idx > sm_start:
                if idx % 4 == 0:
                    count += 1
                    max_spix = self.split_orig(S, max_spix, count % 2 + 1, alpha_hastings,
                                               split_alpha)
                    self.update_params(*a)
                if idx % 4 == 2:
                    self.merge_orig(S, count % 2, alpha_hastings, merge_alpha)
                    self.update_params(*a)
            self.update_seg(S["img"], S["seg"], S["border"], S["sp"], niters_seg, S["sigma2_app"],
                            potts, S["npix"], S["W"], S["H"])
        self.update_params(*a)
        self.store_sample_sigma_shape(S["sp"], S["helper"], S["sp_size"], S["nbuf"])
        self.find_border_end(S["seg"], S["border"], S["npix"], S["W"], S["H"])
        return max_spix

    def run_bass(self, img, H, W, niters, niters_seg, sm_start, sp_size, sigma2_app, potts,
                 alpha_hastings, split_alpha):
        """bass.cu:221-345 on a device image; returns (labels Buf, Params, nspix)."""
        npix = H * W
        seg = self.zeros(4 * npix)
        nspix = self.init_seg(seg, sp_size, W, H)
        nbuf = nspix * 30
        S = self._state(img, seg, npix, W, H, nbuf, sigma2_app, sp_size, 2 * npix, self.SM)
        S["sp"] = self.zeros(nbuf * self.SP)
        nspix = self.compactify(seg, S["sp"], self.extract_unique_ids(seg, npix, 0), 0, npix)
        self.mark_active(S["sp"], np.arange(nspix, dtype=np.int32), nspix, nbuf, sp_size)
        self.init_sp_params(S["sp"], sigma2_app, img, seg, S["helper"], npix, nspix, nbuf, W,
                            sp_size)
        self.find_border(seg, S["border"], npix, W, H)
        max_spix = self.bass(S, niters, niters_seg, sm_start, potts, alpha_hastings, split_alpha,
                             nspix)
        prop_ids = self.extract_unique_ids(seg, npix, 0)
        nspix = self.compactify(seg, S["sp"], prop_ids, 0, npix)
        uniq = self.get_unique(seg, npix)
        pr = self.get_params_as_vectors(S["sp"], len(uniq), nspix)
        self.run_update_prior(pr, uniq, nspix, 0)
        self.find_border_end(seg, S["border"], npix, W, H)
        self._free_state(S, keep=("img", "seg"))
        self.free(S["border"])
        return seg, pr, nspix

    def sp_downsample(self, tensor, seg, nspix, npix, nftrs):
        # sp_pooling.cu:121-147
        down = self.zeros(4 * nspix * nftrs)
        counts = self.zeros(4 * nspix)
        self.launch("sp_pooling", "sp_downsample_kernel", nblk(npix),
                    [P(tensor), P(seg), P(down), P(counts), I(nspix), I(1), I(npix), I(nftrs)])
        self.launch("sp_pooling", "normz_downsample_kernel", nblk(nspix),
                    [P(down), P(counts), I(nspix), I(1), I(nftrs)])
        return down, counts

    def shift_labels(self, spix, flow_ds, sizes, nspix, H, W):
        # shift_labels.cu:175-239
        npix = H * W
        tmp = self.zeros(8 * npix)
        shifted = self.zeros(4 * npix)
        counts = self.zeros(4 * npix)
        min_sizes = self.zeros(4 * npix)
        self.memset32(tmp, 100000, 2 * npix)
        self.memset32(min_sizes, 100000, npix)
        self.launch("shift_labels", "shift_labels_kernel", nblk(npix),
                    [P(spix), P(flow_ds), P(tmp), P(counts), P(sizes), P(min_sizes), I(npix),
                     I(nspix), I(1), I(H), I(W)])
        self.launch("shift_labels", "decode_kernel", nblk(npix),
                    [P(shifted), P(tmp), P(counts), P(min_sizes), I(npix), I(nspix), I(1), I(H),
                     I(W)])
        for b in (tmp, counts, min_sizes):
            self.free(b)
        return shifted

    def spix_counts(self, seg, npix, nspix):
        # seg_utils.cu:104-135
        sizes = self.zeros(4 * nspix)
        self.launch("seg_utils", "get_spix_sizes_kernel", nblk(npix),
                    [P(seg), P(sizes), I(npix), I(nspix)])
        out = self.d2h(sizes, np.int32, nspix)
        self.free(sizes)
        return out

    def fill_missing(self, seg, centers, H, W, break_iter=1000):
        # fill_missing.cu:35-130 + run_fill_missing :656-669
        npix = H * W
        border = self.zeros(npix)
        nn = self.zeros(4)
        it, prev_neg, num_neg = 0, 1410065408, 1   # (int)10000000000 as the reference stores it
        while num_neg > 0:
            if break_iter > 0 and it >= break_iter:
                break
            self.memset8(nn, 0, 4)
            self.memset8(border, 0, npix)
            self.launch("fill_missing", "find_border_along_missing", nblk(npix),
                        [P(seg), P(border), I(1), I(H), I(W), P(nn)])
            num_neg = self.int_at(nn)
            for xm in range(2):
                for ym in range(2):
                    self.launch("fill_missing", "update_missing_seg_nn", nblk(npix),
                                [P(seg), P(centers), P(border), I(1), I(H), I(W), I(npix), I(xm),
                                 I(ym), B(False)])
            it += 1
            if num_neg == prev_neg:
                raise RefError("fill_missing: the border won't shrink (%d)" % num_neg)
            prev_neg = num_neg
        self.free(border)
        self.free(nn)
        self.log.append(("fill", it))
        return it

    def invalidate_disconnected(self, seg, H, W, nspix):
        # split_disconnected.cu:33-96 + get_regions :107-185
        npix = H * W
        lab = self.labels(seg, npix)
        if lab.min() < 0 or lab.max() >= nspix:  # assign_spix_to_regions indexes by label
            raise RefError("labels outside [0, %d) before invalidate_disconnected" % nspix)
        regions = self.h2d(np.arange(npix, dtype=np.int32))
        prev = self.zeros(4 * npix)
        ch = self.zeros(4)
        changes = 1
        while changes:
            self.d2d(prev, regions, 4 * npix)
            self.memset8(ch, 0, 4)
            self.launch("split_disconnected", "find_spix_min", nblk(npix),
                        [P(seg), P(regions), P(prev), P(ch), I(H), I(W), I(npix)])
            changes = self.int_at(ch)
        roots = self.d2h(regions, np.int32, npix)
        ids = np.unique(roots).astype(np.int32)
        nregions = len(ids)
        dids = self.h2d(ids)
        self.launch("split_disconnected", "relabel_spix", nblk(npix),
                    [P(regions), P(dids), I(npix), I(nregions)])
        region_spix = self.labels(seg, npix)[ids]
        rs = self.h2d(region_spix.astype(np.int32))
        sizes = self.zeros(4 * nspix)
        self.launch("seg_utils", "get_spix_sizes_kernel", nblk(npix),
                    [P(seg), P(sizes), I(npix), I(nspix)])
        rsz = self.zeros(4 * nregions)
        self.launch("split_disconnected", "compute_region_sizes", nblk(npix),
                    [P(rsz), P(regions), I(npix), I(nregions)])
        tmp = self.zeros(8 * nspix)
        self.launch("split_disconnected", "assign_spix_to_regions", nblk(nregions),
                    [P(tmp), P(rs), P(rsz), I(nregions), I(nspix)])
        s2r = self.alloc(4 * nspix)
        self.memset8(s2r, 0xFF, 4 * nspix)
        valid = self.zeros(nregions)
        self.launch("split_disconnected", "decode_spix_to_regions", nblk(nspix),
                    [P(s2r), P(sizes), P(valid), P(tmp), I(nregions), I(nspix)])
        self.launch("split_disconnected", "invalidate_disconnected_spix", nblk(npix),
                    [P(seg), P(regions), P(valid), I(npix)])
        for b in (regions, prev, ch, dids, rs, sizes, rsz, tmp, s2r, valid):
            self.free(b)

    def shift_and_fill(self, spix, pr: Params, flow, H, W):
        """shift_and_fill.cu:108-339; updates pr.prior_counts / invalid_counts in place."""
        nspix, npix = pr.size, H * W
        lab = self.labels(spix, npix)
        if lab.min() < 0 or lab.max() >= nspix:  # shift_labels_kernel indexes sizes/flow by it
            raise RefError("previous labels outside [0, %d)" % nspix)
        flow_gpu = self.alloc(8 * npix)
        self.d2d(flow_gpu, flow, 8 * npix)     # the reference's H2D copy of a device pointer
        flow_ds, counts = self.sp_downsample(flow_gpu, spix, nspix, npix, 2)
        fds = self.d2h(flow_ds, np.float32, 2 * nspix)
        centers_h = self.d2h(pr.mu_shape, np.float64, 2 * nspix) + fds.astype(np.float64)
        centers = self.h2d(centers_h)
        shifted = self.shift_labels(spix, flow_ds, counts, nspix, H, W)
        filled = self.alloc(4 * npix)
        self.d2d(filled, shifted, 4 * npix)
        counts_s = self.spix_counts(filled, npix, nspix)
        self.fill_missing(filled, centers, H, W, 1000)
        self.invalidate_disconnected(filled, H, W, nspix)
        self.fill_missing(filled, centers, H, W, 1000)
        counts_f = self.spix_counts(filled, npix, nspix)
        inv = ((counts_f - counts_s).astype(np.float64) /
               (counts_f.astype(np.float32).astype(np.float64) + 1e-8)).astype(np.float32)
        cur = self.d2h(counts, np.int32, nspix)
        pc = self.d2h(pr.prior_counts, np.float32, nspix)
        pc = np.where(cur > 0, np.minimum(np.maximum(cur.astype(np.float64), 100.0), 10000.0),
                      pc.astype(np.float64)).astype(np.float32)
        self.upload(pr.prior_counts, pc)
        self.upload(pr.invalid_counts, inv)
        for b in (counts, flow_ds, flow_gpu, centers):
            self.free(b)
        return filled, shifted

    def prop_bass_v3(self, S, niters, niters_seg, sm_start, potts, alpha_hastings, nspix, prev,
                     nspix_prev, thresh_relabel, thresh_new, merge_alpha, split_alpha):
        # prop.cu:326-468 (target_nspix = 0)
        count, max_spix = 1, nspix - 1
        a = (S["img"], S["seg"], S["sp"], S["helper"], S["sigma2_app"], S["npix"], S["sp_size"],
             S["nbuf"], S["W"])
        for idx in range(niters):
            self.update_params(*a)
            if idx > sm_start:
                if idx % 4 == 0:
                    count += 1
                    max_spix = self.split_p(S, max_spix, count % 2 + 1, alpha_hastings,
                                            split_alpha)
                    self.update_params(*a)
                if idx % 4 == 2:
                    living = self.extract_unique_ids(S["seg"], S["npix"], 0)
                    max_spix = self.relabel_spix(S, prev, living, thresh_relabel, thresh_new,
                                                 nspix_prev, max_spix)
                    count += 1
                    self.merge_p(S, count % 2, alpha_hastings, merge_alpha)
                    self.update_params(*a)
            self.update_seg(S["img"], S["seg"], S["border"], S["sp"], niters_seg, S["sigma2_app"],
                            potts, S["npix"], S["W"], S["H"])
        self.update_params(*a)
        self.store_sample_sigma_shape(S["sp"], S["helper"], S["sp_size"], S["nbuf"])
        self.find_border_end(S["seg"], S["border"], S["npix"], S["W"], S["H"])
        return max_spix

    def run_prop(self, img, H, W, niters, niters_seg, sm_start, sp_size, sigma2_app, potts,
                 alpha_hastings, filled, shifted, prev: Params, thresh_relabel, thresh_new,
                 merge_alpha, split_alpha):
        """prop.cu:677-865; returns (labels Buf, Params, nspix)."""
        npix = H * W
        nspix = prev.size
        seg = self.alloc(4 * npix)
        self.d2d(seg, filled, 4 * npix)
        nspix_prev = nspix
        nbuf = nspix * 10
        S = self._state(img, seg, npix, W, H, nbuf, sigma2_app, sp_size, 2 * nbuf, self.SM2)
        S["shifted"] = shifted
        S["sp"] = self.get_vectors_as_params(prev, nbuf)
        init_ids = self.get_unique(seg, npix)
        self.mark_active(S["sp"], init_ids, nspix, nbuf, sp_size)
        max_spix = self.prop_bass_v3(S, niters, niters_seg, sm_start, potts, alpha_hastings, nspix,
                                     prev, nspix_prev, thresh_relabel, thresh_new, merge_alpha,
                                     split_alpha)
        prop_ids = self.extract_unique_ids(seg, npix, 0)
        new_ids = prop_ids[prop_ids >= nspix_prev]
        nspix = self.compactify(seg, S["sp"], new_ids, nspix_prev, npix)
        uniq = self.get_unique(seg, npix)
        pr = self.get_params_as_vectors(S["sp"], nspix, nspix)
        self.run_update_prior(pr, uniq, nspix, nspix_prev)
        self.find_border_end(seg, S["border"], npix, W, H)
        self._free_state(S, keep=("img", "seg"))
        self.free(S["border"])
        return seg, pr, nspix

    def prop_frame(self, img_h: np.ndarray, labels_prev: np.ndarray, params_prev: dict,
                   flow_h: np.ndarray, niters: int, sp_size: int, potts: float,
                   sigma2_app: float, alpha: float, split_alpha: float) -> np.ndarray:
        """One propagated frame of main_loop (pyapi.cu:120-170) from a given host state:
        the previous frame's labels and SuperpixelParams fields (as recorded by
        bist_forward(record=True)), the flow into this frame and the iteration count
        the recorded run chose.  Returns the frame's int32 [H,W] labels.  Rerunning a
        recorded frame this way measures how much the reference's races alone change
        one frame."""
        H, W = labels_prev.shape
        npix = H * W
        n = int(len(params_prev["counts"]))
        pr = Params(self, n)
        for name, dt, k in Params.FIELDS:
            self.upload(getattr(pr, name), np.ascontiguousarray(params_prev[name][: n * k], dt))
        spix = self.h2d(np.ascontiguousarray(labels_prev, np.int32))
        flow = self.h2d(np.ascontiguousarray(flow_h, np.float32))
        img = self.h2d(np.ascontiguousarray(img_h, np.float32))
        filled, shifted = self.shift_and_fill(spix, pr, flow, H, W)
        seg, pr2, _ = self.run_prop(img, H, W, niters, 4, 0, sp_size, sigma2_app, potts, alpha,
                                    filled, shifted, pr, 1e-5, 1e-2, 0.0, split_alpha)
        out = self.labels(seg, npix).reshape(H, W)
        for b in (spix, flow, img, filled, shifted, seg):
            self.free(b)
        pr.free(self)
        pr2.free(self)
        self.sync()
        return out

    def bist_forward(self, vid: np.ndarray, flows: np.ndarray, niters: int, sp_size: int,
                     potts: float, sigma2_app: float, alpha: float, split_alpha: float,
                     video_mode: bool, record: bool = False) -> np.ndarray:
        """pyapi.cu:200-215 + main_loop :46-195 on host arrays; returns int32 [T,H,W].
        With record, self.frames keeps per frame the host copies of the labels, the
        parameters handed to the next frame (SuperpixelParams fields), and for
        propagated frames the filled / shifted maps and the iteration count."""
        vid = np.ascontiguousarray(vid, np.float32)
        T, H, W, nftrs = vid.shape
        assert nftrs == 3
        npix = H * W
        sm_start, niters_seg = 0, 4
        merge_alpha, thresh_relabel, thresh_new = 0.0, 1e-5, 1e-2
        out = np.zeros((T, H, W), np.int32)
        spix_prev, params_prev = None, None
        self.log = []
        self.frame_niters = []
        self.frames = []
        for fidx in range(T):
            rec = {}
            img = self.h2d(vid[fidx])
            if fidx == 0 or not video_mode:
                seg, pr, _ = self.run_bass(img, H, W, niters, niters_seg, sm_start, sp_size,
                                           sigma2_app, potts, alpha, split_alpha)
                self.frame_niters.append(niters)
            else:
                flow = self.h2d(np.ascontiguousarray(flows[fidx - 1], np.float32))
                filled, shifted = self.shift_and_fill(spix_prev, params_prev, flow, H, W)
                if record:
                    rec["filled"] = self.labels(filled, npix).reshape(H, W)
                    rec["shifted"] = self.labels(shifted, npix).reshape(H, W)
                    rec["params_prev_after_shift"] = params_prev.host(self)
                ninvalid = int((self.labels(shifted, npix) == -1).sum())
                iperc = ninvalid / (1.0 * npix)
                niters = 12 if iperc > 0.20 else (4 if iperc < 0.01 else 8)
                self.frame_niters.append(niters)
                seg, pr, _ = self.run_prop(img, H, W, niters, niters_seg, sm_start, sp_size,
                                           sigma2_app, potts, alpha, filled, shifted, params_prev,
                                           thresh_relabel, thresh_new, merge_alpha, split_alpha)
                for b in (flow, filled, shifted):
                    self.free(b)
            out[fidx] = self.labels(seg, npix).reshape(H, W)
            if record:
                rec["labels"] = out[fidx].copy()
                rec["params"] = pr.host(self)
                rec["niters"] = self.frame_niters[-1]
                self.frames.append(rec)
            self.free(img)
            if spix_prev is not None:
                self.free(spix_prev)
                params_prev.free(self)
            spix_prev, params_prev = seg, pr
        self.free(spix_prev)
        params_prev.free(self)
        self.sync()
        return out
