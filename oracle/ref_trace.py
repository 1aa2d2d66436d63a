"""ORACLE -- test infrastructure only: traces where the reference's trajectory and this
project's deterministic rules part ways.

Tracer runs the reference's own run_bass (oracle/ref_runner.py) and, at every
decision of that trajectory, evaluates the oracle's rule (the rule the engine runs,
bit for bit) on the reference's OWN state at that moment:

  * sweep_arith   update_seg (update_seg.cu:281-311) on the reference's parameters:
                  pixels where the oracle's sweep labels differ from the reference's
                  (the same IEEE arithmetic, so none with the -fmad=false build);
  * sweep_stats   the same sweep with the statistics the oracle computes exactly
                  (int64 sums) instead of the reference's FP32 atomic sums: pixels
                  whose label flips under that last-bits change of a mean (each one a
                  near tie of the score);
  * split / merge the Hastings decision per superpixel (split_merge_orig.cu:618-656,
                  900-986): flips, each with the FP64 ratio's distance to the -2
                  threshold;
  * merge_claim   targets claimed by several accepted merges, where the reference's
                  first atomicMax caller (:635-639) and the smallest claimant differ;
  * split_ids     accepted splits whose new id (atomicAdd order, :968) differs from
                  the ascending-order id, which later changes merge candidates (the
                  largest neighbouring id, split_merge.cu:719-755);
  * stale_read    a merge whose candidate scored no merge of its own in this step:
                  the reference then reads the candidate's ratio terms left in its
                  split/merge scratch by an earlier step (never reset), the oracle
                  reads them as never written (ratio -inf, rule R7);
  * warp_ties     (propagated frames) pixels where the reference's forward warp of the
                  previous labels, whose equal-size collisions race, and the oracle's
                  rule (smallest (size, id) wins) give different shifted / filled maps.

Split and merge decisions are evaluated on the state the reference's loop holds at
that moment: its border mask, and for a merge right after a propagated frame's
relabel, the statistics update_params left with the relabel's id changes applied.

Every event is a tie or a near-threshold decision by construction; a run with no
event ends with the oracle's labels.
"""
from __future__ import annotations

import numpy as np

from oracle import oracle as O
from oracle import ref_runner as RR


class Tracer(RR.Ref):
    def __init__(self, variant="nofma"):
        super().__init__(variant)
        self.events = []

    # -- reference state on the host -------------------------------------------------
    def _sp_fields(self, sp, nbuf):
        raw = self.d2h(sp, np.uint8, nbuf * self.SP)
        lay, SP = self.lay, self.SP

        def f(name, dt, k):
            dt = np.dtype(dt)
            v = np.ndarray((nbuf, k), dt, buffer=raw, offset=lay["REF_OFF_" + name],
                           strides=(SP, dt.itemsize))
            return v.copy().reshape(-1)
        return dict(count=f("count", np.int32, 1), valid=f("valid", np.int32, 1),
                    prop=f("prop", np.uint8, 1), prior_count=f("prior_count", np.float32, 1),
                    mu_app=f("mu_app", np.float32, 3), mu_shape=f("mu_shape", np.float64, 2),
                    sigma_shape=f("sigma_shape", np.float64, 3),
                    logdet=f("logdet_sigma_shape", np.float64, 1),
                    prior_icov=f("prior_icov", np.float64, 3),
                    sample_sigma=f("sample_sigma_shape", np.float64, 3))

    # -- traced stages --------------------------------------------------------------------
    def update_seg(self, img, seg, border, sp, niters, sigma2_app, potts, npix, W, H):
        if getattr(self, "_img_h", None) is None:
            return super().update_seg(img, seg, border, sp, niters, sigma2_app, potts, npix, W, H)
        nbuf = self._nbuf
        lab0 = self.labels(seg, npix).reshape(H, W)
        st = self._sp_fields(sp, nbuf)
        super().update_seg(img, seg, border, sp, niters, sigma2_app, potts, npix, W, H)
        lab1 = self.labels(seg, npix).reshape(H, W)
        mine = O.update_seg_given(self._img_h, lab0, nbuf, niters, sigma2_app, potts, st["count"],
                                  st["mu_app"], st["mu_shape"], st["sigma_shape"], st["logdet"])
        n_arith = int((mine != lab1).sum())
        ex = O.update_params_given(self._img_h, lab0, nbuf, self._sp_size, sigma2_app,
                                   st["valid"], st["prop"], st["prior_count"], st["prior_icov"],
                                   st["sample_sigma"])
        exact = O.update_seg_given(self._img_h, lab0, nbuf, niters, sigma2_app, potts,
                                   ex["count"], ex["mu_app"], ex["mu_shape"], ex["sigma_shape"],
                                   ex["logdet"])
        n_stats = int((exact != mine).sum())
        if n_arith:
            self.events.append(("sweep_arith", n_arith))
        if n_stats:
            self.events.append(("sweep_stats", n_stats))

    def _decisions(self, S, kind, direction, max_spix):
        H, W = S["H"], S["W"]
        lab = self.labels(S["seg"], S["npix"]).reshape(H, W)
        st = self._sp_fields(S["sp"], S["nbuf"])
        relabel = None
        border = self.d2h(S["border"], np.uint8, S["npix"])    # what the loop's merge reads
        rl = getattr(self, "_relabel", None)
        if kind == 3 and rl is not None:
            # a merge right after a relabel: the state update_params left, then the ids
            # relabel_spix changed (the loop runs no update_params in between)
            lab, st, relabel = rl["labels"], rl["st"], (rl["rid"], rl["nspix_prev"])
        self._relabel = None
        cfg = O.default_config(sp_size=self._sp_size, sigma2_app=S["sigma2_app"],
                               alpha_hastings=self._alpha)
        if kind in (2, 3):      # propagated: the superpixels' prop flags and sampled shapes
            prop, sample = st["prop"].astype(np.uint8), st["sample_sigma"]
            shifted = self.labels(S["shifted"], S["npix"]).reshape(H, W)
        else:
            prop, sample, shifted = np.zeros(S["nbuf"], np.uint8), np.zeros(3 * S["nbuf"]), None
        return O.sm_step(self._img_h, lab, cfg, S["nbuf"], (st["valid"] != 0).astype(np.uint8),
                         st["prior_count"], prop, sample, max_spix, kind, direction, shifted,
                         relabel, border)

    def relabel_spix(self, S, prev, living, thresh_replace, thresh_new, nspix_prev, max_spix_in):
        if getattr(self, "_img_h", None) is None:
            return super().relabel_spix(S, prev, living, thresh_replace, thresh_new, nspix_prev,
                                        max_spix_in)
        st = self._sp_fields(S["sp"], S["nbuf"])

        def hook(lab_pre, rid, nprev):
            self._relabel = dict(labels=lab_pre, rid=rid, nspix_prev=nprev, st=st)
        S["relabel_hook"] = hook
        try:
            return super().relabel_spix(S, prev, living, thresh_replace, thresh_new, nspix_prev,
                                        max_spix_in)
        finally:
            S.pop("relabel_hook")

    def _hook(self, S, got, prop=False):
        smsize = self.SM2 if prop else self.SM
        pre = "REF_SM2OFF_" if prop else "REF_SMOFF_"

        def hook(_event, _mx):
            raw = self.d2h(S["smh"], np.uint8, S["nbuf"] * smsize)
            got["h"] = np.ndarray((S["nbuf"],), np.float32, buffer=raw,
                                  offset=self.lay[pre + "hasting"], strides=(smsize,)).copy()
            got["merge"] = np.ndarray((S["nbuf"],), np.uint8, buffer=raw,
                                      offset=self.lay[pre + "merge"],
                                      strides=(smsize,)).copy()
            got["pairs"] = self.d2h(S["pairs"], np.int32, 2 * S["nbuf"]).reshape(-1, 2).copy()
        return hook

    def _flips(self, name, r, o, valid):
        scored = ~np.isnan(o["h"]) & (valid != 0)
        want_r = (r["h"].astype(np.float64) > -2) & scored
        want_o = (o["want"] > 0) & scored
        for k in np.nonzero(want_r != want_o)[0]:
            if name == "merge" and o["h"][k] == -np.inf:
                # the candidate f scored no merge of its own this step, so the reference
                # reads f's numerator / denominator left in sm_helper by an earlier step
                # (init_sm_p, split_merge_prop.cu:461-530, does not reset them); the
                # oracle reads them as never written (zero b_n: ratio -inf, rule R7)
                self.events.append(("stale_read", int(k)))
            else:
                self.events.append((name, float(abs(o["h"][k] + 2))))
        return want_r, want_o

    def _split(self, S, max_spix, direction, log_alpha, split_alpha, prop):
        run = super().split_p if prop else super().split_orig
        if getattr(self, "_img_h", None) is None:
            return run(S, max_spix, direction, log_alpha, split_alpha)
        o = self._decisions(S, 2 if prop else 0, direction, max_spix)
        valid = self._sp_fields(S["sp"], S["nbuf"])["valid"]
        got = {}
        S["decision_hook"] = self._hook(S, got, prop)
        new_max = run(S, max_spix, direction, log_alpha, split_alpha)
        S.pop("decision_hook")
        if got:
            want_r, _ = self._flips("split", got, o, valid)
            # ids: the reference's atomicAdd order against ascending order
            ks = np.nonzero(want_r)[0]
            ref_ids = got["pairs"][ks, 0]
            asc = max_spix + 1 + np.arange(len(ks))
            n_id = int((ref_ids != asc).sum())
            if n_id:
                self.events.append(("split_ids", n_id))
        return new_max

    def split_orig(self, S, max_spix, direction, log_alpha, split_alpha):
        return self._split(S, max_spix, direction, log_alpha, split_alpha, False)

    def split_p(self, S, max_spix, direction, alpha, split_alpha):
        return self._split(S, max_spix, direction, alpha, split_alpha, True)

    def merge_p(self, S, direction, log_alpha, merge_alpha):
        return self._merge(S, direction, log_alpha, merge_alpha, True)

    def merge_orig(self, S, direction, log_alpha, alpha_merge):
        return self._merge(S, direction, log_alpha, alpha_merge, False)

    def _merge(self, S, direction, log_alpha, alpha_merge, prop):
        run = super().merge_p if prop else super().merge_orig
        if getattr(self, "_img_h", None) is None:
            return run(S, direction, log_alpha, alpha_merge)
        o = self._decisions(S, 3 if prop else 1, direction, 0)
        valid = self._sp_fields(S["sp"], S["nbuf"])["valid"]
        got = {}
        S["decision_hook"] = self._hook(S, got, prop)
        run(S, direction, log_alpha, alpha_merge)
        S.pop("decision_hook")
        if got:
            want_r, want_o = self._flips("merge", got, o, valid)
            # claims: per target, the reference's winner against the smallest claimant
            won_r = got["merge"] > 0
            for f in np.unique(got["pairs"][want_r, 1]):
                cl = np.nonzero(want_r & (got["pairs"][:, 1] == f))[0]
                if len(cl) > 1:
                    wr = cl[won_r[cl]]
                    if len(wr) != 1 or wr[0] != cl.min():
                        self.events.append(("merge_claim", int(len(cl))))
        return None

    def run_bass_traced(self, img_h, H, W, niters, sp_size, sigma2_app, potts, alpha,
                        split_alpha):
        """run_bass on a host image with tracing; returns (labels, events)."""
        self.events = []
        self._img_h = np.ascontiguousarray(img_h, np.float32)
        self._sp_size = sp_size
        self._alpha = alpha
        hh = np.sqrt(float(sp_size) ** 2 / (1.5 * np.sqrt(3.0)))
        nx = int(np.floor(W / (np.sqrt(3.0) * hh))) + 2
        ny = int(np.floor(H / (1.5 * hh))) + 2
        self._nbuf = 30 * nx * ny
        img = self.h2d(self._img_h)
        try:
            seg, pr, n = self.run_bass(img, H, W, niters, 4, 0, sp_size, sigma2_app, potts, alpha,
                                       split_alpha)
            lab = self.labels(seg, H * W).reshape(H, W)
            self.free(seg)
            pr.free(self)
        finally:
            self.free(img)
            self._img_h = None
        return lab, list(self.events)

    def prop_frame_traced(self, img_h, labels_prev, params_prev, flow_h, niters, sp_size,
                          sigma2_app, potts, alpha, split_alpha):
        """One propagated frame (prop_frame) with tracing; returns (labels, events).
        The relabel stage is not traced: its ties (equal distances, duplicate
        revivals) are resolved by the engine's fixed rule and count as id-order
        events only through the later merge candidates they change."""
        self.events = []
        self._img_h = np.ascontiguousarray(img_h, np.float32)
        self._sp_size = sp_size
        self._alpha = alpha
        self._nbuf = 10 * int(len(params_prev["counts"]))
        try:
            lab = self.prop_frame(img_h, labels_prev, params_prev, flow_h, niters, sp_size, potts,
                                  sigma2_app, alpha, split_alpha)
        finally:
            self._img_h = None
        return lab, list(self.events)

    def shift_and_fill(self, spix, pr, flow, H, W):
        """shift_and_fill with a warp_ties event: pixels where the reference's forward
        warp (shift_labels.cu:33-164, collisions by atomic size order, equal sizes
        racy) and the oracle's rule R4 (smallest (size, id) wins) on the same previous
        labels, parameters and flow give different shifted or filled maps."""
        if getattr(self, "_img_h", None) is None:
            return super().shift_and_fill(spix, pr, flow, H, W)
        npix = H * W
        lab_prev = self.labels(spix, npix).reshape(H, W)
        params = pr.host(self)
        fl = self.d2h(flow, np.float32, 2 * npix).reshape(H, W, 2)
        filled, shifted = super().shift_and_fill(spix, pr, flow, H, W)
        st, o_filled, o_shifted, _ = O.shift_and_fill(lab_prev, params, pr.size, fl)
        n_sh = int((self.labels(shifted, npix).reshape(H, W) != o_shifted).sum())
        n_fi = int((self.labels(filled, npix).reshape(H, W) != o_filled).sum())
        if st == 0 and (n_sh or n_fi):
            self.events.append(("warp_ties", max(n_sh, n_fi)))
        return filled, shifted
