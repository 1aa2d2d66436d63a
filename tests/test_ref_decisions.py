"""Pins the split / merge decisions against the reference's OWN kernels on shared states.

The reference scores every split and merge with an FP32 Hastings ratio built from
__logf / lgammaf terms of size ~1e5 (split_merge_orig.cu:456-656, 735-986;
split_merge_prop.cu:2572-3149); the engine and the oracle evaluate the same ratio in
FP64 with the cancelling lgamma(a_n) terms removed.  On an identical state (labels,
valid flags, prior counts, propagation flags, hole map) both sides must score the
same set of superpixels, pick the same merge candidates, agree on the ratio within
the FP32 evaluation error of the reference (RATIO_ATOL), and take the same decision
(ratio > -2) everywhere except where the FP64 ratio lies within NEAR of the
threshold, which is where the reference's rounding can flip it.  The engine matches
the oracle bit for bit on the whole loop (tests/test_gpu_parity.py), so this pins the
engine's decisions too.  Skipped where oracle/_ref was not built."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import ref_runner as RR
from st_spix_gb300 import synth

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not RR.available("nofma"), reason="oracle/_ref not built")]

S2 = 0.009 ** 2
LOG_ALPHA = float(np.log(0.5))
# absolute agreement of the FP32 reference ratio with the FP64 oracle ratio, and the
# band around the -2 threshold inside which the two may decide differently.  The
# reference's colour sums are FP32 atomics whose order varies from run to run, so its
# ratio does too: runs on GB300 gave errors up to 0.26 on the 480x854 case.
RATIO_ATOL = 0.5
NEAR = 0.5
_ref = {}


def ref(variant="nofma"):
    if variant not in _ref:
        _ref[variant] = RR.Ref(variant)
    return _ref[variant]


def _state(img, sp, iters):
    cfg = O.default_config(niters=100, sp_size=sp)
    st, lab, d, nbuf, mx = O.bass_partial(img, cfg, iters)
    assert st == 0
    return lab, d, nbuf, mx, cfg


def _prop_inputs(lab, d, nbuf, sp, seed):
    """Propagation flags on two thirds of the living ids and a hole map with a few
    rectangular holes (the propagated steps read both)."""
    rng = np.random.default_rng(seed)
    prop = ((np.arange(nbuf) % 3) != 0).astype(np.uint8) * d["valid"]
    shifted = lab.copy()
    H, W = lab.shape
    for _ in range(12):
        y, x = rng.integers(0, H - 12), rng.integers(0, W - 12)
        shifted[y:y + rng.integers(3, 12), x:x + rng.integers(3, 12)] = -1
    return prop, shifted


def _compare(r, o, kind, valid):
    init = -999999.0 if kind in (0, 1) else -99999.0
    scored_r = (r["h"] != np.float32(init)) & (valid > 0)
    scored_o = ~np.isnan(o["h"]) & (valid > 0)
    np.testing.assert_array_equal(scored_r, scored_o, err_msg="scored ids differ")
    if kind in (1, 3):
        np.testing.assert_array_equal(r["pair"][valid > 0], o["pair"][valid > 0],
                                      err_msg="merge candidates differ")
    hr = r["h"][scored_o].astype(np.float64)
    ho = o["h"][scored_o]
    fin = np.isfinite(ho)
    np.testing.assert_array_equal(np.isfinite(hr), fin)
    np.testing.assert_array_equal(hr[~fin], ho[~fin])
    err = np.abs(hr[fin] - ho[fin])
    assert err.size == 0 or err.max() <= RATIO_ATOL, f"ratio error {err.max()}"
    want_r = hr > -2
    want_o = o["want"][scored_o] > 0
    flips = np.nonzero(want_r != want_o)[0]
    for i in flips:
        assert abs(ho[i] + 2) < NEAR, f"decision differs away from the threshold: {ho[i]}"
    return int(scored_o.sum()), int(want_o.sum()), float(err.max() if err.size else 0), len(flips)


CASES = [(240, 320, 15, 200, 0.05, it) for it in (2, 10, 30, 60)] + [(480, 854, 20, 400, 0.03, 8)]


@pytest.mark.parametrize("variant", ["nofma", "stock"])
@pytest.mark.parametrize("H,W,sp,nseeds,sigma,iters", CASES)
def test_bass_split_merge_decisions_pinned(H, W, sp, nseeds, sigma, iters, variant):
    img, _ = synth.voronoi_frame(H, W, nseeds, sigma, 0)
    lab, d, nbuf, mx, cfg = _state(img, sp, iters)
    R = ref(variant)
    sample = np.zeros(3 * nbuf)
    zeros = np.zeros(nbuf, np.uint8)
    totals = []
    for kind, direction in ((0, 1), (0, 2), (1, 0), (1, 1)):
        r = R.sm_step(img, lab, nbuf, d["valid"], d["prior_count"], zeros, sample, mx, kind,
                      direction, None, sp, S2, LOG_ALPHA, 0.0, 0.0)
        o = O.sm_step(img, lab, cfg, nbuf, d["valid"], d["prior_count"], zeros, sample, mx, kind,
                      direction)
        assert o["status"] == 0
        totals.append(_compare(r, o, kind, d["valid"]))
    scored = sum(t[0] for t in totals)
    assert scored > 50
    # some splits and some merges pass the threshold at these states
    assert sum(t[1] for t in totals[:2]) > 0 or iters < 10
    print(f"{H}x{W} it{iters} {variant}: (scored, accepted, max |dh|, flips) = {totals}")


@pytest.mark.parametrize("variant", ["nofma", "stock"])
@pytest.mark.parametrize("iters", [8, 30])
def test_propagated_split_merge_decisions_pinned(iters, variant):
    H, W, sp = 240, 320, 15
    img, _ = synth.voronoi_frame(H, W, 200, 0.05, 1)
    lab, d, nbuf, mx, cfg = _state(img, sp, iters)
    prop, shifted = _prop_inputs(lab, d, nbuf, sp, iters)
    sample = np.tile(np.array([sp * sp / 4.0, 0.0, sp * sp / 4.0]), nbuf)
    R = ref(variant)
    totals = []
    for kind, direction in ((2, 1), (2, 2), (3, 0), (3, 1)):
        r = R.sm_step(img, lab, nbuf, d["valid"], d["prior_count"], prop, sample, mx, kind,
                      direction, shifted, sp, S2, LOG_ALPHA, 0.0, 0.0)
        o = O.sm_step(img, lab, cfg, nbuf, d["valid"], d["prior_count"], prop, sample, mx, kind,
                      direction, shifted)
        assert o["status"] == 0
        totals.append(_compare(r, o, kind, d["valid"]))
    assert sum(t[0] for t in totals) > 50
    print(f"prop it{iters} {variant}: (scored, accepted, max |dh|, flips) = {totals}")
