"""Quality metrics (st_spix/spix_utils/evaluate.py): the oracle pinned to the
reference's own metric functions (tests/golden/quality_ref.npz), the GPU kernels
against the oracle.  Integer tables exact; FP64 scores within 1e-9 relative (FP64
atomics sum in a different order than the oracle)."""
import math

import numpy as np
import pytest

from oracle import quality as Q

GOLDEN = "tests/golden/quality_ref.npz"
CASES = ["bist_40x56x4", "ragged_17x23x5"]
PINNED = ["tex", "szv", "ev", "ue2d", "sa2d", "ue3d", "sa3d", "spnum", "ave_nsp"]
SCORES = PINNED + ["ev3d", "pooling"]


def _golden(name):
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.dirname(__file__)), GOLDEN))
    return {k.split("/", 1)[1]: d[k] for k in d.files if k.startswith(name + "/")}


def _close(a, b, rel):
    if isinstance(b, float) and math.isnan(b):
        return math.isnan(a)
    return abs(a - b) <= rel * max(abs(b), 1e-300)


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    g = _golden(name)
    spo = g["spix"] - g["spix"].min()
    np.testing.assert_array_equal(Q.count_spix(spo), g["counts"])
    s = Q.compute_summary(g["vid"], g["spix"], g["gt"])
    for k in PINNED:
        assert _close(s[k], float(g[k]), 1e-12), (k, s[k], float(g[k]))


def test_oracle_edge_cases():
    rng = np.random.default_rng(1)
    vid = rng.uniform(0, 1, (1, 6, 7, 3)).astype(np.float32)
    lab = np.zeros((1, 6, 7), np.int32)
    lab[:, 3:] = 1
    s = Q.compute_summary(vid, lab, np.zeros_like(lab))
    assert math.isnan(s["szv"])                 # no id alive in two frames
    assert math.isnan(s["sa2d"]) and math.isnan(s["sa3d"])   # only the background id
    assert s["ue2d"] == 0.0 and s["tex"] == 1.0 and s["spnum"] == 2
    with pytest.raises(ValueError):
        Q.count_spix(lab - 1)
    gap = np.zeros_like(lab)
    gap[:, :2] = 2                              # id 1 missing
    with pytest.raises(ValueError):
        Q.ue_and_sa(lab, gap)
    # a perfect labelling: UE 0, SA 1, EV 1 on a piecewise-constant video
    gt = np.repeat(np.repeat(np.arange(4).reshape(2, 2), 3, 0), 4, 1)[None].repeat(3, 0)
    pc = rng.uniform(0, 1, (4, 3))[gt].astype(np.float32)
    s = Q.compute_summary(pc, gt.astype(np.int32), gt.astype(np.int32))
    assert s["ue2d"] == 0.0 and s["ue3d"] == 0.0 and s["sa2d"] == 1.0 and s["sa3d"] == 1.0
    # pooled means are sum / (count + 1e-8), as sp_pooling: EV falls short of 1 by ~1e-9
    assert abs(s["ev"] - 1.0) < 1e-8 and s["szv"] == 0.0


# ---------------------------------------------------------------------------- GPU
def _engine_video(T=6, H=96, W=128):
    import torch
    from st_spix_gb300 import bist_cuda, synth
    vid, flows, regs = synth.voronoi_video(H, W, T, 30, 0.03, seed=3, max_shift=3.0)
    lab = bist_cuda.bist_forward(torch.from_numpy(vid).cuda(), torch.from_numpy(flows).cuda(),
                                 8, 10, 0.5, 0.009 ** 2, math.log(0.5), 0.0, True, False)
    return vid, lab.cpu().numpy(), (regs % 5).astype(np.int32)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES + ["engine_96x128x6"])
def test_evaluate_matches_oracle(name):
    from st_spix_gb300 import metrics
    if name in CASES:
        g = _golden(name)
        vid, spix, gt = g["vid"], g["spix"], g["gt"]
    else:
        vid, spix, gt = _engine_video()
    ref = Q.compute_summary(vid, spix, gt)
    got = metrics.computeSummary(vid, gt, spix)
    for k in SCORES:
        assert _close(got[k], ref[k], 1e-9), (k, got[k], ref[k])
    if name in CASES:     # the reference's own numbers
        g = _golden(name)
        for k in PINNED:
            assert _close(got[k], float(g[k]), 1e-9), (k, got[k], float(g[k]))
    nogt = metrics.evaluate(vid, spix)
    assert nogt.ue2d == -1.0 and _close(nogt.ev, ref["ev"], 1e-9)


@pytest.mark.gpu
def test_count_and_size_scores_exact():
    import torch
    from st_spix_gb300 import metrics
    g = _golden("ragged_17x23x5")
    spix = g["spix"]
    counts = metrics.count_spix(spix)
    np.testing.assert_array_equal(counts.cpu().numpy(), Q.count_spix(spix))
    tex, szv = metrics.scoreMeanDurationAndSizeVariation(counts)
    rt, rs = Q.mean_duration_and_size_variation(Q.count_spix(spix))
    assert tex == rt and _close(szv, rs, 1e-12)
    assert metrics.averge_unique_spix_v1(counts) == float(np.mean(np.sum(Q.count_spix(spix) > 0, 1)))
    with pytest.raises(RuntimeError):
        metrics.count_spix(torch.from_numpy(spix - 100).cuda())


@pytest.mark.gpu
def test_sp_pooling_and_psnr():
    import torch
    from st_spix_gb300 import metrics
    vid, spix, _ = _engine_video(T=3, H=48, W=64)
    pooled, down = metrics.sp_pooling(vid, spix)
    S = int(spix.max()) + 1
    for t in range(3):
        s = spix[t].reshape(-1)
        cnt = np.bincount(s, minlength=S)
        for c in range(3):
            ref = np.bincount(s, weights=vid[t].reshape(-1, 3)[:, c].astype(np.float64),
                              minlength=S) / (cnt + 1e-8)
            np.testing.assert_allclose(down[t, :, c].cpu().numpy(), ref, rtol=1e-6, atol=1e-7)
        np.testing.assert_array_equal(pooled[t].cpu().numpy(), down[t].cpu().numpy()[spix[t]])
    psnr, pooled2 = metrics.scoreSpixPoolingQuality(vid, spix)
    assert _close(psnr, Q.pooling_psnr(vid, spix), 1e-9)
    assert pooled2.shape == (3, 3, 48, 64)
    assert _close(metrics.scoreExplainedVariance(torch.from_numpy(vid).cuda(), spix),
                  Q.explained_variance(vid, spix), 1e-9)
    assert _close(metrics.scoreExplainedVariance3D(vid, spix),
                  Q.explained_variance_3d(vid, spix), 1e-9)


@pytest.mark.gpu
def test_ue_sa_interface_and_errors():
    from st_spix_gb300 import metrics, _lib
    g = _golden("bist_40x56x4")
    spix, gt = g["spix"] - g["spix"].min(), g["gt"]
    T = spix.shape[0]
    got = metrics.scoreUEandSA(spix, None, gt, None, np.unique(gt), np.arange(T))
    ref = Q.ue_and_sa(spix, gt)
    for a, b in zip(got, ref):
        assert _close(a, b, 1e-12)
    assert metrics.scoreUEandSA(spix, None, gt[:2], None, np.unique(gt), np.arange(T)) == \
        (-1., -1., -1., -1.)
    gap = gt.copy()
    gap[gap == 1] = 0                            # id 1 never occurs
    with pytest.raises(_lib.StspixError):
        metrics.evaluate(g["vid"], spix, gap)
