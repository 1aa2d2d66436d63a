"""CPU tests of the oracle (the CPU restatement the GPU engine is checked against).

Known answers come from independent numpy restatements of the reference's formulas
(init_seg.cu, seg_utils.cu, fill_missing.cu, split_disconnected.cu,
shift_labels.cu) and from invariants the reference's algorithm guarantees."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from st_spix_gb300 import synth
from tests.helpers import small_frame, small_video


def np_hex(H, W, sp):
    """init_seg.cu:20-75 restated with numpy (brute force, last minimum wins)."""
    Hh = math.sqrt(sp ** 2 / (1.5 * math.sqrt(3.0)))
    w = math.sqrt(3.0) * Hh
    nx = int(math.floor(W / w)) + 2
    ny = int(math.floor(H / (1.5 * Hh))) + 2
    idx = np.arange(nx * ny)
    cx = (idx % nx) * w + np.where((idx // nx) % 2 == 0, 0.5 * w, 0.0)
    cy = (idx // nx) * 1.5 * Hh
    ys, xs = np.mgrid[0:H, 0:W]
    d2 = (xs[..., None] - cx) ** 2 + (ys[..., None] - cy) ** 2
    # last index attaining the minimum
    rev = d2[..., ::-1]
    lab = nx * ny - 1 - rev.argmin(-1)
    return lab.astype(np.int32), nx * ny


@pytest.mark.parametrize("H,W,sp", [(24, 32, 5), (30, 17, 7), (40, 40, 15)])
def test_init_seg_known_answer(H, W, sp):
    lab, n = O.init_seg(H, W, sp)
    ref, nref = np_hex(H, W, sp)
    assert n == nref == O.hex_count(H, W, sp)
    np.testing.assert_array_equal(lab, ref)


def np_border(lab, mode):
    H, W = lab.shape
    pad = np.pad(lab, 1, constant_values=-1)
    C = lab
    N, S, Wl, E = pad[:-2, 1:-1], pad[2:, 1:-1], pad[1:-1, :-2], pad[1:-1, 2:]
    if mode == 0:
        b = (C != N) | (C != S) | (C != E) | (C != Wl)
        b[0, :] = b[-1, :] = True
        b[:, 0] = b[:, -1] = True
        return b.astype(np.uint8)
    out = np.zeros_like(lab, dtype=bool)
    for nb in (N, S, E, Wl):
        out |= (nb >= 0) & (C > nb)
    return out.astype(np.uint8)


@pytest.mark.parametrize("mode", [0, 1])
def test_find_border_known_answer(mode):
    rng = np.random.default_rng(0)
    lab = rng.integers(0, 4, size=(19, 23)).astype(np.int32)
    np.testing.assert_array_equal(O.find_border(lab, mode), np_border(lab, mode))


def test_run_bass_invariants():
    img = small_frame()
    st, lab, p, n = O.run_bass(img, O.default_config(niters=15))
    assert st == 0
    H, W = lab.shape
    assert lab.min() == 0 and lab.max() == n - 1
    counts = np.bincount(lab.ravel(), minlength=n)
    np.testing.assert_array_equal(p["counts"], counts)
    assert (counts > 0).all()
    # means against an FP64 numpy computation (tolerance 1e-5 relative)
    for k in range(n):
        m = lab == k
        ys, xs = np.nonzero(m)
        np.testing.assert_allclose(p["mu_app"][3 * k:3 * k + 3],
                                   img[m].astype(np.float64).mean(0), rtol=1e-5, atol=1e-7)
        assert p["mu_shape"][2 * k] == pytest.approx(xs.mean(), rel=1e-12)
        assert p["mu_shape"][2 * k + 1] == pytest.approx(ys.mean(), rel=1e-12)
    # prior := estimate after the frame (sparams_io.cu:583-640)
    np.testing.assert_array_equal(p["prior_mu_app"], p["mu_app"])
    np.testing.assert_array_equal(p["prior_sigma_shape"], p["sigma_shape"])
    np.testing.assert_array_equal(p["ids"], np.arange(n))


def test_run_bass_sample_cov_is_sample_covariance():
    img = small_frame(seed=2)
    st, lab, p, n = O.run_bass(img, O.default_config(niters=8))
    for k in range(0, n, 7):
        ys, xs = np.nonzero(lab == k)
        c = np.cov(np.stack([xs, ys]).astype(np.float64), bias=True)
        np.testing.assert_allclose(p["sample_sigma_shape"][3 * k:3 * k + 3],
                                   [c[0, 0], c[0, 1], c[1, 1]], rtol=1e-9, atol=1e-9)


def test_oracle_deterministic():
    img = small_frame(seed=5)
    a = O.run_bass(img, O.default_config(niters=12))
    b = O.run_bass(img, O.default_config(niters=12))
    np.testing.assert_array_equal(a[1], b[1])
    for k in a[2]:
        np.testing.assert_array_equal(a[2][k], b[2][k])


def test_superpixels_are_connected():
    """Boundary moves keep every superpixel 4-connected (simple-point test)."""
    from scipy import ndimage
    img = small_frame(seed=1)
    st, lab, p, n = O.run_bass(img, O.default_config(niters=20))
    for k in range(n):
        _, ncomp = ndimage.label(lab == k)
        assert ncomp <= 2  # splits seed halves by geodesic distance; allow one detached piece


def test_fill_missing_known_answer():
    # two labels, a two-column hole; centres at x=1 and x=4.5
    seg = np.array([[0, 0, -1, -1, 1, 1]] * 3, np.int32)
    centers = np.array([[1.0, 1.0], [4.5, 1.0]])
    st, out, it = O.fill_missing(seg, centers)
    assert st == 0 and (out >= 0).all() and it == 2
    np.testing.assert_array_equal(out[:, 2], 0)   # only label 0 is adjacent
    np.testing.assert_array_equal(out[:, 3], 1)   # nearer to centre 1


def test_fill_missing_tie_keeps_first_candidate():
    # equidistant centres: the strict '>' keeps the first candidate in N,S,W,E
    # order, here the west neighbour filled earlier in the same iteration
    seg = np.array([[0, 0, -1, -1, 1, 1]] * 3, np.int32)
    centers = np.array([[1.0, 1.0], [5.0, 1.0]])
    st, out, it = O.fill_missing(seg, centers)
    assert st == 0
    np.testing.assert_array_equal(out[:, 3], 0)


def test_fill_missing_no_progress_reports_error():
    seg = -np.ones((4, 4), np.int32)
    st, out, it = O.fill_missing(seg, np.zeros((1, 2)))
    assert st == 4  # STSPIX_ERR_NOPROGRESS (the reference exits the process here)


def test_invalidate_disconnected_known_answer():
    seg = np.array([[0, 0, 1, 0],
                    [0, 0, 1, 1],
                    [1, 1, 1, 1]], np.int32)
    out = O.invalidate_disconnected(seg, 2)
    # label 0: regions of size 4 (top-left) and 1 (top-right, 8-connected to nothing
    # of label 0) -> the single pixel is invalidated
    exp = seg.copy()
    exp[0, 3] = -1
    np.testing.assert_array_equal(out, exp)


def test_shift_translates_labels():
    vid, flows = small_video(T=2)
    st, lab0, p0, n0 = O.run_bass(vid[0], O.default_config(niters=6))
    flow = np.zeros_like(flows[0])
    flow[..., 0] = 2.0  # everything moves 2 px right
    st, filled, shifted, p = O.shift_and_fill(lab0, p0, n0, flow)
    assert st == 0
    np.testing.assert_array_equal(shifted[:, 2:], lab0[:, :-2])
    assert (shifted[:, :2] == -1).all()
    assert (filled >= 0).all()
    assert np.isclose(p["invalid_counts"][:n0].sum() > 0, True)


def test_bist_forward_video_invariants():
    vid, flows = small_video(T=4)
    st, out, used = O.bist_forward(vid, flows, O.default_config(niters=10), True)
    assert st == 0
    assert (out >= 0).all()
    assert used[0] == 10 and set(used[1:]) <= {4, 8, 12}


def test_config0_generator_shape():
    img, reg = synth.config0()
    assert img.shape == (240, 320, 3) and img.dtype == np.float32
    assert 0 <= img.min() and img.max() <= 1
    assert len(np.unique(reg)) <= 200
    img2, _ = synth.config0()
    np.testing.assert_array_equal(img, img2)
