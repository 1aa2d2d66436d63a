"""Pins the CPU oracle against the reference's OWN kernels.

oracle/ref_build.py compiles the reference's bist kernels (unmodified sources,
-fmad=false) into sm_103a cubins under oracle/_ref; oracle/ref_harness.cpp runs them on
the GPU through the driver API, sequenced as the reference's host code does.  Each
test feeds the same seeded state to the reference kernels and to the oracle.

Exactness: labels, counts, distances, roots and integer-derived FP64 values are
identical (FP64 log may differ by one ulp between libraries: rtol 1e-12).  The
reference accumulates colour sums with FP32 atomicAdd in arbitrary order, so colour
means are compared within 1e-5 relative (the tolerance for FP32 sufficient
statistics against an FP64 oracle).  Skipped where oracle/_ref was not built (the
reference sources are needed to build it)."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import ref_harness as R
from tests.helpers import small_frame, small_video

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not R.cubins_present(), reason="oracle/_ref not built")]

S2 = 0.009 ** 2


@pytest.mark.parametrize("H,W,sp", [(72, 96, 15), (61, 83, 9), (120, 160, 20), (100, 37, 25)])
def test_init_seg_pinned(H, W, sp):
    ref, nref = R.init_seg(H, W, sp)
    lab, n = O.init_seg(H, W, sp)
    assert n == nref
    np.testing.assert_array_equal(lab, ref)


@pytest.mark.parametrize("mode", [0, 1])
def test_find_border_pinned(mode):
    rng = np.random.default_rng(7)
    lab = rng.integers(-1, 6, size=(45, 67)).astype(np.int32)
    np.testing.assert_array_equal(O.find_border(lab, mode), R.find_border(lab, mode))


def _state(seed, iters, H=72, W=96):
    img = small_frame(H=H, W=W, nseeds=24, seed=seed)
    st, lab, d, nbuf, mx = O.bass_partial(img, O.default_config(), iters, 1)
    assert st == 0
    return img, lab, d, nbuf, mx


@pytest.mark.parametrize("seed,iters,prop", [(0, 0, 0), (0, 3, 0), (1, 6, 0), (2, 4, 1)])
def test_update_params_pinned(seed, iters, prop):
    img, lab, d, nbuf, mx = _state(seed, iters)
    valid = d["valid"].astype(np.int32)
    prop_v = np.full(nbuf, prop, np.int32)
    icov = np.tile([1.0, 0.0, 1.0], nbuf)
    rng = np.random.default_rng(seed)
    a = rng.uniform(5, 40, nbuf)
    c = rng.uniform(5, 40, nbuf)
    b = rng.uniform(-0.5, 0.5, nbuf) * np.sqrt(a * c)
    sample = np.stack([a, b, c], 1).reshape(-1)
    args = (img, lab, nbuf, 15, S2, valid, prop_v, d["prior_count"], icov, sample)
    ref = R.update_params(*args)
    ora = O.update_params_given(*args)
    for k in ("count", "valid"):
        np.testing.assert_array_equal(ora[k], ref[k], err_msg=k)
    np.testing.assert_array_equal(ora["mu_shape"], ref["mu_shape"])
    live = ora["valid"].astype(bool)
    np.testing.assert_allclose(ora["sigma_shape"].reshape(-1, 3)[live],
                               ref["sigma_shape"].reshape(-1, 3)[live], rtol=1e-12, atol=0)
    np.testing.assert_allclose(ora["logdet"][live], ref["logdet"][live], rtol=1e-12, atol=0)
    np.testing.assert_allclose(ora["mu_app"].reshape(-1, 3)[live],
                               ref["mu_app"].reshape(-1, 3)[live], rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("seed,iters", [(0, 1), (0, 5), (1, 9), (3, 2)])
def test_update_seg_pinned(seed, iters):
    """Given identical parameters the reference's sweeps and the oracle's produce the
    same labels (4 sweeps x 4 parity phases)."""
    img, lab, d, nbuf, mx = _state(seed, iters)
    args = (img, lab, nbuf, 4, S2, 0.5, d["count"], d["mu_app"], d["mu_shape"],
            d["sigma_shape"], d["logdet"])
    ref = R.update_seg(*args)
    ora = O.update_seg_given(*args)
    assert (ref != lab).sum() > 0  # the sweep moved pixels
    np.testing.assert_array_equal(ora, ref)


@pytest.mark.parametrize("direction", [1, -1, 2, -2])
def test_split_bfs_pinned(direction):
    img, lab, d, nbuf, mx = _state(4, 6)
    valid = d["valid"].astype(np.int32)
    ref = R.split_bfs(lab, nbuf, valid, d["mu_shape"], direction, mx)
    ora = O.split_bfs(lab, nbuf, valid, d["mu_shape"], direction)
    assert ref.max() > 5
    np.testing.assert_array_equal(ora, ref)


def test_fill_pinned():
    vid, flows = small_video(T=2)
    st, lab0, p0, n0 = O.run_bass(vid[0], O.default_config(niters=8))
    flow = np.zeros_like(flows[0])
    flow[..., 0] = 3.0
    flow[: flow.shape[0] // 2, :, 1] = -2.0
    st, filled, shifted, p = O.shift_and_fill(lab0, p0, n0, flow)
    centers = (p0["mu_shape"].reshape(-1, 2) + 0.0).copy()
    rit, ref = R.fill(shifted, centers)
    ost, ora, oit = O.fill_missing(shifted, centers)
    assert ost == 0 and rit == oit and (shifted < 0).sum() > 0
    np.testing.assert_array_equal(ora, ref)


def test_components_pinned():
    rng = np.random.default_rng(3)
    seg = (rng.random((40, 52)) < 0.45).astype(np.int32) + 2 * (rng.random((40, 52)) < 0.2)
    seg[5:9, 5:30] = -1
    np.testing.assert_array_equal(O.cc_roots(seg), R.cc_roots(seg))


def test_color_pinned():
    """The engine's colour kernels against the reference's (same device powf)."""
    torch = pytest.importorskip("torch")
    from st_spix_gb300 import bist_cuda
    rng = np.random.default_rng(1)
    rgb = rng.uniform(0, 1, size=(40, 56, 3)).astype(np.float32)
    rgb[0, 0, 0] = np.nan                     # left unwritten by both
    lab_ref = R.rgb2lab(rgb)
    lab = bist_cuda.rgb2lab(torch.from_numpy(rgb).cuda()).cpu().numpy()
    np.testing.assert_array_equal(lab, lab_ref)
    lab[0, 0] = lab_ref[0, 0] = 0.5
    np.testing.assert_array_equal(bist_cuda.lab2rgb(torch.from_numpy(lab).cuda()).cpu().numpy(),
                                  R.lab2rgb(lab_ref))
    u8 = rng.integers(0, 256, size=(24, 30, 3)).astype(np.uint8)
    np.testing.assert_array_equal(bist_cuda.rescale_u8(torch.from_numpy(u8).cuda()).cpu().numpy(),
                                  R.rescale_u8(u8))
