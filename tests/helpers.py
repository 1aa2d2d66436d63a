"""Shared helpers of the test suite (inputs, comparisons)."""
import numpy as np

from st_spix_gb300 import synth


def small_frame(H=72, W=96, nseeds=24, sigma=0.05, seed=0):
    img, _ = synth.voronoi_frame(H, W, nseeds, sigma, seed)
    return img


def small_video(T=4, H=72, W=96, nseeds=24, sigma=0.03, seed=0):
    vid, flows, _ = synth.voronoi_video(H, W, T, nseeds, sigma, seed, max_shift=3.0)
    return vid, flows


def assert_params_equal(a: dict, b: dict, n: int, exact_fields=("counts", "ids")):
    for k in a:
        x, y = np.asarray(a[k]), np.asarray(b[k])
        assert x.shape == y.shape, (k, x.shape, y.shape)
        if k in exact_fields:
            np.testing.assert_array_equal(x, y, err_msg=k)
        else:
            np.testing.assert_allclose(x, y, rtol=1e-6, atol=1e-9, err_msg=k)


def label_agreement(a, b) -> float:
    """Fraction of pixels on which two label maps agree after one-to-one matching of
    their ids by overlap (greedy, largest overlap first): the comparison for label maps
    whose ids are not comparable (the reference numbers split products in atomic
    order)."""
    a = np.asarray(a).ravel().astype(np.int64)
    b = np.asarray(b).ravel().astype(np.int64)
    _, ai = np.unique(a, return_inverse=True)
    _, bi = np.unique(b, return_inverse=True)
    pairs, counts = np.unique(ai * (bi.max() + 1) + bi, return_counts=True)
    order = np.argsort(-counts, kind="stable")
    used_a, used_b, agree = set(), set(), 0
    nb = bi.max() + 1
    for k in order:
        x, y = divmod(int(pairs[k]), int(nb))
        if x in used_a or y in used_b:
            continue
        used_a.add(x)
        used_b.add(y)
        agree += int(counts[k])
    return agree / a.size
