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
