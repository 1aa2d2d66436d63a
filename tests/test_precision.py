"""Accumulator precision study entry points: statistics of a labelling with the
int64 fixed-point accumulator equal the exact integer computation; the FP64 and FP32
accumulators are within their rounding; runs with the study accumulators complete."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import small_frame

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from st_spix_gb300 import _lib, bist_cuda  # noqa: E402


def stats(img, lab, n, acc):
    ctx = bist_cuda._ctx(torch.device("cuda", 0))
    out = torch.empty(7 * n, dtype=torch.float64, device="cuda")
    H, W = lab.shape
    ctx.check(ctx.lib.stspix_label_stats(ctx.handle, bist_cuda._stream(0), img.data_ptr(),
                                         lab.data_ptr(), H, W, n, acc, out.data_ptr()))
    return out.view(n, 7).cpu().numpy()


def test_label_stats_accumulators():
    img = small_frame(H=96, W=128, nseeds=30, seed=3)
    lab, params = bist_cuda.run_bass(torch.from_numpy(img).cuda(), niters=6, sp_size=12)
    L = lab.cpu().numpy()
    n = int(L.max()) + 1
    g_img = torch.from_numpy(img).cuda()
    s0, s1, s2 = (stats(g_img, lab, n, a) for a in (0, 1, 2))
    v = img.reshape(-1, 3).astype(np.float32)
    k = L.ravel()
    cnt = np.bincount(k, minlength=n).astype(np.float64)
    q = np.rint(v * np.float32(2.0 ** 28)).astype(np.int64)
    qq = np.rint((v * v) * np.float32(2.0 ** 20)).astype(np.int64)
    for c in range(3):
        exact = np.zeros(n, np.int64)
        np.add.at(exact, k, q[:, c])
        np.testing.assert_array_equal(s0[:, 1 + c], np.ldexp(exact.astype(np.float64), -28))
        exact2 = np.zeros(n, np.int64)
        np.add.at(exact2, k, qq[:, c])
        np.testing.assert_array_equal(s0[:, 4 + c], np.ldexp(exact2.astype(np.float64), -20))
        ref = np.bincount(k, weights=v[:, c].astype(np.float64), minlength=n)
        np.testing.assert_allclose(s2[:, 1 + c], ref, rtol=1e-12)
        np.testing.assert_allclose(s1[:, 1 + c], ref, rtol=1e-4)
    np.testing.assert_array_equal(s0[:, 0], cnt)


@pytest.mark.parametrize("acc", [1, 2])
def test_study_accumulators_run(acc):
    img = torch.from_numpy(small_frame(H=72, W=96, seed=5)).cuda()
    lab0, _ = bist_cuda.run_bass(img, niters=8, sp_size=12)
    lab, p = bist_cuda.run_bass(img, niters=8, sp_size=12, accumulator=acc)
    agree = float((lab == lab0).float().mean().item())
    assert p.n > 10 and agree > 0.5
