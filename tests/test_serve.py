"""Serving form on the GPU: streams of different sizes admitted under a budget and
served by continuous batching on two lanes give, for every stream, exactly the
labels of bist_forward on that stream alone."""
import numpy as np
import pytest

from st_spix_gb300 import synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from st_spix_gb300 import _lib, bist_cuda, serve  # noqa: E402

CFG = dict(niters=8, sp_size=12, sm_period=4, prop_niters=0)


def streams():
    specs = [(48, 64, 0), (56, 72, 1), (40, 40, 2), (64, 48, 3), (48, 64, 4)]
    out = []
    for H, W, s in specs:
        v, f, _ = synth.voronoi_video(H, W, 4, 16, 0.03, seed=s, max_shift=3.0)
        out.append((torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda()))
    return out


def alone(v, f):
    return bist_cuda.bist_forward(v, f, CFG["niters"], CFG["sp_size"], 0.5, 0.009 ** 2,
                                  float(np.log(0.5)), 0.0, True, False, sm_period=4,
                                  prop_niters=0).cpu().numpy()


@pytest.mark.parametrize("tight", [False, True])
def test_serving_results_equal_alone(tight):
    data = streams()
    ref = [alone(v, f) for v, f in data]
    probe = serve.Server(1 << 40, max_batch=3, lanes=2, **CFG)
    req0 = [serve.StreamRequest(i, v, f, fps=1e5, keep_labels=True) for i, (v, f) in
            enumerate(data)]
    per = max(probe.stream_bytes(r) for r in req0)
    slot = max(_lib.footprint(v.shape[1], v.shape[2], 12)[1] for v, _ in data)
    budget = 2 * 3 * slot + (2 * per if tight else 100 * per)
    srv = serve.Server(budget, max_batch=3, lanes=2, **CFG)
    for r in req0:
        srv.add(r)
    st = srv.run()
    assert st["frames"] == 5 * 4
    assert st["peak_bytes"] <= budget
    for i in range(5):
        np.testing.assert_array_equal(srv.labels[i].cpu().numpy(), ref[i], err_msg=f"stream {i}")
    if not tight:
        assert st["mean_batch"] > 1.0   # frames of different streams shared batches
