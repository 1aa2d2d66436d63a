"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py): the
oracle must reproduce them (CPU) and the GPU engine must match them (GPU)."""
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(HERE, name)))


def test_oracle_reproduces_bass_golden():
    g = load("bass_64x96.npz")
    st, lab, p, n = O.run_bass(g["img"], O.default_config(niters=int(g["niters"])))
    assert st == 0 and n == int(g["nspix"])
    np.testing.assert_array_equal(lab, g["labels"])
    for k, v in p.items():
        np.testing.assert_array_equal(v, g[k], err_msg=k)


def test_oracle_reproduces_video_golden():
    g = load("bist_video_48x64x3.npz")
    st, out, used = O.bist_forward(g["vid"], g["flows"], O.default_config(niters=int(g["niters"])),
                                   True)
    assert st == 0
    np.testing.assert_array_equal(out, g["labels"])
    np.testing.assert_array_equal(used, g["niters_used"])


@pytest.mark.gpu
def test_gpu_matches_bass_golden():
    import torch
    from st_spix_gb300 import bist_cuda
    g = load("bass_64x96.npz")
    lab, p = bist_cuda.run_bass(torch.from_numpy(g["img"]).cuda(), niters=int(g["niters"]))
    assert p.n == int(g["nspix"])
    np.testing.assert_array_equal(lab.cpu().numpy(), g["labels"])
    for k, v in p.as_dict().items():
        v = v.cpu().numpy().reshape(-1)
        if v.dtype == np.float64:
            np.testing.assert_allclose(v, g[k], rtol=1e-12, atol=0, err_msg=k)
        else:
            np.testing.assert_array_equal(v, g[k], err_msg=k)


@pytest.mark.gpu
def test_gpu_matches_video_golden():
    import torch
    from st_spix_gb300 import bist_cuda
    g = load("bist_video_48x64x3.npz")
    out = bist_cuda.bist_forward(torch.from_numpy(g["vid"]).cuda(),
                                 torch.from_numpy(g["flows"]).cuda(), int(g["niters"]), 15, 0.5,
                                 0.009 ** 2, float(np.log(0.5)), 0.0, True, False)
    np.testing.assert_array_equal(out.cpu().numpy(), g["labels"])


@pytest.mark.gpu
@pytest.mark.parametrize("schedule", [0, 1, 2])
@pytest.mark.parametrize("niters_seg", [3, 4, 5])
def test_gpu_sweep_schedules_match_oracle(schedule, niters_seg):
    """One sweep per launch, two sweeps per launch (8-pixel halo) and the autotuned mix
    give the oracle's labels, with even and odd sweep counts (the final copy, the single
    after pairs).  Each case runs on a new CUDA stream, i.e. a new engine context, so the
    autotuner's first update (tuning launches) is exercised for every sweep count."""
    import torch
    from st_spix_gb300 import bist_cuda
    g = load("bist_video_48x64x3.npz")
    cfg = O.default_config(niters=int(g["niters"]), niters_seg=niters_seg)
    st, ref, _ = O.bist_forward(g["vid"], g["flows"], cfg, True)
    assert st == 0
    with torch.cuda.stream(torch.cuda.Stream()):
        out = bist_cuda.bist_forward(torch.from_numpy(g["vid"]).cuda(),
                                     torch.from_numpy(g["flows"]).cuda(), int(g["niters"]), 15,
                                     0.5, 0.009 ** 2, float(np.log(0.5)), 0.0, True, False,
                                     niters_seg=niters_seg, sweep_schedule=schedule)
        torch.cuda.current_stream().synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.gpu
@pytest.mark.parametrize("schedule", [1, 2])
@pytest.mark.parametrize("tile", [16, 32, 64])
def test_gpu_forced_sweep_tile_matches_oracle(tile, schedule):
    """A forced tile width (no autotuning), one or two sweeps per launch, gives the
    oracle's labels."""
    import torch
    from st_spix_gb300 import bist_cuda
    g = load("bist_video_48x64x3.npz")
    st, ref, _ = O.bist_forward(g["vid"], g["flows"], O.default_config(niters=int(g["niters"])),
                                True)
    assert st == 0
    with torch.cuda.stream(torch.cuda.Stream()):
        out = bist_cuda.bist_forward(torch.from_numpy(g["vid"]).cuda(),
                                     torch.from_numpy(g["flows"]).cuda(), int(g["niters"]), 15,
                                     0.5, 0.009 ** 2, float(np.log(0.5)), 0.0, True, False,
                                     sweep_tile=tile, sweep_schedule=schedule)
        torch.cuda.current_stream().synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.gpu
@pytest.mark.parametrize("tile", [0, 16, 32, 64])
def test_gpu_work_queue_sweep_matches_oracle(tile):
    """The persistent work-queue sweep (resident blocks taking tiles from an atomic
    counter that resets itself after each launch) gives the oracle's labels, with the
    autotuned width and every forced width, over many consecutive launches of one
    context (a counter left non-zero would skip tiles of the next launch)."""
    import torch
    from st_spix_gb300 import bist_cuda
    g = load("bist_video_48x64x3.npz")
    st, ref, _ = O.bist_forward(g["vid"], g["flows"], O.default_config(niters=int(g["niters"])),
                                True)
    assert st == 0
    with torch.cuda.stream(torch.cuda.Stream()):
        for _ in range(2):
            out = bist_cuda.bist_forward(torch.from_numpy(g["vid"]).cuda(),
                                         torch.from_numpy(g["flows"]).cuda(), int(g["niters"]),
                                         15, 0.5, 0.009 ** 2, float(np.log(0.5)), 0.0, True,
                                         False, sweep_tile=tile, sweep_schedule=1,
                                         sweep_queue=1)
            torch.cuda.current_stream().synchronize()
            np.testing.assert_array_equal(out.cpu().numpy(), ref)
