"""Batched form: frames of uneven size (and video streams with resident state) run
as one batch give exactly the labels of the plain per-frame path, alone or in any
mix, and the plain path keeps matching the oracle (tested elsewhere), so the batch
matches the oracle too (checked directly here on a small mixed batch)."""
import numpy as np
import pytest

from oracle import oracle as O
from st_spix_gb300 import synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from st_spix_gb300 import batch, bist_cuda  # noqa: E402


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


CFG = dict(niters=12, sm_period=4)


def uneven_frames(n, seed=0, lo=40, hi=130):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        H = int(rng.integers(lo, hi)) // 8 * 8
        W = int(rng.integers(lo, hi)) // 8 * 8
        img, _ = synth.voronoi_frame(H, W, int(rng.integers(10, 60)),
                                     float(rng.uniform(0.02, 0.08)), seed * 100 + i)
        out.append((img, int(rng.choice([9, 12, 16]))))
    return out


def test_batch_independent_frames_match_single():
    frames = uneven_frames(7, seed=1)
    singles = []
    for img, sp in frames:
        lab, params = bist_cuda.run_bass(cuda(img), sp_size=sp, **CFG)
        singles.append((lab.cpu().numpy(), params.n))
    fr = [batch.Frame(img=cuda(img), sp_size=sp) for img, sp in frames]
    batch.process_batch(fr, **CFG)
    for f, (lab, n) in zip(fr, singles):
        assert f.status == 0
        assert f.nspix == n
        np.testing.assert_array_equal(f.labels.cpu().numpy(), lab)
    # and in another order / subset
    sub = [batch.Frame(img=fr[i].img, sp_size=fr[i].sp_size) for i in (5, 2, 6)]
    batch.process_batch(sub, **CFG)
    for f, i in zip(sub, (5, 2, 6)):
        np.testing.assert_array_equal(f.labels.cpu().numpy(), singles[i][0])


def test_batch_matches_oracle():
    frames = uneven_frames(3, seed=2)
    fr = [batch.Frame(img=cuda(img), sp_size=sp) for img, sp in frames]
    batch.process_batch(fr, **CFG)
    for f, (img, sp) in zip(fr, frames):
        st, lab, p, n = O.run_bass(img, O.default_config(sp_size=sp, **CFG))
        assert st == 0 and f.nspix == n
        np.testing.assert_array_equal(f.labels.cpu().numpy(), lab)


@pytest.mark.parametrize("prop_niters", [0, 6])
def test_batch_videos_match_bist_forward(prop_niters):
    """Three videos of different sizes advanced one frame per batch (plus an
    independent frame in every batch) equal bist_forward on each video."""
    kw = dict(niters=10, sm_period=4, prop_niters=prop_niters)
    specs = [(56, 72, 0), (64, 96, 1), (48, 40, 2)]
    T = 4
    vids = []
    for H, W, s in specs:
        v, f, _ = synth.voronoi_video(H, W, T, 20, 0.03, seed=s, max_shift=3.0)
        vids.append((cuda(v), cuda(f)))
    ref = []
    for v, f in vids:
        ref.append(bist_cuda.bist_forward(v, f, kw["niters"], 15, 0.5, 0.009 ** 2,
                                          float(np.log(0.5)), 0.0, True, False,
                                          sm_period=4, prop_niters=prop_niters).cpu().numpy())
    extra_img, _ = synth.voronoi_frame(64, 64, 15, 0.05, 9)
    extra_ref, _ = bist_cuda.run_bass(cuda(extra_img), sp_size=12, **kw)
    videos = [batch.Video(v.shape[1], v.shape[2]) for v, _ in vids]
    for t in range(T):
        fr = []
        for (v, f), vs in zip(vids, videos):
            fr.append(batch.Frame(img=v[t], flow=f[t - 1] if t > 0 else None, video=vs))
        fr.insert(1, batch.Frame(img=cuda(extra_img), sp_size=12))
        batch.process_batch(fr, **kw)
        np.testing.assert_array_equal(fr[1].labels.cpu().numpy(), extra_ref.cpu().numpy())
        del fr[1]
        for k, f in enumerate(fr):
            assert f.status == 0
            np.testing.assert_array_equal(f.labels.cpu().numpy(), ref[k][t],
                                          err_msg=f"video {k} frame {t}")
            assert videos[k].nspix == f.nspix
    for vs in videos:
        assert vs.frames == T
        vs.close()


def test_image_mode_bist_forward_batches():
    """Image mode runs its frames as batches: same labels as one frame at a time."""
    v, f, _ = synth.voronoi_video(64, 80, 5, 20, 0.03, seed=4, max_shift=3.0)
    vid = cuda(v)
    out = bist_cuda.bist_forward(vid, cuda(f), 9, 12, 0.5, 0.009 ** 2, float(np.log(0.5)), 0.0,
                                 False, False, sm_period=4)
    for t in range(5):
        lab, _ = bist_cuda.run_bass(vid[t].contiguous(), niters=9, sp_size=12, sm_period=4)
        np.testing.assert_array_equal(out[t].cpu().numpy(), lab.cpu().numpy())


def test_batch_rejects_same_video_twice():
    v, f, _ = synth.voronoi_video(32, 32, 2, 8, 0.03, seed=5, max_shift=2.0)
    vs = batch.Video(32, 32)
    fr = [batch.Frame(img=cuda(v[0]), video=vs), batch.Frame(img=cuda(v[1]), video=vs)]
    with pytest.raises(RuntimeError):
        batch.process_batch(fr, niters=4)
    vs.close()


def test_repeated_batch_steps_replay_a_graph_with_the_oracle_labels():
    """A stream with fixed propagated iterations repeats its batch step: the step is
    captured as a CUDA graph on its second occurrence and replayed after, with labels
    equal to the oracle's for every frame."""
    import torch
    T = 6
    kw = dict(niters=8, sm_period=4, prop_niters=6, sp_size=12)
    v, f, _ = synth.voronoi_video(48, 64, T, 16, 0.03, seed=7, max_shift=2.0)
    st, ref, _ = O.bist_forward(v, f, O.default_config(**kw), True)
    assert st == 0
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ctx = bist_cuda._ctx(torch.device("cuda", 0))
        r0 = ctx.graph_replays()
        vs = batch.Video(48, 64)
        vid, flo = cuda(v), cuda(f)
        for t in range(T):
            fr = [batch.Frame(img=vid[t], flow=flo[t - 1] if t else None, video=vs, sp_size=12)]
            batch.process_batch(fr, **kw)
            assert fr[0].status == 0
            np.testing.assert_array_equal(fr[0].labels.cpu().numpy(), ref[t], err_msg=f"frame {t}")
        vs.close()
        assert ctx.graph_replays() > r0


def test_batch_graphs_off_launch_eagerly_with_the_same_labels():
    T = 5
    kw = dict(niters=8, sm_period=4, prop_niters=6, sp_size=12)
    v, f, _ = synth.voronoi_video(48, 64, T, 16, 0.03, seed=8, max_shift=2.0)
    st, ref, _ = O.bist_forward(v, f, O.default_config(**kw), True)
    assert st == 0
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ctx = bist_cuda._ctx(torch.device("cuda", 0))
        ctx.set_batch_graphs(False)
        try:
            r0 = ctx.graph_replays()
            vs = batch.Video(48, 64)
            vid, flo = cuda(v), cuda(f)
            for t in range(T):
                fr = [batch.Frame(img=vid[t], flow=flo[t - 1] if t else None, video=vs,
                                  sp_size=12)]
                batch.process_batch(fr, **kw)
                np.testing.assert_array_equal(fr[0].labels.cpu().numpy(), ref[t])
            vs.close()
            assert ctx.graph_replays() == r0
        finally:
            ctx.set_batch_graphs(True)


def test_laddered_steps_replay_graphs_with_the_oracle_labels():
    """Propagated frames with the 4/8/12 ladder run as a head and a tail: both replay as
    CUDA graphs once their launch sequences repeat (the tail's key holds the ladder's
    outcome), with the oracle's labels on every pass."""
    T = 5
    kw = dict(niters=8, sm_period=4, sp_size=12)
    v, f, _ = synth.voronoi_video(48, 64, T, 16, 0.03, seed=9, max_shift=2.0)
    st, ref, _ = O.bist_forward(v, f, O.default_config(**kw), True)
    assert st == 0
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ctx = bist_cuda._ctx(torch.device("cuda", 0))
        r0 = ctx.graph_replays()
        vs = batch.Video(48, 64)
        vid, flo = cuda(v), cuda(f)
        for _ in range(3):
            vs.reset()
            for t in range(T):
                fr = [batch.Frame(img=vid[t], flow=flo[t - 1] if t else None, video=vs,
                                  sp_size=12)]
                batch.process_batch(fr, **kw)
                np.testing.assert_array_equal(fr[0].labels.cpu().numpy(), ref[t])
        vs.close()
        assert ctx.graph_replays() > r0


def test_uneven_batch_at_full_size_matches_oracle_and_plain_path():
    """A subset of the 64-frame uneven batch at its real sizes (H, W uniform in
    [240, 1080] rounded to multiples of 8, 100-800 seeds, noise 0.02-0.08, superpixel
    size from {12, 16, 20, 25}, 20 iterations, split/merge every 10): 4 frames in one
    batch give the oracle's labels and the plain per-frame path's, and each frame is
    the same alone and in the batch."""
    rng = np.random.Generator(np.random.PCG64(11))
    specs = []
    for i in range(4):
        H = int(rng.integers(240, 1081)) // 8 * 8
        W = int(rng.integers(240, 1081)) // 8 * 8
        specs.append((H, W, int(rng.integers(100, 801)), float(rng.uniform(0.02, 0.08)),
                      int(rng.choice([12, 16, 20, 25])), 7000 + i))
    imgs = [(synth.voronoi_frame(H, W, ns, sg, sd)[0], sp) for H, W, ns, sg, sp, sd in specs]
    cfg = dict(niters=20, sm_period=10)
    fr = [batch.Frame(img=cuda(img), sp_size=sp) for img, sp in imgs]
    batch.process_batch(fr, **cfg)
    for f, (img, sp) in zip(fr, imgs):
        assert f.status == 0
        st, lab, _, n = O.run_bass(img, O.default_config(sp_size=sp, **cfg))
        assert st == 0 and f.nspix == n
        np.testing.assert_array_equal(f.labels.cpu().numpy(), lab)
        alone, p = bist_cuda.run_bass(cuda(img), sp_size=sp, **cfg)
        np.testing.assert_array_equal(alone.cpu().numpy(), lab)
        assert p.n == n
    # the persistent work-queue sweep gives the same labels on the same batch
    fq = [batch.Frame(img=cuda(img), sp_size=sp) for img, sp in imgs]
    batch.process_batch(fq, sweep_queue=1, **cfg)
    for a, b in zip(fr, fq):
        assert b.status == 0
        assert torch.equal(a.labels, b.labels)
