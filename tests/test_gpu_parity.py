"""GPU parity: the CUDA engine (called through the C ABI) against the CPU oracle on
identical seeded inputs.  Integer results (labels, counts, sums) must be bit-exact;
float results must match to the last bits (both sides evaluate the same IEEE
expressions without contraction; FP64 log() may differ by one ulp between the CUDA
and host math libraries, hence the relative tolerance of 1e-12 on doubles)."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import small_frame, small_video

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from st_spix_gb300 import _lib, bist_cuda  # noqa: E402

F64_RTOL = 1e-12


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def ctx():
    c = _lib.Context(0)
    yield c
    c.close()


def stream():
    return torch.cuda.current_stream().cuda_stream


def ocfg(**kw):
    return O.default_config(**kw)


def gcfg(**kw):
    return _lib.default_config(**kw)


def compare_params(gp: dict, op: dict):
    for name, g in gp.items():
        g = g.detach().cpu().numpy().reshape(-1)
        o = np.asarray(op[name]).reshape(-1)
        assert g.shape == o.shape, (name, g.shape, o.shape)
        if g.dtype == np.float64:
            np.testing.assert_allclose(g, o, rtol=F64_RTOL, atol=0, err_msg=name)
        else:
            np.testing.assert_array_equal(g, o, err_msg=name)


@pytest.mark.parametrize("H,W,sp", [(72, 96, 15), (61, 83, 9), (240, 320, 15), (100, 37, 25)])
def test_init_seg_matches_bruteforce(ctx, H, W, sp):
    lab = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    n = C.c_int(0)
    ctx.check(ctx.lib.stspix_init_seg(ctx.handle, stream(), lab.data_ptr(), H, W, sp, C.byref(n)))
    torch.cuda.synchronize()
    ref, nref = O.init_seg(H, W, sp)
    assert n.value == nref
    np.testing.assert_array_equal(lab.cpu().numpy(), ref)


@pytest.mark.parametrize("mode", [0, 1])
def test_find_border(ctx, mode):
    rng = np.random.default_rng(3)
    lab = rng.integers(-1, 5, size=(33, 47)).astype(np.int32)
    g = cuda(lab)
    b = torch.zeros(lab.shape, dtype=torch.uint8, device="cuda")
    ctx.check(ctx.lib.stspix_find_border(ctx.handle, stream(), g.data_ptr(), b.data_ptr(),
                                         lab.shape[0], lab.shape[1], mode))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(b.cpu().numpy(), O.find_border(lab, mode))


def gpu_partial(ctx, img, cfg, iters, extra):
    H, W = img.shape[:2]
    cap = 30 * O.hex_count(H, W, cfg.sp_size)
    d = {"count": torch.zeros(cap, dtype=torch.int32), "valid": torch.zeros(cap, dtype=torch.uint8),
         "prior_count": torch.zeros(cap, dtype=torch.float32),
         "mu_app": torch.zeros(cap * 3, dtype=torch.float32),
         "mu_shape": torch.zeros(cap * 2, dtype=torch.float64),
         "sigma_shape": torch.zeros(cap * 3, dtype=torch.float64),
         "logdet": torch.zeros(cap, dtype=torch.float64),
         "sums": torch.zeros(cap * 8, dtype=torch.int64)}
    d = {k: v.cuda() for k, v in d.items()}
    ds = _lib.DumpC()
    for k, v in d.items():
        setattr(ds, k, v.data_ptr())
    ds.capacity = cap
    gimg = cuda(img)
    lab = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    nbuf, mx = C.c_int(0), C.c_int(0)
    st = ctx.lib.stspix_bass_partial(ctx.handle, stream(), gimg.data_ptr(), H, W, C.byref(cfg),
                                     iters, extra, lab.data_ptr(), C.byref(ds), C.byref(nbuf),
                                     C.byref(mx))
    assert st == 0, ctx.lib.stspix_last_error(ctx.handle)
    return lab.cpu().numpy(), {k: v.cpu().numpy() for k, v in d.items()}, nbuf.value, mx.value


@pytest.mark.parametrize("iters,extra", [(0, 0), (0, 1), (1, 0), (1, 1), (3, 1), (5, 1),
                                         (7, 1), (10, 1), (15, 0)])
def test_bass_partial_state(ctx, iters, extra):
    img = small_frame()
    g_lab, g, g_nbuf, g_mx = gpu_partial(ctx, img, gcfg(niters=15), iters, extra)
    st, o_lab, o, o_nbuf, o_mx = O.bass_partial(img, ocfg(niters=15), iters, extra)
    assert st == 0
    assert g_nbuf == o_nbuf and g_mx == o_mx
    np.testing.assert_array_equal(g_lab, o_lab)
    for k in ("count", "valid", "sums", "prior_count", "mu_app"):
        np.testing.assert_array_equal(g[k], o[k], err_msg=k)
    for k in ("mu_shape", "sigma_shape", "logdet"):
        np.testing.assert_allclose(g[k], o[k], rtol=F64_RTOL, atol=0, err_msg=k)


@pytest.mark.parametrize("seed,niters,period", [(0, 15, 4), (1, 24, 4), (2, 40, 20)])
def test_run_bass_parity(seed, niters, period):
    img = small_frame(H=96, W=128, nseeds=30, seed=seed)
    glab, gp = bist_cuda.run_bass(cuda(img), niters=niters, sm_period=period)
    st, olab, op, n = O.run_bass(img, ocfg(niters=niters, sm_period=period))
    assert st == 0
    assert gp.n == n
    np.testing.assert_array_equal(glab.cpu().numpy(), olab)
    compare_params(gp.as_dict(), op)


def test_run_bass_config0_100_iters():
    from st_spix_gb300 import synth
    img, _ = synth.config0()
    glab, gp = bist_cuda.run_bass(cuda(img), niters=100, sm_period=20)
    st, olab, op, n = O.run_bass(img, ocfg(niters=100, sm_period=20))
    assert gp.n == n
    np.testing.assert_array_equal(glab.cpu().numpy(), olab)
    compare_params(gp.as_dict(), op)


@pytest.mark.parametrize("lo,hi", [(-0.6, 1.4), (0.0, 1.0)])
def test_run_bass_colours_outside_unit_range(lo, hi):
    """Colours outside [0, 1] (e.g. CIELAB scaled as the colour front end writes it)
    take the statistics' general fixed-point path; [0, 1] the 32-bit one.  Both must
    give the oracle's labels and parameters bit for bit, also with a frame whose blocks
    mix both kinds."""
    img = small_frame(H=96, W=128, nseeds=30, seed=3)
    img = (lo + (hi - lo) * img).astype(np.float32)
    if lo < 0:
        img[:, :64] = np.clip(img[:, :64], 0.0, 1.0)    # left half in range, right half not
    glab, gp = bist_cuda.run_bass(cuda(img), niters=24, sm_period=4)
    st, olab, op, n = O.run_bass(img, ocfg(niters=24, sm_period=4))
    assert st == 0
    assert gp.n == n
    np.testing.assert_array_equal(glab.cpu().numpy(), olab)
    compare_params(gp.as_dict(), op)


def _oracle_params_for_gpu(op, n, dev="cuda"):
    p = bist_cuda.SuperpixelParams(n, dev)
    p.n = n
    for name, dt, per in bist_cuda.PARAM_FIELDS:
        getattr(p, "_" + name).copy_(torch.from_numpy(np.ascontiguousarray(op[name]).reshape(-1)))
    return p


def test_shift_fill_and_prop_parity():
    vid, flows = small_video(T=2)
    st, lab0, op0, n0 = O.run_bass(vid[0], ocfg())
    assert st == 0
    gp0 = _oracle_params_for_gpu(op0, n0)
    gfilled, gshifted = bist_cuda.shift_and_fill(cuda(lab0), gp0, cuda(flows[0]))
    st, ofilled, oshifted, op0u = O.shift_and_fill(lab0, op0, n0, flows[0])
    assert st == 0
    np.testing.assert_array_equal(gshifted.cpu().numpy(), oshifted)
    np.testing.assert_array_equal(gfilled.cpu().numpy(), ofilled)
    compare_params({"prior_counts": gp0.field("prior_counts"),
                    "invalid_counts": gp0.field("invalid_counts")},
                   {"prior_counts": op0u["prior_counts"][:n0],
                    "invalid_counts": op0u["invalid_counts"][:n0]})
    for niters in (4, 8, 12):
        glab, gp = bist_cuda.run_prop(cuda(vid[1]), niters, gfilled, gshifted, gp0)
        st, olab, op, n = O.run_prop(vid[1], ocfg(), niters, ofilled, oshifted, op0u, n0)
        assert st == 0
        assert gp.n == n
        np.testing.assert_array_equal(glab.cpu().numpy(), olab)
        compare_params(gp.as_dict(), op)


@pytest.mark.parametrize("video_mode", [False, True])
def test_bist_forward_parity(video_mode):
    vid, flows = small_video(T=5)
    gv, gf = cuda(vid), cuda(flows)
    out = bist_cuda.bist_forward(gv, gf, 15, 15, 0.5, 0.009 ** 2, float(np.log(0.5)), 0.0,
                                 video_mode, False)
    st, ref, used = O.bist_forward(vid, flows, ocfg(niters=15), video_mode)
    assert st == 0
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


def test_get_marked_video_parity():
    vid, flows = small_video(T=2)
    gv = cuda(vid)
    spix = bist_cuda.bist_forward(gv, cuda(flows), 8, 15, 0.5, 0.009 ** 2, float(np.log(0.5)),
                                  0.0, True, False)
    color = torch.tensor([0.0, 0.0, 1.0])
    marked = bist_cuda.get_marked_video(gv, spix, color)
    ref = O.get_marked_video(vid, spix.cpu().numpy(), np.array([0, 0, 1], np.float32))
    np.testing.assert_array_equal(marked.cpu().numpy(), ref)


def test_input_checks():
    vid = torch.zeros((1, 8, 8, 3))
    with pytest.raises(RuntimeError):
        bist_cuda.bist_forward(vid, vid, 4, 15, 0.5, 1e-4, -0.69, 0.0, False, False)
    g = torch.zeros((1, 8, 8, 3), device="cuda")
    nc = torch.zeros((1, 8, 8, 2), device="cuda").transpose(1, 2)
    with pytest.raises(RuntimeError):
        bist_cuda.bist_forward(g, nc, 4, 15, 0.5, 1e-4, -0.69, 0.0, False, False)


def test_concurrent_streams_match_sequential():
    """Four host threads, each with its own CUDA stream and engine context, process
    four different videos at once; every result equals the single-stream run."""
    import threading
    vids = [small_video(T=3, seed=s) for s in range(4)]
    seq = []
    for v, f in vids:
        seq.append(bist_cuda.bist_forward(cuda(v), cuda(f), 10, 15, 0.5, 0.009 ** 2,
                                          float(np.log(0.5)), 0.0, True, False).cpu().numpy())
    out = [None] * 4
    err = []
    gate = threading.Barrier(4)

    def run(i):
        try:
            s = torch.cuda.Stream()
            v, f = vids[i]
            with torch.cuda.stream(s):
                gv, gf = cuda(v), cuda(f)
                gate.wait()
                for _ in range(3):
                    o = bist_cuda.bist_forward(gv, gf, 10, 15, 0.5, 0.009 ** 2,
                                               float(np.log(0.5)), 0.0, True, False)
                s.synchronize()
                out[i] = o.cpu().numpy()
        except Exception as e:  # pragma: no cover - reported below
            err.append(repr(e))

    th = [threading.Thread(target=run, args=(i,)) for i in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not err, err
    for i in range(4):
        np.testing.assert_array_equal(out[i], seq[i])


def _log_tuple(lg):
    return (lg.nsplits, lg.nmerges, lg.nrevived, lg.nminted, lg.near_ties)


def test_run_bass_config0_decisions_fire_and_match_the_oracle():
    """Config 0 with the reference's own period (split at idx % 4 == 0, merge at 2): the
    split and merge paths fire, and the counts of accepted splits / merges equal the
    oracle's."""
    from st_spix_gb300 import synth
    img, _ = synth.config0()
    glab, gp = bist_cuda.run_bass(cuda(img), niters=100, sm_period=4)
    glog = _log_tuple(bist_cuda.frame_log())
    st, olab, op, n = O.run_bass(img, ocfg(niters=100, sm_period=4))
    assert st == 0 and gp.n == n
    np.testing.assert_array_equal(glab.cpu().numpy(), olab)
    assert glog == _log_tuple(O.last_log())
    assert glog[0] > 0 and glog[1] > 0, glog


def test_propagated_chain_relabels_fire_and_match_the_oracle():
    """A fast-moving video (shifts up to 6 px per frame) frame by frame through
    shift_and_fill + run_prop with the reference's 4/8/12 ladder: labels identical to
    the oracle on every frame, and revivals, new ids, splits and merges all occur."""
    from st_spix_gb300 import synth
    vid, flows, _ = synth.voronoi_video(120, 160, 8, 30, 0.05, 1, max_shift=6.0)
    st, olab, op, n = O.run_bass(vid[0], ocfg(niters=20))
    assert st == 0
    glab, gp = bist_cuda.run_bass(cuda(vid[0]), niters=20)
    np.testing.assert_array_equal(glab.cpu().numpy(), olab)
    totals = np.zeros(5, np.int64)
    for t in range(1, vid.shape[0]):
        gf, gs = bist_cuda.shift_and_fill(glab, gp, cuda(flows[t - 1]))
        st, of, osh, opu = O.shift_and_fill(olab, op, n, flows[t - 1])
        assert st == 0
        np.testing.assert_array_equal(gs.cpu().numpy(), osh)
        np.testing.assert_array_equal(gf.cpu().numpy(), of)
        hole = float((osh < 0).mean())
        niters = 12 if hole > 0.20 else (4 if hole < 0.01 else 8)
        glab, gp = bist_cuda.run_prop(cuda(vid[t]), niters, gf, gs, gp)
        glog = _log_tuple(bist_cuda.frame_log())
        st, olab, op, n = O.run_prop(vid[t], ocfg(), niters, of, osh, opu, n)
        assert st == 0 and gp.n == n
        np.testing.assert_array_equal(glab.cpu().numpy(), olab)
        assert glog == _log_tuple(O.last_log()), (t, glog)
        compare_params(gp.as_dict(), op)
        totals += np.array(glog)
    assert totals[0] > 0 and totals[1] > 0 and totals[2] > 0 and totals[3] > 0, totals


def test_streaming_workload_size_matches_the_oracle():
    """The streaming workload at full size (480x854, 400 seeds, 20 iterations,
    split/merge every 10, 20 iterations on propagated frames), first 3 frames through
    bist_forward, against the oracle; the last frame's decisions fire."""
    from st_spix_gb300 import synth
    vid, flows, _ = synth.config1(0, T=3)
    out = bist_cuda.bist_forward(cuda(vid), cuda(flows), 20, 20, 0.5, 0.009 ** 2,
                                 float(np.log(0.5)), 0.0, True, False, sm_period=10,
                                 prop_niters=20)
    glog = _log_tuple(bist_cuda.frame_log())
    st, ref, _ = O.bist_forward(vid, flows, ocfg(niters=20, sp_size=20, sm_period=10,
                                                 prop_niters=20), True)
    assert st == 0
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
    assert glog == _log_tuple(O.last_log())
    assert glog[0] > 0 and glog[1] > 0, glog
