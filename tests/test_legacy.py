"""Legacy prop_cuda surface (st_spix/csrc/prop via pybind_prop.cpp): the exact entries
against the oracle restatement (integers and labels bit-exact, FP32 means within
1e-6), the BASS drivers against the engine's own run_bass / run_prop."""
import math

import numpy as np
import pytest

from oracle import legacy as LG


def test_oracle_shift_known_answer():
    sp = np.array([[0, 0, 1], [2, 2, 1]], np.int32)
    flow = np.array([[1, 0], [0, 1], [0, -1]], np.int32)     # (dx, dy) per superpixel
    sh, cnt = LG.shift_labels(sp, flow)
    # 0 moves right, 1 moves down (off the frame at the bottom), 2 moves up
    np.testing.assert_array_equal(sh, [[2, 2, 0], [-1, -1, 1]])
    np.testing.assert_array_equal(cnt, [[1, 2, 1], [0, 0, 1]])


def test_oracle_fill_known_answer():
    sp = np.array([[0, -1, -1, 1]], np.int32)
    centers = np.array([[0.0, 0.0], [3.0, 0.0]], np.float32)
    missing = np.array([[1, 2]], np.int32)
    out, it, rem = LG.fill_missing(sp, centers, missing, 0)
    np.testing.assert_array_equal(out, [[0, 0, 1, 1]])
    assert rem == 0 and it >= 1
    # a hole with no labelled neighbour never fills: the count repeats and the loop stops
    out2, _, rem2 = LG.fill_missing(np.full((1, 3), -1, np.int32), centers,
                                    np.array([[0, 1, 2]], np.int32), 0)
    assert rem2 == 3 and (out2 == -1).all()


def _legacy_case(seed=0, H=40, W=56):
    from st_spix_gb300 import synth
    rng = np.random.default_rng(seed)
    img, reg = synth.voronoi_frame(H, W, 12, 0.03, seed=seed)
    spix = reg.astype(np.int32)
    nspix = int(spix.max()) + 1
    flow = rng.integers(-3, 4, size=(nspix, 2)).astype(np.int32)
    return img, spix, flow


@pytest.mark.gpu
def test_shift_labels_and_fill_missing_exact():
    import torch
    from st_spix_gb300 import prop_cuda
    img, spix, flow = _legacy_case()
    sh, cnt = prop_cuda.shift_labels(torch.from_numpy(spix)[None].cuda(),
                                     torch.from_numpy(flow)[None].cuda())
    rsh, rcnt = LG.shift_labels(spix, flow)
    np.testing.assert_array_equal(sh[0].cpu().numpy(), rsh)
    np.testing.assert_array_equal(cnt[0].cpu().numpy(), rcnt)
    # fill the holes of the shifted labels from the superpixels' mean positions
    nspix = flow.shape[0]
    ys, xs = np.mgrid[: spix.shape[0], : spix.shape[1]]
    centers = np.stack([np.bincount(spix.ravel(), xs.ravel(), nspix) / np.bincount(spix.ravel(), minlength=nspix),
                        np.bincount(spix.ravel(), ys.ravel(), nspix) / np.bincount(spix.ravel(), minlength=nspix)],
                       1).astype(np.float32)
    miss = np.nonzero(rsh.ravel() == -1)[0].astype(np.int32)[None]
    out = prop_cuda.fill_missing(sh, torch.from_numpy(centers).cuda(),
                                 torch.from_numpy(miss).cuda(), 2000)
    ref, _, rem = LG.fill_missing(rsh, centers, miss, 2000)
    np.testing.assert_array_equal(out[0].cpu().numpy(), ref)
    assert rem == 0 and (out >= 0).all()


@pytest.mark.gpu
def test_border_init_colour_pooling():
    import torch
    from st_spix_gb300 import bist_cuda, prop_cuda
    from oracle import oracle as O
    img, spix, _ = _legacy_case(1)
    b = prop_cuda.find_border(torch.from_numpy(spix)[None].cuda())
    np.testing.assert_array_equal(b[0].cpu().numpy(), LG.find_border(spix))
    (lab,) = prop_cuda.init_spix(torch.from_numpy(img)[None].cuda(), 9)
    ref, _ = O.init_seg(img.shape[0], img.shape[1], 9)
    np.testing.assert_array_equal(lab[0].cpu().numpy(), ref)
    # legacy rgb_to_lab reads RGB; the bist one reads the first channel as blue
    g = torch.from_numpy(img).cuda()
    lab_legacy = prop_cuda.rgb_to_lab(g)
    lab_bist = bist_cuda.rgb2lab(g.flip(-1).contiguous())
    assert torch.equal(lab_legacy, lab_bist)
    assert torch.equal(prop_cuda.lab_to_rgb(lab_legacy), bist_cuda.lab2rgb(lab_legacy))
    rng = np.random.default_rng(2)
    vid = rng.uniform(0, 1, (2, 3, 12, 14, 5)).astype(np.float32)
    seg = rng.integers(-1, 9, (2, 3, 12, 14)).astype(np.int32)
    seg[0, 0, 0, 0] = 8
    pooled, down, counts = prop_cuda.sp_video_pooling(torch.from_numpy(vid).cuda(),
                                                      torch.from_numpy(seg).cuda())
    rp, rd, rc = LG.sp_video_pooling(vid, seg, 9)
    np.testing.assert_array_equal(counts.cpu().numpy(), rc)
    np.testing.assert_allclose(down.cpu().numpy(), rd, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(pooled.cpu().numpy(), rp, rtol=1e-6, atol=1e-7)
    back = prop_cuda.downsampled_video_to_pooled(down, torch.from_numpy(seg).cuda())
    assert torch.equal(back, pooled)


@pytest.mark.gpu
def test_bass_drivers_run_the_engine():
    import torch
    from st_spix_gb300 import bist_cuda, prop_cuda, synth
    vid, flows, _ = synth.voronoi_video(48, 64, 2, 10, 0.03, seed=5, max_shift=2.0)
    img0 = torch.from_numpy(vid[0]).cuda()
    args = dict(niters=8, niters_seg=4, sm_start=0, sp_size=10, sigma2_app=0.009 ** 2,
                sigma2_size=0.0, potts=0.5, alpha_hastings=math.log(0.5))
    spix, params = prop_cuda.bass(img0[None], *args.values())
    ref, rp = bist_cuda.run_bass(img0, niters=8, niters_seg=4, sm_start=0, sp_size=10,
                                 sigma2_app=0.009 ** 2, potts=0.5, alpha=math.log(0.5))
    assert spix.shape == (1, 48, 64) and torch.equal(spix[0], ref)
    n = rp.n
    for k in prop_cuda.KEYS:
        t = getattr(params, k)
        assert t.shape[0] == n and t.is_cuda, k
    assert params.mu_app.shape == (n, 3) and params.mu_shape.dtype == torch.float64
    assert params.counts.dtype == torch.int32 and params.prior_counts.dtype == torch.float32
    assert torch.equal(params.counts, rp.field("counts"))
    # propagated frame: prop_bass on labels with no holes equals run_prop on them
    img1 = torch.from_numpy(vid[1]).cuda()
    s1, p1 = prop_cuda.prop_bass(img1[None], spix, params, 6, 4, 0, 10, 0.009 ** 2, 0.0, 0.5,
                                 math.log(0.5))
    r1, _ = bist_cuda.run_prop(img1, 6, spix[0].contiguous(), spix[0].contiguous(), rp,
                               niters_seg=4, sm_start=0, sp_size=10, sigma2_app=0.009 ** 2,
                               potts=0.5, alpha=math.log(0.5))
    assert torch.equal(s1[0], r1)
    # a SuperpixelParams rebuilt from its 17 tensors drives prop_bass as well
    rebuilt = prop_cuda.SuperpixelParams(*[getattr(params, k) for k in prop_cuda.KEYS])
    s2, _ = prop_cuda.prop_bass(img1[None], spix, rebuilt, 6, 4, 0, 10, 0.009 ** 2, 0.0, 0.5,
                                math.log(0.5))
    assert s2.shape == s1.shape and (s2 >= 0).all()
    out, _, log = prop_cuda.refine_missing(img1[None], spix, None, params, n, 5, 4, 10,
                                           0.009 ** 2, 0.5)
    assert out.shape == (1, 48, 64) and log.shape == (5, 1)


def _split_case():
    """A BASS labelling of a Voronoi frame with every three ids joined (superpixels
    spanning several colour regions) and the BASS params of the first ids as the
    previous params."""
    from oracle import oracle as O
    from st_spix_gb300 import synth
    img, _ = synth.voronoi_frame(64, 80, 12, 0.03, seed=3)
    st, lab0, op0, _ = O.run_bass(img, O.default_config(niters=8, sp_size=16))
    assert st == 0
    lab = (lab0 // 3).astype(np.int32)
    n = int(lab.max()) + 1
    per = {name: p for name, _, p in O.PARAM_FIELDS}
    prev = {k: np.ascontiguousarray(v[: n * per[k]]) for k, v in op0.items()}
    return img, lab, prev, n


def test_oracle_split_divides_coarse_superpixels():
    from oracle import oracle as O
    img, lab, prev, n = _split_case()
    outs = []
    for d in (0, 1):
        st, out, _, nout = O.legacy_split(img, O.default_config(sp_size=16), d, lab, prev, n)
        assert st == 0 and nout > n
        assert out.min() == 0 and out.max() == nout - 1
        # a split only divides: every new superpixel lies inside one old one
        for k in range(nout):
            assert len(np.unique(lab[out == k])) == 1
        outs.append(out)
    assert (outs[0] != outs[1]).any()    # the two directions bisect differently


@pytest.mark.gpu
@pytest.mark.parametrize("direction", [0, 1])
def test_split_matches_the_oracle(direction):
    import torch
    from oracle import oracle as O
    from st_spix_gb300 import bist_cuda, prop_cuda
    img, lab, prev, n = _split_case()
    gp = bist_cuda.SuperpixelParams(n, "cuda")
    gp.n = n
    for name, _, _ in bist_cuda.PARAM_FIELDS:
        getattr(gp, "_" + name).copy_(torch.from_numpy(prev[name].reshape(-1)))
    params = prop_cuda._legacy_params(gp, 0.009 ** 2)
    out, p = prop_cuda.split(torch.from_numpy(img)[None].cuda(), torch.from_numpy(lab)[None].cuda(),
                             params, direction, 16, 0.009 ** 2, 0.0, math.log(0.5))
    st, ref, rp, rn = O.legacy_split(img, O.default_config(sp_size=16), direction, lab, prev, n)
    assert st == 0 and rn > n
    np.testing.assert_array_equal(out[0].cpu().numpy(), ref)
    assert p.counts.shape[0] == rn
    np.testing.assert_array_equal(p.counts.cpu().numpy(), rp["counts"])
    np.testing.assert_allclose(p.mu_shape.cpu().numpy().reshape(-1), rp["mu_shape"],
                               rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_refine_is_propagated_bass_without_split_merge():
    import torch
    from oracle import oracle as O
    from st_spix_gb300 import bist_cuda, prop_cuda
    img, lab, prev, n = _split_case()
    gp = bist_cuda.SuperpixelParams(n, "cuda")
    gp.n = n
    for name, _, _ in bist_cuda.PARAM_FIELDS:
        getattr(gp, "_" + name).copy_(torch.from_numpy(prev[name].reshape(-1)))
    params = prop_cuda._legacy_params(gp, 0.009 ** 2)
    out, p, log = prop_cuda.refine(torch.from_numpy(img)[None].cuda(),
                                   torch.from_numpy(lab)[None].cuda(), params, 6, 4, 16,
                                   0.009 ** 2, 0.5)
    st, ref, rp, rn = O.run_prop(img, O.default_config(sp_size=16, sm_start=6), 6, lab, lab,
                                 prev, n)
    assert st == 0 and rn <= n and log.shape == (6, 1)
    np.testing.assert_array_equal(out[0].cpu().numpy(), ref)
    np.testing.assert_array_equal(p.counts.cpu().numpy(), rp["counts"])


# ---- run_update_prior, shift_tensor(_ordered), shift_order, split_disconnected -------
def _blocky(H, W, seed, nlab=12):
    rng = np.random.default_rng(seed)
    ys, xs = np.mgrid[0:H, 0:W]
    lab = ((ys // 7) * 5 + (xs // 9)) % nlab
    lab[rng.integers(0, H, 30), rng.integers(0, W, 30)] = rng.integers(0, nlab, 30)
    return lab.astype(np.int32)


@pytest.mark.gpu
@pytest.mark.parametrize("invert", [False, True])
def test_update_prior_matches_restatement(invert):
    import torch
    from st_spix_gb300 import prop_cuda
    rng = np.random.default_rng(3)
    n, prev = 40, 15
    spix = _blocky(30, 41, 3, nlab=37)
    p = prop_cuda.SuperpixelParams(*[None] * len(prop_cuda.KEYS))
    host = dict(mu_app=rng.random((n, 3)).astype(np.float32),
                prior_mu_app=rng.random((n, 3)).astype(np.float32),
                mu_shape=rng.random((n, 2)) * 30, prior_mu_shape=rng.random((n, 2)) * 30,
                sigma_shape=np.stack([rng.uniform(0.5, 2, n), rng.uniform(-0.3, 0.3, n),
                                      rng.uniform(0.5, 2, n)], 1),
                prior_sigma_shape=rng.random((n, 3)))
    host["sigma_shape"][3] = (0.1, 1.0, 0.1)     # negative determinant
    for k, v in host.items():
        setattr(p, k, torch.from_numpy(np.ascontiguousarray(v)).cuda())
    prop_cuda.run_update_prior(torch.from_numpy(spix[None]).cuda(), p, prev, invert)
    pma, pms, pss = LG.update_prior(spix, host["mu_app"], host["prior_mu_app"], host["mu_shape"],
                                   host["prior_mu_shape"], host["sigma_shape"],
                                   host["prior_sigma_shape"], prev, invert)
    np.testing.assert_array_equal(p.prior_mu_app.cpu().numpy(), pma)
    np.testing.assert_array_equal(p.prior_mu_shape.cpu().numpy(), pms)
    np.testing.assert_allclose(p.prior_sigma_shape.cpu().numpy(), pss, rtol=1e-15, atol=0)


@pytest.mark.gpu
def test_shift_tensor_and_order_match_restatement():
    import torch
    from st_spix_gb300 import prop_cuda
    rng = np.random.default_rng(4)
    H, W, F = 24, 31, 3
    spix = _blocky(H, W, 4, nlab=9)
    nspix = int(spix.max()) + 1
    flow = rng.integers(-3, 4, size=(nspix, 2)).astype(np.int32)
    x = rng.random((H, W, F)).astype(np.float32)
    g = lambda a: torch.from_numpy(np.ascontiguousarray(a)[None]).cuda()
    out, counts, contrib = prop_cuda.shift_tensor(g(x), g(spix), g(flow))
    ro, rc, rcon = LG.shift_tensor(x, spix, flow)
    np.testing.assert_array_equal(counts[0].cpu().numpy(), rc)
    np.testing.assert_array_equal(contrib[0].cpu().numpy(), rcon)
    np.testing.assert_array_equal(out[0].cpu().numpy(), ro)
    sizes = np.bincount(spix.reshape(-1), minlength=nspix).astype(np.int32)
    sel = prop_cuda.shift_order(contrib, g(sizes))
    rsel = LG.shift_order(rcon, sizes)
    np.testing.assert_array_equal(sel[0].cpu().numpy(), rsel)
    out2, counts2 = prop_cuda.shift_tensor_ordered(g(x), g(spix), g(flow), sel)
    ro2, rc2, _ = LG.shift_tensor(x, spix, flow, rsel)
    np.testing.assert_array_equal(counts2[0].cpu().numpy(), rc2)
    np.testing.assert_array_equal(out2[0].cpu().numpy(), ro2)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [5, 6])
def test_split_disconnected_matches_restatement(seed):
    import torch
    from st_spix_gb300 import prop_cuda
    H, W = 40, 52
    spix = _blocky(H, W, seed, nlab=14)
    # cut some labels into pieces further than 2 pixels apart
    spix[:, 20:24] = 13
    nspix = int(spix.max()) + 1
    ref_lab, ref_children, ref_starts = LG.split_disconnected(spix, nspix)
    t = torch.from_numpy(spix[None].copy()).cuda()
    lab, children, starts = prop_cuda.split_disconnected(t, nspix)
    np.testing.assert_array_equal(lab[0].cpu().numpy(), ref_lab)
    np.testing.assert_array_equal(starts.cpu().numpy(), ref_starts)
    np.testing.assert_array_equal(children.cpu().numpy(), ref_children)
    assert ref_children.shape[1] > 0
