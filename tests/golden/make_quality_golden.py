"""Golden vectors of the superpixel quality metrics, computed by the reference's own
metric functions (gauenk/st_spix st_spix/spix_utils/evaluate.py) on small seeded
label videos.

    python tests/golden/make_quality_golden.py [reference checkout, default /root/reference]

evaluate.py imports modules that are not needed by the functions used here and are
absent in this environment (pandas, easydict, h5py, PIL, skvideo, the bass_cuda and
prop_cuda extensions); they are replaced by empty stub modules, and the st_spix
package is registered without running its __init__ (which imports the unbuilt
extensions).  Two adjustments, neither of which changes what the functions compute:
tensors are kept on the CPU (scoreMeanDurationAndSizeVariation moves its input to
"cuda"; the move is redirected to the CPU), and torch's default dtype is float64, so
that the integer-by-integer divisions of the reference (which produce the default
float type) are evaluated in FP64, the precision of this project's implementation.

Functions pinned: count_spix (evaluate.py:71), scoreMeanDurationAndSizeVariation
(:284), scoreExplainedVariance (:230, with sp_pooling from st_spix/sp_pooling.py),
scoreUEandSA (:372), averge_unique_spix_v1 (:184), and the spix - spix.min() offset
and argument preparation of computeSummary (:94-126).  Not pinnable:
scoreExplainedVariance3D (:254) needs the unbuilt prop_cuda video pooling, and
scoreSpixPoolingQuality (:214) calls st_spix.metrics.compute_psnrs, which is not
in the reference repository.
"""
import os
import sys
import types
import importlib.util

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def load_reference_evaluate(root):
    import torch
    pkg_dir = os.path.join(root, "st_spix")
    for name in ["pandas", "easydict", "h5py", "PIL", "PIL.Image", "skvideo",
                 "skvideo.measure", "bass_cuda", "prop_cuda"]:
        sys.modules.setdefault(name, types.ModuleType(name))

    class EDict(dict):
        __getattr__ = dict.__getitem__
        __setattr__ = dict.__setitem__

    sys.modules["easydict"].EasyDict = EDict
    sys.modules["PIL"].Image = sys.modules["PIL.Image"]
    sys.modules["skvideo"].measure = sys.modules["skvideo.measure"]
    pkg = types.ModuleType("st_spix")
    pkg.__path__ = [pkg_dir]
    sys.modules["st_spix"] = pkg
    sub = types.ModuleType("st_spix.spix_utils")
    sub.__path__ = [os.path.join(pkg_dir, "spix_utils")]
    sys.modules["st_spix.spix_utils"] = sub
    spec = importlib.util.spec_from_file_location(
        "st_spix.spix_utils.evaluate", os.path.join(pkg_dir, "spix_utils", "evaluate.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)

    orig_to = torch.Tensor.to

    def to_cpu(self, *a, **k):
        a = tuple("cpu" if isinstance(x, str) and x.startswith("cuda") else x for x in a)
        if isinstance(k.get("device"), str) and k["device"].startswith("cuda"):
            k["device"] = "cpu"
        return orig_to(self, *a, **k)

    torch.Tensor.to = to_cpu
    torch.set_default_dtype(torch.float64)
    return mod


def reference_metrics(ev, vid, spix, seg):
    """The computeSummary steps (evaluate.py:94-165) that the pinned functions cover,
    on CPU tensors."""
    import torch as th
    spix = spix - spix.min()
    sizes = ev.count_spix(spix)
    seg_sizes = ev.count_spix(seg)[:, 1:]
    gt_ids = np.unique(seg)
    gtpos = np.arange(seg.shape[0])
    vid_t = th.from_numpy(vid).double()
    spix_t = th.from_numpy(spix).int()
    seg_t = th.from_numpy(seg).int()
    tex, szv = ev.scoreMeanDurationAndSizeVariation(sizes)
    evar = ev.scoreExplainedVariance(vid_t, spix_t)
    ue2d, sa2d, ue3d, sa3d = ev.scoreUEandSA(spix_t, sizes, seg_t, seg_sizes, gt_ids, gtpos)
    return dict(counts=sizes.numpy().astype(np.int64), tex=tex, szv=szv, ev=evar,
                ue2d=ue2d, sa2d=sa2d, ue3d=ue3d, sa3d=sa3d,
                spnum=int(spix.max()) + 1, ave_nsp=ev.averge_unique_spix_v1(sizes))


def cases():
    from oracle import oracle as O
    from st_spix_gb300 import synth
    out = {}
    # superpixels of a propagated video (the oracle's bist_forward), ground truth = the
    # generator's regions folded onto 4 objects
    vid, flows, regs = synth.voronoi_video(40, 56, 4, 10, 0.03, seed=21, max_shift=3.0)
    st, lab, _ = O.bist_forward(vid, flows, O.default_config(niters=8, sp_size=8), True)
    assert st == 0
    out["bist_40x56x4"] = (vid, lab.astype(np.int32), (regs % 4).astype(np.int32))
    # ragged ids: offset labels (min 7), ids that never occur, an id alive in one frame,
    # ground truth with 3 objects on random blocks
    rng = np.random.Generator(np.random.PCG64(5))
    T, H, W = 5, 17, 23
    base = (np.arange(H)[:, None] // 6) * 4 + (np.arange(W)[None, :] // 6)
    lab = np.stack([base + 7 + 3 * (base % 2) * (t % 2) for t in range(T)]).astype(np.int32)
    lab[2, :3, :3] = 200
    vid = rng.uniform(0, 1, size=(T, H, W, 3)).astype(np.float32)
    gt = (rng.integers(0, 3, size=(T, (H + 3) // 4, (W + 3) // 4))
          .repeat(4, 1).repeat(4, 2)[:, :H, :W]).astype(np.int32)
    out["ragged_17x23x5"] = (vid, lab, gt)
    return out


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    ev = load_reference_evaluate(root)
    arrays = {}
    for name, (vid, lab, gt) in cases().items():
        m = reference_metrics(ev, vid, lab, gt)
        arrays[f"{name}/vid"] = vid
        arrays[f"{name}/spix"] = lab
        arrays[f"{name}/gt"] = gt
        for k, v in m.items():
            arrays[f"{name}/{k}"] = np.asarray(v)
        print(name, {k: v for k, v in m.items() if k != "counts"})
    np.savez_compressed(os.path.join(HERE, "quality_ref.npz"), **arrays)


if __name__ == "__main__":
    main()
