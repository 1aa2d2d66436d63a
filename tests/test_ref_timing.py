"""Per-stage speed against the reference's OWN GPU kernels on the same box.

The reference's kernels (oracle/_ref/stock: the unmodified sources built with nvcc's
default flags, as its setup.py builds them) are timed per stage on one 480x854 frame of
the streaming workload and a BASS state after 10 iterations, each stage restarted from
the same labels and parameters (oracle/ref_runner.py Ref.time_stages): update_params,
update_seg's 4 sweeps, one split step (its host BFS loop reads a done flag back after
every distance step) and one merge step.  The engine runs the same frame (20
iterations, split/merge every 10) with per-family CUDA-event profiling, alone and as
one frame of a batch of 8; per BASS pass = (sweep + statistics + posterior) / 20.

Printed as a table (the figures behind the per-stage speed-ups reported for this
build); asserted: the engine is faster per BASS pass and per split step."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import ref_runner as RR
from st_spix_gb300 import synth

torch = pytest.importorskip("torch")
pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not RR.available("stock"), reason="oracle/_ref not built")]

S2 = 0.009 ** 2
LA = float(np.log(0.5))


def _engine_families(imgs, reps=3):
    from st_spix_gb300 import batch, bist_cuda
    dev = torch.device("cuda")
    ctx = bist_cuda._ctx(dev)
    cfg = dict(niters=20, sp_size=20, sm_period=10)
    fr = [batch.Frame(img=im, sp_size=20) for im in imgs]
    batch.process_batch(fr, **cfg)          # warm-up: workspaces, tuner
    torch.cuda.synchronize()
    tot = {}
    for _ in range(reps):
        ctx.profile(True)
        fr = [batch.Frame(img=im, sp_size=20) for im in imgs]
        batch.process_batch(fr, **cfg)
        torch.cuda.synchronize()
        for k, (n, ms) in ctx.profile_get().items():
            a = tot.setdefault(k, [0, 0.0])
            a[0] += n
            a[1] += ms
        ctx.profile(False)
    return {k: (n // reps, ms / reps) for k, (n, ms) in tot.items()}


def test_stage_times_against_the_reference_kernels():
    vid, _, _ = synth.config1(0, T=1)
    img = vid[0]
    cfg = O.default_config(niters=20, sp_size=20, sm_period=10)
    st, lab, d, nbuf, mx = O.bass_partial(img, cfg, 10)
    assert st == 0
    R = RR.Ref("stock")
    ref = R.time_stages(img, lab, nbuf, d["valid"], d["prior_count"], mx, 20, S2, 0.5, LA,
                        reps=10)
    dimg = torch.from_numpy(img).cuda()
    one = _engine_families([dimg])
    eight = _engine_families([dimg] * 8)
    ref_pass = ref["update_params"][0] + ref["update_seg_4_sweeps"][0]

    def per_pass(f, nframes):
        return (f["sweep"][1] + f["stats"][1] + f["posterior"][1]) / 20 / nframes

    def per_split(f, nframes):
        return f["split"][1] / nframes          # one split step per frame (idx 10)

    def per_merge(f, nframes):
        return f["merge"][1] / 2 / nframes       # two merge steps per frame (idx 5, 15)

    rows = [("BASS pass (update_params + 4 sweeps)", ref_pass, per_pass(one, 1), per_pass(eight, 8)),
            ("  update_params", ref["update_params"][0],
             (one["stats"][1] + one["posterior"][1]) / 20, None),
            ("  update_seg (4 sweeps)", ref["update_seg_4_sweeps"][0], one["sweep"][1] / 20, None),
            ("split step (GPU)", ref["split_step"][0], per_split(one, 1), per_split(eight, 8)),
            ("split step (host wall, reference)", ref["split_step"][1], None, None),
            ("merge step", ref["merge_step"][0], per_merge(one, 1), per_merge(eight, 8))]
    print("\nstage | reference ms | engine ms (frame alone) | engine ms per frame (batch of 8) |"
          " speed-up alone | speed-up batched")
    for name, r, e1, e8 in rows:
        sp1 = f"{r / e1:.1f}x" if e1 else "-"
        sp8 = f"{r / e8:.1f}x" if e8 else "-"
        f1 = f"{e1:.4f}" if e1 is not None else "-"
        f8 = f"{e8:.4f}" if e8 is not None else "-"
        print(f"{name} | {r:.4f} | {f1} | {f8} | {sp1} | {sp8}")
    assert per_pass(one, 1) < ref_pass
    assert per_split(one, 1) < ref["split_step"][0]
