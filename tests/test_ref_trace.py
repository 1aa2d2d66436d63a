"""Traces every place where the reference's own trajectory parts from this project's
deterministic rules (oracle/ref_trace.py), on config 0 (240x320, 100 iterations,
split/merge every 4 as the reference hard-codes).

Along the reference's run the oracle's rule is evaluated on the reference's own state
at every sweep, split and merge: each event found is a near tie by construction
(a sweep decision flipped by the last bits of an FP32 atomic mean, a Hastings ratio
within NEAR of the threshold, a merge target claimed by several superpixels, split ids
handed out in atomic order).  Asserted: the -fmad=false build's sweeps are identical to
the oracle's on the same parameters, every decision flip lies near the threshold, and a
run whose final labels differ from the engine's has at least one traced event (a run
with none ends with the engine's labels)."""
import numpy as np
import pytest

from oracle import ref_runner as RR
from st_spix_gb300 import synth
from tests.helpers import label_agreement

torch = pytest.importorskip("torch")
pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not RR.available("nofma"), reason="oracle/_ref not built")]

S2 = 0.009 ** 2
LA = float(np.log(0.5))
NEAR = 0.25


@pytest.mark.parametrize("variant", ["nofma", "stock"])
@pytest.mark.parametrize("seed", [0, 1, 2, 4])
def test_every_divergence_is_a_traced_tie(seed, variant):
    from oracle import ref_trace
    from st_spix_gb300 import bist_cuda
    img, _ = synth.config0(seed)
    T = ref_trace.Tracer(variant)
    lab_ref, events = T.run_bass_traced(img, 240, 320, 100, 15, S2, 0.5, LA, 0.0)
    eng, _ = bist_cuda.run_bass(torch.from_numpy(img).cuda(), niters=100, sm_period=4)
    agree = label_agreement(eng.cpu().numpy(), lab_ref)
    kinds = {}
    for e in events:
        kinds.setdefault(e[0], []).append(e[1])
    summary = {k: (len(v), round(max(v), 4)) for k, v in kinds.items()}
    print(f"config0 seed {seed} [{variant}]: engine~reference {agree:.5f}; traced events "
          f"(count, max size or margin) {summary}")
    for k in ("split", "merge"):
        for margin in kinds.get(k, []):
            assert margin < NEAR, (k, margin)
    if variant == "nofma":
        assert "sweep_arith" not in kinds, kinds.get("sweep_arith")
    if agree < 1.0:
        assert events, "labels differ without a traced tie"


@pytest.mark.parametrize("variant", ["nofma", "stock"])
def test_every_propagated_divergence_is_a_traced_tie(variant):
    """Propagated frames (shift_and_fill + run_prop, split/merge of split_merge_prop.cu):
    a fast-moving 120x160 video, every frame traced in lockstep from the reference's own
    recorded previous state, against the engine's frame from the same state."""
    from oracle import ref_trace
    from st_spix_gb300 import bist_cuda
    vid, flows, _ = synth.voronoi_video(120, 160, 8, 30, 0.05, 1, max_shift=6.0)
    R = RR.Ref(variant)
    R.bist_forward(vid, flows, 20, 15, 0.5, S2, LA, 0.0, True, record=True)
    recs = R.frames
    dev = torch.device("cuda")
    tr = ref_trace.Tracer(variant)
    rows = []
    for t in range(1, vid.shape[0]):
        prev = recs[t - 1]
        n_prev = int(len(prev["params"]["counts"]))
        pe = bist_cuda.SuperpixelParams(n_prev, dev)
        pe.n = n_prev
        for name, _, per in bist_cuda.PARAM_FIELDS:
            getattr(pe, "_" + name).copy_(torch.from_numpy(
                np.ascontiguousarray(prev["params"][name][: n_prev * per])))
        flow = torch.from_numpy(np.ascontiguousarray(flows[t - 1])).to(dev)
        filled, shifted = bist_cuda.shift_and_fill(torch.from_numpy(prev["labels"]).to(dev), pe,
                                                   flow)
        eng, _ = bist_cuda.run_prop(torch.from_numpy(vid[t]).to(dev), recs[t]["niters"], filled,
                                    shifted, pe, sp_size=15)
        lab_ref, events = tr.prop_frame_traced(vid[t], prev["labels"], prev["params"],
                                               flows[t - 1], recs[t]["niters"], 15, S2, 0.5, LA,
                                               0.0)
        agree = label_agreement(eng.cpu().numpy(), lab_ref)
        kinds = {}
        for e in events:
            kinds.setdefault(e[0], []).append(e[1])
        rows.append((t, round(agree, 5), {k: (len(v), round(max(v), 4)) for k, v in kinds.items()}))
        for k in ("split", "merge"):
            for margin in kinds.get(k, []):
                assert margin < NEAR, (t, k, margin)
        if variant == "nofma":
            assert "sweep_arith" not in kinds, (t, kinds.get("sweep_arith"))
        if agree < 1.0:
            assert events, (t, agree, "labels differ without a traced tie")
    print(f"video_120x160_T8 [{variant}] (frame, engine~reference, traced events): {rows}")
