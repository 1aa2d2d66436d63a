"""Regenerate the golden fixtures of tests/test_golden.py from the CPU oracle.

    python tests/golden/make_golden.py

These vectors are outputs of the oracle's restatement, not of the reference: they
pin the CPU tests and the GPU engine against the oracle.  The oracle itself is pinned
to the reference's own kernels on the GPU (tests/test_ref_pin.py, test_ref_decisions.py,
test_ref_e2e.py), which need a GPU and so cannot produce CPU fixtures.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402
from st_spix_gb300 import synth  # noqa: E402


def main():
    img, _ = synth.voronoi_frame(64, 96, 20, 0.05, seed=11)
    cfg = O.default_config(niters=20)
    st, lab, p, n = O.run_bass(img, cfg)
    assert st == 0
    np.savez_compressed(os.path.join(HERE, "bass_64x96.npz"), img=img, labels=lab, nspix=n,
                        niters=20, **{k: v for k, v in p.items()})
    vid, flows, _ = synth.voronoi_video(48, 64, 3, 12, 0.03, seed=12, max_shift=3.0)
    cfg = O.default_config(niters=12)
    st, out, used = O.bist_forward(vid, flows, cfg, True)
    assert st == 0
    np.savez_compressed(os.path.join(HERE, "bist_video_48x64x3.npz"), vid=vid, flows=flows,
                        labels=out, niters=12, niters_used=used)
    print("wrote golden fixtures:", n, "superpixels;", used)


if __name__ == "__main__":
    main()
