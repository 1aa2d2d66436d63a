"""Label files in the reference's on-disk format: one CSV per frame, "%05d.csv", the
label matrix with no header and no index (scripts/run_spix/run_davis_spix.py:77-84),
so results can be scored by the reference's evaluation scripts."""
from __future__ import annotations

import os

import numpy as np


def save_spix_csv(root: str, spix) -> None:
    """spix: int [T, H, W] (numpy or a torch tensor) -> root/00000.csv, 00001.csv, ..."""
    if hasattr(spix, "detach"):
        spix = spix.detach().cpu().numpy()
    spix = np.asarray(spix)
    os.makedirs(root, exist_ok=True)
    for t in range(spix.shape[0]):
        np.savetxt(os.path.join(root, "%05d.csv" % t), spix[t], fmt="%d", delimiter=",")


def load_spix_csv(root: str) -> np.ndarray:
    """The frames written by save_spix_csv (or the reference's scripts), int32 [T, H, W]."""
    names = sorted(f for f in os.listdir(root) if f.endswith(".csv"))
    return np.stack([np.loadtxt(os.path.join(root, f), dtype=np.int64, delimiter=",", ndmin=2)
                     for f in names]).astype(np.int32)
