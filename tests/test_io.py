"""Label files in the reference's CSV format; stream-state snapshots (GPU)."""
import numpy as np
import pytest

from st_spix_gb300 import io, synth


def test_csv_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    spix = rng.integers(-1, 500, size=(3, 7, 11)).astype(np.int32)
    io.save_spix_csv(str(tmp_path / "v"), spix)
    assert sorted(p.name for p in (tmp_path / "v").iterdir()) == ["00000.csv", "00001.csv",
                                                                  "00002.csv"]
    first = (tmp_path / "v" / "00000.csv").read_text().splitlines()[0]
    assert first == ",".join(str(v) for v in spix[0, 0])     # no header, no index
    np.testing.assert_array_equal(io.load_spix_csv(str(tmp_path / "v")), spix)


@pytest.mark.gpu
def test_video_snapshot_resume():
    """A stream saved after frame 1 and restored into a new video continues exactly as
    the uninterrupted stream."""
    torch = pytest.importorskip("torch")
    from st_spix_gb300 import batch
    v, f, _ = synth.voronoi_video(56, 72, 4, 20, 0.03, seed=3, max_shift=3.0)
    vid, flo = torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda()
    kw = dict(niters=8, sp_size=12, sm_period=4, prop_niters=0)
    a = batch.Video(56, 72)
    ref = []
    snap = None
    for t in range(4):
        fr = batch.process_batch([batch.Frame(img=vid[t], flow=flo[t - 1] if t else None,
                                              video=a)], **kw)
        ref.append(fr[0].labels.cpu().numpy())
        if t == 1:
            snap = a.save()
            n1 = a.nspix
    b = batch.Video(56, 72)
    b.load(snap)
    assert b.nspix == n1 and b.frames == 2
    for t in (2, 3):
        fr = batch.process_batch([batch.Frame(img=vid[t], flow=flo[t - 1], video=b)], **kw)
        np.testing.assert_array_equal(fr[0].labels.cpu().numpy(), ref[t])
    with pytest.raises(RuntimeError):
        batch.Video(40, 40).load(snap)
    a.close()
    b.close()
