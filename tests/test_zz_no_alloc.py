"""The allocation-free marked-video entry point (stspix_get_marked_video_noalloc).

It exists for callers that may not allocate device memory while they run (see
include/st_spix_gb300.h).  Checked through the C ABI against the allocating
stspix_get_marked_video on two calls in a row (the shared scratch array keeps the
first call's contents, so the second call checks that nothing stale leaks through),
plus the size limit.  The file name sorts last so a run that stops at the first
failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MAX_PIXELS = 1 << 24
STSPIX_ERR_TOO_LARGE = 9


def _frames(T, H, W, seed):
    rng = np.random.default_rng(seed)
    vid = rng.uniform(-0.2, 1.2, size=(T, H, W, 3)).astype(np.float32)
    # blocky labels with a few irregular cells
    ys, xs = np.mgrid[0:H, 0:W]
    spix = np.stack([((ys // (5 + t)) * 97 + (xs // (7 + t)) * 13 + t) % 50 for t in range(T)])
    spix = spix.astype(np.int32)
    spix[:, rng.integers(0, H, 20), rng.integers(0, W, 20)] = rng.integers(0, 50, 20)
    return vid, spix


def test_marked_video_noalloc_matches_allocating_entry_point():
    from st_spix_gb300 import _lib
    lib = _lib.load()
    ctx = _lib.Context(0)
    stream = torch.cuda.current_stream().cuda_stream
    try:
        for call, (T, H, W) in enumerate([(3, 41, 57), (2, 64, 33)]):
            vid, spix = _frames(T, H, W, seed=call)
            color = torch.tensor([0.1 * call, 0.5, 1.0], dtype=torch.float32, device="cuda")
            gv = torch.from_numpy(vid).cuda()
            gs = torch.from_numpy(spix).cuda()
            ref = torch.full((T, H, W, 3), -7.0, device="cuda")
            got = torch.full((T, H, W, 3), -7.0, device="cuda")
            ctx.check(lib.stspix_get_marked_video(ctx.handle, stream, gv.data_ptr(),
                                                  gs.data_ptr(), color.data_ptr(), T, H, W, 3,
                                                  ref.data_ptr()))
            st = lib.stspix_get_marked_video_noalloc(stream, gv.data_ptr(), gs.data_ptr(),
                                                     color.data_ptr(), T, H, W, 3, got.data_ptr())
            assert st == 0
            torch.cuda.synchronize()
            assert torch.equal(got, ref), f"call {call}: outputs differ"
    finally:
        ctx.close()


def test_marked_video_noalloc_rejects_oversize():
    from st_spix_gb300 import _lib
    lib = _lib.load()
    dummy = torch.zeros(4, device="cuda")
    # 2^24 + 1 pixels: rejected before any launch (pointers are never read)
    st = lib.stspix_get_marked_video_noalloc(torch.cuda.current_stream().cuda_stream,
                                             dummy.data_ptr(), dummy.data_ptr(),
                                             dummy.data_ptr(), 1, 4097, 4096, 3,
                                             dummy.data_ptr())
    assert st == STSPIX_ERR_TOO_LARGE


def test_marked_video_noalloc_at_the_size_limit():
    """Exactly 2^24 pixels (the largest input the fixed scratch holds) is accepted and
    matches the allocating entry point."""
    from st_spix_gb300 import _lib
    lib = _lib.load()
    ctx = _lib.Context(0)
    stream = torch.cuda.current_stream().cuda_stream
    T, H, W = 4, 2048, 2048
    assert T * H * W == MAX_PIXELS
    try:
        g = torch.Generator(device="cuda").manual_seed(5)
        gv = torch.rand((T, H, W, 3), device="cuda", generator=g) * 1.4 - 0.2
        ys = torch.arange(H, device="cuda").view(1, H, 1)
        xs = torch.arange(W, device="cuda").view(1, 1, W)
        ts = torch.arange(T, device="cuda").view(T, 1, 1)
        gs = (((ys // 9) * 131 + (xs // 11) * 7 + ts) % 997).to(torch.int32).contiguous()
        color = torch.tensor([1.0, 0.0, 0.25], dtype=torch.float32, device="cuda")
        ref = torch.empty((T, H, W, 3), device="cuda")
        got = torch.empty((T, H, W, 3), device="cuda")
        ctx.check(lib.stspix_get_marked_video(ctx.handle, stream, gv.data_ptr(), gs.data_ptr(),
                                              color.data_ptr(), T, H, W, 3, ref.data_ptr()))
        st = lib.stspix_get_marked_video_noalloc(stream, gv.data_ptr(), gs.data_ptr(),
                                                 color.data_ptr(), T, H, W, 3, got.data_ptr())
        assert st == 0
        torch.cuda.synchronize()
        assert torch.equal(got, ref)
    finally:
        ctx.close()
