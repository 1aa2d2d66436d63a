"""C ABI checks that need no GPU: the engine library loads and exports every entry
point include/st_spix_gb300.h declares; the default configuration matches the
reference's constants; the drop-in module rejects CPU tensors like the reference."""
import ctypes as C
import math
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "st_spix_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(stspix_[a-z0-9_]+)\s*\(", src)))


def test_header_lists_expected_entry_points():
    from st_spix_gb300 import _lib
    assert set(declared_symbols()) == set(_lib.EXPORTS)


def test_library_loads_and_exports_all_symbols():
    from st_spix_gb300 import _lib
    lib = _lib.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.stspix_version() >= 1


def test_default_config_is_reference_defaults():
    from st_spix_gb300 import _lib
    c = _lib.default_config()
    assert (c.niters_seg, c.sp_size, c.sm_start, c.sm_period) == (4, 15, 0, 4)
    assert c.sigma2_app == pytest.approx(0.009 ** 2)
    assert c.potts == pytest.approx(0.5)
    assert c.alpha_hastings == pytest.approx(math.log(0.5))
    assert c.thresh_relabel == pytest.approx(1e-5) and c.thresh_new == pytest.approx(1e-2)


def test_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("has a GPU")
    from st_spix_gb300 import _lib
    lib = _lib.load()
    h = C.c_void_p()
    assert lib.stspix_create(C.byref(h), 0) != 0
    assert lib.stspix_bist_forward(None, None, None, None, 1, 8, 8, 3, None, 0, 0, None) == 1


def test_dropin_rejects_cpu_tensors():
    import torch
    from st_spix_gb300 import bist_cuda
    vid = torch.zeros((1, 8, 8, 3))
    with pytest.raises(RuntimeError, match="CUDA"):
        bist_cuda.bist_forward(vid, vid, 4, 15, 0.5, 1e-4, -0.69, 0.0, False, False)
