"""The C-ABI library builds for sm_103a, loads, and exports every function
that include/vkvg.h, include/vkvg-svg.h and include/vkvg_gb300.h declare
(no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in ("vkvg.h", "vkvg-svg.h", "vkvg_gb300.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"vkvg_public\s+[\w\s\*]+?\b(vkvg_\w+)\s*\(", src)
    return sorted(set(names))


def test_headers_declare_api():
    names = declared_functions()
    for n in ("vkvg_move_to", "vkvg_curve_to", "vkvg_arc", "vkvg_fill", "vkvg_stroke", "vkvg_set_dash",
              "vkvg_set_fill_rule", "vkvg_surface_write_to_png", "vkvg_gb300_frame_execute", "vkvg_svg_render",
              "vkvg_surface_create_from_svg"):
        assert n in names
    assert len(names) > 100


def test_library_exports_every_declared_symbol(gb):
    L = ctypes.CDLL(gb.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_python_binding_covers_header(gb):
    assert set(declared_functions()) <= set(gb.SIGNATURES)


def test_no_device_fails_loudly_without_gpu(gb):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gb.VkvgError):
        gb.Device(samples=4)


def test_status_strings(gb):
    L = gb.lib()
    assert L.vkvg_status_to_string(0) == b"no error has occurred"
    assert L.vkvg_status(None) == 2  # VKVG_STATUS_NULL_POINTER


@pytest.mark.parametrize("fn", range(6))
def test_pmath_host_matches_oracle_copy(gb, vko, fn):
    """The product's host build of the portable math (used by the recorder) and
    the oracle's copy give identical bits."""
    rng = np.random.default_rng(fn)
    if fn == 0:
        a = rng.uniform(-2000, 2000, 200000).astype(np.float32)
        b = rng.uniform(-2000, 2000, 200000).astype(np.float32)
        a[:100] = 0.0
        b[50:150] = 0.0
    elif fn in (1, 4):
        a = rng.uniform(-1.2, 1.2, 200000).astype(np.float32)
        b = a
    else:
        a = rng.uniform(-100, 100, 200000).astype(np.float32)
        b = a
    x = gb.pmath(fn, a, b, device=False)
    y = vko.pmath(fn, a, b)
    assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
