"""The C-ABI library loads and exports every function declared in include/*.h (CPU)."""

import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(mjx_\w+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = _declared()
    for n in ("mjx_fft_cn2d", "mjx_spectral_apply2d", "mjx_imex_adaptive2d", "mjx_bc_pad2d"):
        assert n in names


def test_library_exports_all_declared(native_lib):
    lib = ctypes.CDLL(os.path.join(ROOT, "moljax_gb300", "_lib", "libmoljax_gb300.so"))
    missing = [n for n in sorted(_declared()) if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(native_lib):
    from moljax_gb300 import _native
    missing = [n for n in sorted(_declared()) if n not in _native.SIGNATURES]
    assert not missing, missing


def test_status_strings_and_sizes(native_lib):
    lib = native_lib
    assert lib.mjx_version().startswith(b"moljax_gb300")
    assert lib.mjx_status_string(10) == b"workspace too small"
    # plan/workspace size queries need no GPU; bad shapes return 0
    assert lib.mjx_spec2d_plan_bytes(1024, 1024, 0) > 0
    assert lib.mjx_spec2d_plan_bytes(1000, 1024, 0) == 0
    assert lib.mjx_imex2d_ws_bytes(1024, 1024, 2, 0) > 4 * 1024 * 1024 * 2 * 3


def test_dft_schedule_candidates_and_registry(native_lib, tmp_path):
    """The autotuner's host side: candidate radix schedules (products equal n, radices
    2-5, no duplicates, the default first), schedule install / query / reset, stencil tile
    heights, and a save / load round trip of the installed choices."""
    import math
    import torch
    from moljax_gb300.core import autotune as AT
    for n in (6, 12, 48, 80, 100, 96, 2000, 1536, 375, 5):
        cands = AT.dft_schedule_candidates(n)
        assert cands and len(set(cands)) == len(cands)
        for c in cands:
            assert math.prod(c) == n and set(c) <= {2, 3, 4, 5}
    assert AT.dft_schedule_candidates(48)[0] == (4, 4, 3)
    assert AT.dft_schedule_candidates(1024) == [] and AT.dft_schedule_candidates(14) == []
    assert AT.dft_schedule(48, torch.float64) == ((4, 4, 3), 6)
    AT.set_dft_schedule(48, torch.float64, (3, 2, 2, 4), 12)
    assert AT.dft_schedule(48, torch.float64) == ((3, 2, 2, 4), 12)
    assert AT.dft_schedule(48, torch.float32) == ((4, 4, 3), 6)  # per element size
    arr = (ctypes.c_int * 16)(4, 4, 4)
    from moljax_gb300 import _native as NV
    assert native_lib.mjx_dft_schedule_set(48, NV.dtype_code(torch.float64), 3, arr, 0) != 0  # product 64 != 48
    AT.set_stencil_rows(100, 70, 2, torch.float32, 16)
    assert AT.stencil_rows(100, 70, 2, torch.float32) == 16
    assert native_lib.mjx_stencil_rows_set(100, 70, 2, NV.dtype_code(torch.float32), 3) != 0  # not a candidate
    path = str(tmp_path / "tune.json")
    AT.save(path)
    AT.set_dft_schedule(48, torch.float64, ())
    AT.set_stencil_rows(100, 70, 2, torch.float32, 0)
    assert AT.dft_schedule(48, torch.float64) == ((4, 4, 3), 6)
    assert AT.load(path) >= 2
    assert AT.dft_schedule(48, torch.float64) == ((3, 2, 2, 4), 12)
    assert AT.stencil_rows(100, 70, 2, torch.float32) == 16
    AT.set_dft_schedule(48, torch.float64, ())
    AT.set_stencil_rows(100, 70, 2, torch.float32, 0)
