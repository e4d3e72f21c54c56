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
