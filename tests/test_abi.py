"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/hp3dg.h (no GPU needed)."""
import ctypes
import os
import re

import numpy as np

from hp3d_gb300 import build as B
from hp3d_gb300 import hp3dg as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "hp3dg.h")).read()
    return sorted(set(re.findall(r"\b(hp3dg_[a-z_0-9]+)\s*\(", txt)))


def test_library_builds_and_exports_all_declared_symbols():
    path = B.build()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 16
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_struct_layouts_match_header():
    assert ctypes.sizeof(H.Opts) == 16 * 4  # 13 fields, tune, 2 reserved
    assert H.DESC_DTYPE.itemsize == 4 * (2 + 19 + 12 + 6 + 26 + 26)


def test_strerror_without_gpu():
    L = H.lib()
    assert L.hp3dg_strerror(-1).decode().startswith("negative Jacobian")
    assert L.hp3dg_strerror(0).decode() == "ok"


def test_null_context_calls_return_arg_errors_without_gpu():
    """Entry points reject a NULL context before touching the device."""
    L = H.lib()
    ERR_ARG = -7
    k = ctypes.c_int64()
    assert L.hp3dg_batch_set_geometry(None, None) == ERR_ARG
    assert L.hp3dg_dpg_pass_stats(None, ctypes.byref(k)) == ERR_ARG
    assert L.hp3dg_pass_stats(None, ctypes.byref(k), None) == ERR_ARG
    assert L.hp3dg_dpg_last_bad_element(None) == -1
    n = ctypes.c_int32()
    assert L.hp3dg_bin_info(None, ctypes.byref(n), 0, None, None) == ERR_ARG
    assert L.hp3dg_gdof_points(None, None, None, ctypes.byref(k)) == ERR_ARG
    assert L.hp3dg_update_gdof(None, None, None, None, None, None, 0) == ERR_ARG


def test_dpg_opts_layout_matches_header():
    # 5 doubles, 8 int32 (ibcflag .. precision), 4 reserved
    assert ctypes.sizeof(H.DpgOpts) == 5 * 8 + 8 * 4 + 4 * 4
