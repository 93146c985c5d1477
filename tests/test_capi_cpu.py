"""CPU checks of the C-ABI boundary: the library loads, exports every symbol
include/gbdpcg.h declares, and rejects bad arguments before touching the GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for hdr in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if hdr.endswith(".h"):
            src = open(os.path.join(ROOT, "include", hdr)).read()
            names += re.findall(r"^GBDPCG_API\s+[\w\s\*]+?\b(gbdpcg_\w+)\s*\(", src, flags=re.M)
    return names


def test_exports_every_declared_symbol(gb):
    names = declared_symbols()
    assert len(names) >= 21
    L = ctypes.CDLL(gb.LIB_PATH)
    for nm in names:
        assert hasattr(L, nm), nm
    assert set(names) == set(gb._SIGS), set(names) ^ set(gb._SIGS)


def test_version_and_strings(gb):
    assert gb.lib().gbdpcg_version() == 1000
    assert gb.status_string(gb.ERR_UNSUPPORTED) == "unsupported size or option"


def test_config_defaults_match_reference(gb):
    c = gb.config()
    # include/constants.cuh:15,17
    assert c.exit_tol == 1e-6 and c.max_iter == 25
    assert c.exit_mode == gb.EXIT_REFERENCE and c.use_graph == 1


def test_rejects_null_and_empty(gb):
    L = gb.lib()
    r = gb.Result()
    assert L.gbdpcg_solve_f32(None, None, None, None, 2, 3, None, ctypes.byref(r)) == gb.ERR_INVALID_ARGUMENT
    a = np.zeros(36, np.float32)
    v = np.zeros(6, np.float32)
    p = a.ctypes.data_as(ctypes.c_void_p)
    q = v.ctypes.data_as(ctypes.c_void_p)
    assert L.gbdpcg_solve_f32(p, p, q, q, 0, 3, None, ctypes.byref(r)) == gb.ERR_INVALID_ARGUMENT
    bad = gb.config(exit_mode=7)
    assert L.gbdpcg_solve_f32(p, p, q, q, 2, 3, ctypes.byref(bad), ctypes.byref(r)) == gb.ERR_INVALID_ARGUMENT
    assert "config" in gb.last_error()
    assert L.gbdpcg_create(None, 0) == gb.ERR_INVALID_ARGUMENT
    assert L.gbdpcg_plan_execute(None, None) == gb.ERR_INVALID_ARGUMENT
    assert L.gbdpcg_destroy(None) == gb.ERR_INVALID_ARGUMENT


def test_python_wrapper_validates_shapes(gb):
    with pytest.raises(ValueError):
        gb.solve(np.zeros(35, np.float32), None, np.zeros(6, np.float32), np.zeros(6, np.float32), 2, 3)
    with pytest.raises(TypeError):
        gb.solve(np.zeros(36, np.float64), None, np.zeros(6, np.float32), np.zeros(6, np.float32), 2, 3)
