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


def test_adapters_and_kkt_reject_bad_arguments(gb):
    """The input adapters and the steps around the solve check their arguments
    before any CUDA call (the pointers below are host memory and are never
    dereferenced)."""
    L = gb.lib()
    buf = np.zeros(64, np.float32)
    p = buf.ctypes.data_as(ctypes.c_void_p)
    INV, UNS = gb.ERR_INVALID_ARGUMENT, gb.ERR_UNSUPPORTED
    # CSR -> cbtd: NULL pointers, empty sizes
    assert L.gbdpcg_csr_to_cbtd_f32(None, p, p, 2, 3, p, p, None) == INV
    assert L.gbdpcg_csr_to_cbtd_f32(p, p, p, 0, 3, p, p, None) == INV
    assert L.gbdpcg_csr_to_cbtd_f64(p, p, p, 2, 0, p, p, None) == INV
    # dense -> cbtd: NULL, n > 32, leading dimension below n N
    assert L.gbdpcg_dense_to_cbtd_f32(None, 6, 0, 2, 3, p, None, None) == INV
    assert L.gbdpcg_dense_to_cbtd_f32(p, 99, 0, 33, 3, p, None, None) == INV
    assert L.gbdpcg_dense_to_cbtd_f64(p, 5, 1, 2, 3, p, None, None) == INV
    assert "leading dimension" in gb.last_error()
    # Schur formation / back-substitution: NULL, empty, too large
    args7 = [p] * 7
    assert L.gbdpcg_form_schur_f32(*([None] + [p] * 6), 2, 1, 3, p, p, None) == INV
    assert L.gbdpcg_form_schur_f32(*args7, 2, 0, 3, p, p, None) == INV
    assert L.gbdpcg_form_schur_f64(*args7, 33, 1, 3, p, p, None) == UNS
    assert L.gbdpcg_form_schur_pinv_f32(*args7, 2, 1, 3, p, p, None, None) == INV
    assert L.gbdpcg_kkt_backsub_f32(*([p] * 6 + [None]), 2, 1, 3, p, p, None) == INV
    assert L.gbdpcg_kkt_backsub_f64(*args7, 0, 1, 3, p, p, None) == INV


def test_noalloc_checks_like_the_handle_entry_points(gb):
    """The allocation-free solve rejects the configs the handle entry points
    reject, with the same status, before any CUDA call (host pointers below,
    never dereferenced), and checks its size limits first."""
    L = gb.lib()
    r = gb.Result()
    a = np.zeros(36, np.float32)
    p = a.ctypes.data_as(ctypes.c_void_p)
    for bad in (gb.config(zero_guess=2), gb.config(exit_mode=7), gb.config(algorithm=9),
                gb.config(exit_tol=-1.0), gb.config(cluster_size=17), gb.config(inner_tol=1.5)):
        rc_noalloc = L.gbdpcg_solve_plain_noalloc_f32(p, p, p, p, 2, 3, ctypes.byref(bad), ctypes.byref(r), None)
        rc_handle = L.gbdpcg_solve_f32(p, p, p, p, 2, 3, ctypes.byref(bad), ctypes.byref(r))
        assert rc_noalloc == rc_handle == gb.ERR_INVALID_ARGUMENT
    # n*N beyond the scratch array (N itself within its limit), and N beyond it
    good = gb.config()
    for n, N in ((64, 2049), (1, 4097)):
        assert L.gbdpcg_solve_plain_noalloc_f32(p, p, p, p, n, N, ctypes.byref(good), ctypes.byref(r),
                                                None) == gb.ERR_UNSUPPORTED
        assert "allocation-free limits" in gb.last_error()
