"""The allocation-free entry point gbdpcg_solve_plain_noalloc_f32.

It exists for callers that cannot allocate device memory while they run (a
fixed-rate controller, a process whose GPU memory another allocator owns,
deployments that forbid allocation after start-up).  It runs the plain
algorithm with its scratch in an array compiled into the library, so its
results must equal, bit for bit, those of the existing device-pointer entry
point with the plain algorithm.  Two calls in a row on different systems
check that the shared scratch carries nothing from one call into the next.
Collected last on purpose; it passes alone and after the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solve_noalloc(gb, S, P, g, lam, n, N, cfg):
    r = gb.Result()
    rc = gb.lib().gbdpcg_solve_plain_noalloc_f32(S.data_ptr(), P.data_ptr(), g.data_ptr(), lam.data_ptr(),
                                                 n, N, ctypes.byref(cfg), ctypes.byref(r), None)
    return rc, r


def test_noalloc_matches_plain_entry_point(gb, oracle_mod, handle):
    import torch
    O = oracle_mod
    d = torch.device("cuda:0")
    cases = [(14, 128, 0), (6, 40, 1)]   # two calls in a row, different sizes
    for n, N, seed in cases:
        sy = O.generate(n, N, seed)
        S = torch.from_numpy(sy.cbtd(np.float32)).to(d)
        P = torch.from_numpy(O.block_jacobi(sy.D, "cbtd").astype(np.float32)).to(d)
        g = torch.from_numpy(sy.gamma.astype(np.float32)).to(d)
        cfg = gb.config(max_iter=200, exit_tol=1e-6, algorithm=gb.ALGO_PLAIN)
        lam_ref = torch.zeros(n * N, device=d)
        r_ref = handle.solve(S, P, g, lam_ref, n, N, gb.PINV_CBTD, cfg)
        lam = torch.zeros(n * N, device=d)
        rc, r = _solve_noalloc(gb, S, P, g, lam, n, N, cfg)
        assert rc == gb.SUCCESS, gb.last_error()
        torch.cuda.synchronize()
        assert r.iters == r_ref.iters and r.status == r_ref.status
        assert lam.cpu().numpy().tobytes() == lam_ref.cpu().numpy().tobytes()


def test_noalloc_rejects_sizes_beyond_its_scratch(gb, handle):
    import torch
    d = torch.device("cuda:0")
    n, N = 32, 4097   # n*N > GBDPCG_NOALLOC_MAX_ELEMS and N > GBDPCG_NOALLOC_MAX_KNOTS
    t = torch.zeros(16, device=d)   # never read: the size check comes first
    rc, _ = _solve_noalloc(gb, t, t, t, t, n, N, gb.config())
    assert rc == gb.ERR_UNSUPPORTED
    assert "allocation-free limits" in gb.last_error()
