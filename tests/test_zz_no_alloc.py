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
    """Three calls in a row on different systems, each compared with the
    device-pointer entry point running the plain algorithm: lambda bit for
    bit, and the same passes, status, eta and relative residual (the second
    and third exit on the relative residual, so it is tracked)."""
    import torch
    O = oracle_mod
    d = torch.device("cuda:0")
    cases = [(14, 128, 0, gb.EXIT_REFERENCE), (6, 40, 1, gb.EXIT_RELRES), (14, 64, 2, gb.EXIT_RELRES)]
    for n, N, seed, mode in cases:
        sy = O.generate(n, N, seed)
        S = torch.from_numpy(sy.cbtd(np.float32)).to(d)
        P = torch.from_numpy(O.block_jacobi(sy.D, "cbtd").astype(np.float32)).to(d)
        g = torch.from_numpy(sy.gamma.astype(np.float32)).to(d)
        cfg = gb.config(max_iter=200, exit_tol=1e-6, algorithm=gb.ALGO_PLAIN, exit_mode=mode)
        lam_ref = torch.zeros(n * N, device=d)
        r_ref = handle.solve(S, P, g, lam_ref, n, N, gb.PINV_CBTD, cfg)
        lam = torch.zeros(n * N, device=d)
        rc, r = _solve_noalloc(gb, S, P, g, lam, n, N, cfg)
        assert rc == gb.SUCCESS, gb.last_error()
        torch.cuda.synchronize()
        assert r.iters == r_ref.iters and r.status == r_ref.status
        assert r.eta == r_ref.eta and r.relres == r_ref.relres, (r.eta, r_ref.eta, r.relres, r_ref.relres)
        if mode == gb.EXIT_RELRES:
            assert 0 <= r.relres <= 1e-6
        assert lam.cpu().numpy().tobytes() == lam_ref.cpu().numpy().tobytes()


@pytest.mark.parametrize("n,N", [(64, 2049), (1, 4097), (32, 4097)])
def test_noalloc_rejects_sizes_beyond_its_scratch(gb, handle, n, N):
    """n*N alone beyond the array (64 x 2049), N alone beyond it (1 x 4097),
    and both (32 x 4097): rejected before anything is read or launched."""
    import torch
    d = torch.device("cuda:0")
    t = torch.zeros(16, device=d)   # never read: the size check comes first
    rc, _ = _solve_noalloc(gb, t, t, t, t, n, N, gb.config())
    assert rc == gb.ERR_UNSUPPORTED
    assert "allocation-free limits" in gb.last_error()
