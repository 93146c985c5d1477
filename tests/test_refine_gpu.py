"""FP32 PCG with FP64 iterative refinement (precision configuration: n=24,
ill-conditioned Q/R, target relative residual 1e-10) against the FP64
block-Cholesky oracle and plain FP64 PCG."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(O, n, N, seed, ill):
    import torch
    d = torch.device("cuda:0")
    sy = O.generate(n, N, seed, ill=ill)
    S64 = torch.from_numpy(sy.cbtd()).to(d)
    g64 = torch.from_numpy(sy.gamma).to(d)
    return sy, S64, g64


@pytest.mark.parametrize("dot", ["fp64", "float2"])
@pytest.mark.parametrize("n,N,seed,ill", [(24, 64, 0, True), (14, 32, 1, False), (6, 100, 2, True), (24, 256, 3, True)])
def test_refined_reaches_fp64_accuracy(gb, oracle_mod, handle, n, N, seed, ill, dot):
    import torch
    O = oracle_mod
    sy, S64, g64 = _setup(O, n, N, seed, ill)
    P32 = torch.empty(n * n * N, dtype=torch.float32, device=S64.device)
    handle.block_jacobi_f64to32(S64, P32, n, N)
    lam = torch.zeros(n * N, dtype=torch.float64, device=S64.device)
    cfg = gb.config(exit_mode=gb.EXIT_RELRES, exit_tol=1e-10, max_iter=40000, max_outer=60, inner_tol=0.05,
                    dot_precision=gb.DOT_FLOAT2 if dot == "float2" else gb.DOT_FP64)
    r = handle.refine_solve(S64, P32, g64, lam, n, N, cfg)
    assert r.status == gb.CONVERGED, r
    lam_h = lam.cpu().numpy()
    rel = O.relres(sy.cbtd(), lam_h, sy.gamma, n, N)
    assert rel <= 1.2e-10 and abs(rel - r.relres) <= 1e-11 + 0.05 * rel, (rel, r)
    x = O.block_cholesky_solve(sy.cbtd(), n, N, sy.gamma)
    # FP64 PCG at the same residual for comparison
    P64 = O.block_jacobi(sy.D, "compact")
    lam64, it64, st64, _, _ = O.pcg(sy.cbtd(), P64, sy.gamma, np.zeros(n * N), n, N, 40000, 1e-10,
                                    flags=O.PINV_BLOCKDIAG | O.EXIT_RELRES)
    err_ref = np.linalg.norm(lam_h - x) / np.linalg.norm(x)
    err_64 = np.linalg.norm(lam64 - x) / np.linalg.norm(x)
    assert err_ref <= 10 * err_64 + 1e-12, (err_ref, err_64)
    if ill:
        assert r.outer >= 2


def test_refined_zero_rhs_and_warm_start(gb, oracle_mod, handle):
    import torch
    O = oracle_mod
    n, N = 12, 20
    sy, S64, g64 = _setup(O, n, N, 5, False)
    P32 = torch.empty(n * n * N, dtype=torch.float32, device=S64.device)
    handle.block_jacobi_f64to32(S64, P32, n, N)
    cfg = gb.config(exit_mode=gb.EXIT_RELRES, exit_tol=1e-10, max_iter=10000)
    lam = torch.zeros(n * N, dtype=torch.float64, device=S64.device)
    r = handle.refine_solve(S64, P32, torch.zeros_like(g64), lam, n, N, cfg)
    assert r.status == gb.CONVERGED and r.outer == 0 and r.iters == 0 and not lam.any()
    # warm start at the exact solution: converged before any inner pass
    x = torch.from_numpy(O.block_cholesky_solve(sy.cbtd(), n, N, sy.gamma)).to(S64.device)
    lam = x.clone()
    r = handle.refine_solve(S64, P32, g64, lam, n, N, cfg)
    assert r.status == gb.CONVERGED and r.iters == 0


@pytest.mark.parametrize("dot", ["fp64", "float2"])
def test_refined_plan_batch(gb, oracle_mod, handle, dot):
    """Batched refinement (plan dtype 2) over ill-conditioned n=24 systems."""
    import torch
    O = oracle_mod
    d = torch.device("cuda:0")
    systems, keep = [], []
    for seed in range(6):
        n, N = (24, 48) if seed % 2 == 0 else (14, 30)
        sy = O.generate(n, N, 50 + seed, ill=True)
        S = torch.from_numpy(sy.cbtd()).to(d)
        systems.append({"S": S, "Pinv": torch.empty(n * n * N, dtype=torch.float32, device=d),
                        "gamma": torch.from_numpy(sy.gamma).to(d),
                        "lambda": torch.zeros(n * N, dtype=torch.float64, device=d), "n": n, "N": N})
        keep.append(sy)
    cfg = gb.config(exit_mode=gb.EXIT_RELRES, exit_tol=1e-10, max_iter=40000, max_outer=60, zero_guess=1,
                    dot_precision=gb.DOT_FLOAT2 if dot == "float2" else gb.DOT_FP64)
    plan = gb.Plan(handle, systems, gb.PINV_BLOCKDIAG, cfg, dtype=2)
    plan.build_block_jacobi()
    plan.execute()
    for s, r, sy in zip(systems, plan.results(), keep):
        assert r.status == gb.CONVERGED
        assert O.relres(sy.cbtd(), s["lambda"].cpu().numpy(), sy.gamma, s["n"], s["N"]) <= 1.2e-10
    plan.close()
