"""Streamed matrix rows (GBDPCG_STORAGE_STREAM): the cluster solver reading S
and Phi^-1 from global memory in every product, for systems whose rows do
not fit on chip.

  * With one row group per thread it performs the shared-memory storage's
    products, updates and reductions in the same order: bit for bit the
    same solution and passes.
  * With many row groups (n = 14, N = 2048 and 20000, which no on-chip shape
    holds) it is checked against the oracle (the CPU restatement of the
    reference PCG, include/pcg.cuh:54-218): passes within one, accuracy
    against the FP64 block-Cholesky solution no worse than 1.5 x the
    reference's.
  * The adjoint epilogue runs over the row groups too.
  * FP64 systems of n = 24, N = 256 (no on-chip FP64 shape holds them) solve
    in one batched plan to a relative residual of 1e-10."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - np.asarray(b, np.float64)) /
                 max(np.linalg.norm(np.asarray(b, np.float64)), 1e-300))


def _dev(*arrays):
    import torch
    d = torch.device("cuda:0")
    return [torch.from_numpy(np.ascontiguousarray(a)).to(d) for a in arrays]


@pytest.mark.parametrize("dts,layout,other", [("f32", "cbtd", "shared"), ("f32", "compact", "split"),
                                              ("f64", "compact", "shared"), ("f64", "cbtd", "shared")])
def test_stream_matches_on_chip_storage_bitwise(gb, oracle_mod, handle, dts, layout, other):
    """n = 12, N = 50, two CTAs: one row group per thread; the same CTA size
    and rows per thread as the on-chip storage it is compared with."""
    O = oracle_mod
    dt = np.float64 if dts == "f64" else np.float32
    n, N = 12, 50
    sy = O.generate(n, N, 3)
    S, P, g = _dev(sy.cbtd(dt), O.block_jacobi(sy.D, layout).astype(dt), sy.gamma.astype(dt))
    lay = gb.PINV_BLOCKDIAG if layout == "compact" else gb.PINV_CBTD
    st = {"shared": gb.STORAGE_SHARED, "split": gb.STORAGE_SPLIT}[other]
    outs = []
    for storage in (st, gb.STORAGE_STREAM):
        import torch
        lam = torch.zeros(n * N, dtype=S.dtype, device=S.device)
        r = handle.solve(S, P, g, lam, n, N, lay,
                         gb.config(max_iter=300, exit_tol=1e-12 if dts == "f64" else 1e-6, storage=storage,
                                   cluster_size=2))
        assert r.status == gb.CONVERGED
        outs.append((r.iters, r.eta, lam.cpu().numpy().tobytes()))
    assert outs[0] == outs[1]


@pytest.mark.parametrize("dts,layout,N,C", [("f32", "compact", 2048, 4), ("f32", "cbtd", 2048, 16),
                                            ("f64", "compact", 2048, 8), ("f32", "cbtd", 20000, 0)])
def test_stream_many_row_groups_vs_oracle(gb, oracle_mod, handle, dts, layout, N, C):
    """Systems no on-chip shape holds.  C = 0 lets AUTO choose (n = 14,
    N = 20000 was UNSUPPORTED before streamed rows)."""
    import torch
    O = oracle_mod
    dt = np.float64 if dts == "f64" else np.float32
    tol = 1e-12 if dts == "f64" else 1e-6
    n = 14
    sy = O.generate(n, N, 7)
    S = sy.cbtd(dt)
    Pt = O.block_jacobi(sy.D, "cbtd").astype(dt)
    g = sy.gamma.astype(dt)
    lam_o, it_o, mie = O.ref_pcg(S, Pt, g, np.zeros(n * N, dt), n, N, 400, tol)
    assert not mie
    P = Pt if layout == "cbtd" else O.block_jacobi(sy.D, "compact").astype(dt)
    tS, tP, tg = _dev(S, P, g)
    lam = torch.zeros(n * N, dtype=tS.dtype, device=tS.device)
    cfg = gb.config(max_iter=400, exit_tol=tol, cluster_size=C,
                    storage=gb.STORAGE_STREAM if C else gb.STORAGE_AUTO)
    r = handle.solve(tS, tP, tg, lam, n, N, gb.PINV_BLOCKDIAG if layout == "compact" else gb.PINV_CBTD, cfg)
    assert r.status == gb.CONVERGED
    assert abs(int(r.iters) - it_o) <= 1, (r.iters, it_o)
    x = O.block_cholesky_solve(S.astype(np.float64), n, N, g.astype(np.float64))
    lam_g = lam.cpu().numpy()
    assert relerr(lam_g, x) <= 1.5 * relerr(lam_o, x) + (1e-12 if dts == "f64" else 1e-6)


def test_stream_adjoint(gb, oracle_mod, handle):
    """dL/dgamma and dL/dS from the streamed storage (three row groups per
    thread at 64 threads) against the default storage's, to the solve's
    tolerance."""
    import torch
    O = oracle_mod
    n, N = 12, 64
    sy = O.generate(n, N, 5)
    S, P, g = _dev(sy.cbtd(np.float32), O.block_jacobi(sy.D, "compact").astype(np.float32),
                   sy.gamma.astype(np.float32))
    star = torch.from_numpy(np.random.default_rng(9).standard_normal(n * N).astype(np.float32)).to(S.device)
    outs = []
    for storage, mt in ((gb.STORAGE_AUTO, 0), (gb.STORAGE_STREAM, 64)):
        cfg = gb.config(max_iter=500, exit_tol=1e-7, exit_mode=gb.EXIT_RELRES, storage=storage, max_threads=mt,
                        cluster_size=2)
        lam = torch.zeros(n * N, device=S.device)
        assert handle.solve(S, P, g, lam, n, N, gb.PINV_BLOCKDIAG, cfg).status == gb.CONVERGED
        dg = torch.empty_like(lam)
        dS = torch.full_like(S, float("nan"))
        r = handle.adjoint(S, P, lam, lam - star, dg, dS, n, N, gb.PINV_BLOCKDIAG, cfg)
        assert r.status == gb.CONVERGED
        outs.append((dg.cpu().numpy(), dS.cpu().numpy()))
    assert not np.isnan(outs[1][1]).any()
    assert relerr(outs[1][0], outs[0][0]) < 1e-5
    assert relerr(outs[1][1], outs[0][1]) < 1e-5


def test_fp64_batched_plan_streams_n24_N256(gb, oracle_mod, handle):
    """Four FP64 systems of n = 24, N = 256 in one plan (AUTO picks the
    streamed storage: the rows exceed any on-chip FP64 shape), to a relative
    residual of 1e-10; the true FP64 residual is checked on the host."""
    import torch
    O = oracle_mod
    n, N = 24, 256
    systems, keep = [], []
    d = torch.device("cuda:0")
    for seed in range(4):
        sy = O.generate(n, N, 300 + seed)
        systems.append({"S": torch.from_numpy(sy.cbtd()).to(d),
                        "Pinv": torch.from_numpy(O.block_jacobi(sy.D, "compact")).to(d),
                        "gamma": torch.from_numpy(sy.gamma).to(d),
                        "lambda": torch.zeros(n * N, dtype=torch.float64, device=d), "n": n, "N": N})
        keep.append(sy)
    plan = gb.Plan(handle, systems, gb.PINV_BLOCKDIAG,
                   gb.config(max_iter=2000, exit_tol=1e-10, exit_mode=gb.EXIT_RELRES, zero_guess=1))
    assert all(l["storage"] == 5 for l in plan.launches())
    plan.execute()
    res = plan.results()
    for sy, s, r in zip(keep, systems, res):
        assert r.status == gb.CONVERGED, r
        assert O.relres(sy.cbtd(), s["lambda"].cpu().numpy(), sy.gamma, n, N) < 1e-9
    plan.close()
