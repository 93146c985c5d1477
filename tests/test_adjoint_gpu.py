"""Adjoint of the PCG solve (no reference counterpart; the differentiation
configuration): dL/dgamma = mu with S mu = dL/dlambda, and the
block-tridiagonal dL/dS = -1/2 (mu lambda^T + lambda mu^T), for
L = 1/2 ||lambda - lambda*||^2.  Checked against a dense FP64 gradient and
FP64 central finite differences (step 1e-6) on 64 random symmetric
perturbation directions of S and gamma."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sys(O, n, N, seed):
    sy = O.generate(n, N, seed)
    rng = np.random.default_rng(1000 + seed)
    lam_star = rng.standard_normal(n * N)
    return sy, lam_star


def _gpu_forward_adjoint(gb, handle, O, sy, lam_star, layout):
    import torch
    n, N = sy.n, sy.N
    d = torch.device("cuda:0")
    S = torch.from_numpy(sy.cbtd(np.float32)).to(d)
    if layout == gb.PINV_BLOCKDIAG:
        P = torch.from_numpy(O.block_jacobi(sy.D, "compact").astype(np.float32)).to(d)
    else:
        P = torch.from_numpy(O.block_jacobi(sy.D, "cbtd").astype(np.float32)).to(d)
    g = torch.from_numpy(sy.gamma.astype(np.float32)).to(d)
    lam = torch.zeros(n * N, device=d)
    cfg = gb.config(max_iter=500, exit_tol=1e-7, exit_mode=gb.EXIT_RELRES)
    r = handle.solve(S, P, g, lam, n, N, layout, cfg)
    assert r.status == gb.CONVERGED
    grad_lam = lam - torch.from_numpy(lam_star.astype(np.float32)).to(d)
    dg = torch.empty_like(lam)
    dS = torch.full_like(S, float("nan"))
    r2 = handle.adjoint(S, P, lam, grad_lam, dg, dS, n, N, layout, cfg)
    assert r2.status == gb.CONVERGED
    return lam.cpu().numpy(), dg.cpu().numpy(), dS.cpu().numpy()


def _dense_grads(O, sy, lam_star):
    n, N = sy.n, sy.N
    S = sy.cbtd()
    A = O.dense_from_cbtd(S, n, N)
    lam = np.linalg.solve(A, sy.gamma)
    mu = np.linalg.solve(A, lam - lam_star)
    G = -0.5 * (np.outer(mu, lam) + np.outer(lam, mu))
    # restrict to the cbtd pattern
    dS = np.zeros((N, 3 * n, n))
    for k in range(N):
        for b in range(3):
            kk = k + b - 1
            if 0 <= kk < N:
                dS[k, b * n:(b + 1) * n, :] = G[k * n:(k + 1) * n, kk * n:(kk + 1) * n].T
    return lam, mu, dS.reshape(-1)


@pytest.mark.parametrize("layout", [1, 0])
@pytest.mark.parametrize("n,N,seed", [(14, 64, 0), (6, 20, 1), (24, 40, 2)])
def test_adjoint_vs_dense_fp64(gb, oracle_mod, handle, n, N, seed, layout):
    O = oracle_mod
    sy, lam_star = _sys(O, n, N, seed)
    lam, dg, dS = _gpu_forward_adjoint(gb, handle, O, sy, lam_star, layout)
    lam64, mu64, dS64 = _dense_grads(O, sy, lam_star)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    assert rel(lam, lam64) < 1e-4
    assert rel(dg, mu64) < 1e-4
    assert rel(dS, dS64) < 2e-4
    # padding blocks are written as zeros
    dSr = dS.reshape(N, 3 * n, n)
    assert not dSr[0, :n].any() and not dSr[-1, 2 * n:].any()


def test_adjoint_finite_differences(gb, oracle_mod, handle):
    """64 random symmetric directions (dS block-tridiagonal symmetric, dgamma),
    central differences of L in FP64 with step 1e-6."""
    O = oracle_mod
    n, N = 14, 64
    sy, lam_star = _sys(O, n, N, 3)
    lam, dg, dS = _gpu_forward_adjoint(gb, handle, O, sy, lam_star, gb.PINV_BLOCKDIAG)
    S = sy.cbtd()
    rng = np.random.default_rng(7)

    def loss(Sc, g):
        x = O.block_cholesky_solve(Sc, n, N, g)
        return 0.5 * float(np.dot(x - lam_star, x - lam_star))

    h = 1e-6
    errs = []
    for _ in range(64):
        Dd = rng.standard_normal((N, n, n))
        Dd = 0.5 * (Dd + Dd.transpose(0, 2, 1))
        Do = rng.standard_normal((N - 1, n, n))
        dSdir = O.pack_cbtd(Dd, Do) * 1e-2
        dgdir = rng.standard_normal(n * N)
        fd = (loss(S + h * dSdir, sy.gamma + h * dgdir) - loss(S - h * dSdir, sy.gamma - h * dgdir)) / (2 * h)
        an = float(np.dot(dS.astype(np.float64), dSdir) + np.dot(dg.astype(np.float64), dgdir))
        errs.append(abs(fd - an) / max(abs(fd), 1e-12))
    assert np.median(errs) < 1e-4 and max(errs) < 1e-2, (np.median(errs), max(errs))


def test_autograd_function(gb, oracle_mod, handle):
    import torch
    O = oracle_mod
    n, N = 12, 30
    sy, lam_star = _sys(O, n, N, 4)
    d = torch.device("cuda:0")
    S = torch.from_numpy(sy.cbtd(np.float32)).to(d).requires_grad_(True)
    P = torch.from_numpy(O.block_jacobi(sy.D, "compact").astype(np.float32)).to(d)
    g = torch.from_numpy(sy.gamma.astype(np.float32)).to(d).requires_grad_(True)
    ls = torch.from_numpy(lam_star.astype(np.float32)).to(d)
    lam = gb.pcg_solve_autograd(S, P, g, n, N, gb.PINV_BLOCKDIAG, max_iter=500, exit_tol=1e-7,
                                exit_mode=gb.EXIT_RELRES)
    L = 0.5 * ((lam - ls) ** 2).sum()
    L.backward()
    lam64, mu64, dS64 = _dense_grads(O, sy, lam_star)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    assert rel(g.grad.cpu().numpy(), mu64) < 1e-4
    assert rel(S.grad.cpu().numpy(), dS64) < 2e-4


def test_batched_adjoint_plan(gb, oracle_mod, handle):
    """Config of the differentiation benchmark at reduced batch: n=14, N=64."""
    import torch
    O = oracle_mod
    n, N, B = 14, 64, 24
    d = torch.device("cuda:0")
    fwd, adj, keep = [], [], []
    for b in range(B):
        sy, lam_star = _sys(O, n, N, 100 + b)
        S = torch.from_numpy(sy.cbtd(np.float32)).to(d)
        P = torch.from_numpy(O.block_jacobi(sy.D, "compact").astype(np.float32)).to(d)
        g = torch.from_numpy(sy.gamma.astype(np.float32)).to(d)
        lam = torch.zeros(n * N, device=d)
        fwd.append({"S": S, "Pinv": P, "gamma": g, "lambda": lam, "n": n, "N": N})
        keep.append((sy, lam_star))
    cfg = gb.config(max_iter=500, exit_tol=1e-7, exit_mode=gb.EXIT_RELRES)
    pf = gb.Plan(handle, fwd, gb.PINV_BLOCKDIAG, cfg)
    pf.execute()
    assert all(r.status == gb.CONVERGED for r in pf.results())
    for f, (sy, lam_star) in zip(fwd, keep):
        gl = f["lambda"] - torch.from_numpy(lam_star.astype(np.float32)).to(d)
        adj.append({"S": f["S"], "Pinv": f["Pinv"], "gamma": gl, "lambda": torch.empty_like(gl),
                    "lambda_fwd": f["lambda"], "dS": torch.empty_like(f["S"]), "n": n, "N": N})
    pa = gb.Plan(handle, adj, gb.PINV_BLOCKDIAG, cfg)
    pa.execute()
    assert all(r.status == gb.CONVERGED for r in pa.results())
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    for a, (sy, lam_star) in list(zip(adj, keep))[:6]:
        lam64, mu64, dS64 = _dense_grads(O, sy, lam_star)
        assert rel(a["lambda"].cpu().numpy(), mu64) < 1e-4
        assert rel(a["dS"].cpu().numpy(), dS64) < 2e-4


@pytest.mark.parametrize("layout,algorithm,dts", [(1, "auto", "f32"), (0, "auto", "f32"), (1, "recurrence", "f32")])
def test_fused_forward_adjoint_matches_two_plans(gb, oracle_mod, layout, algorithm, dts):
    """gbdpcg_plan_create_fwd_adj: forward solve and adjoint solve with the dS,
    dgamma epilogue in one launch give the bits of a forward plan followed by
    an adjoint plan (same launch shapes: a fresh handle, no tuning table), on
    the batched-adjoint systems (n = 14, N = 64), and the results of both
    solves."""
    import torch
    O = oracle_mod
    n, N, B = 14, 64, 12
    dt = np.float64 if dts == "f64" else np.float32
    td = torch.float64 if dts == "f64" else torch.float32
    d = torch.device("cuda:0")
    h = gb.Handle(0)
    algo = gb.ALGO_RECURRENCE if algorithm == "recurrence" else gb.ALGO_AUTO
    cfg = gb.config(max_iter=500, exit_tol=1e-7, exit_mode=gb.EXIT_RELRES, zero_guess=1, algorithm=algo)
    fwd, adj, fused = [], [], []
    for b in range(B):
        sy, lam_star = _sys(O, n, N, 100 + b)
        S = torch.from_numpy(sy.cbtd(dt)).to(d)
        P = torch.from_numpy(O.block_jacobi(sy.D, "compact" if layout == 1 else "cbtd").astype(dt)).to(d)
        g = torch.from_numpy(sy.gamma.astype(dt)).to(d)
        star = torch.from_numpy(lam_star.astype(dt)).to(d)
        fwd.append({"S": S, "Pinv": P, "gamma": g, "lambda": torch.zeros(n * N, dtype=td, device=d), "n": n, "N": N,
                    "star": star})
        fused.append({"S": S, "Pinv": P, "gamma": g, "lambda": torch.zeros(n * N, dtype=td, device=d),
                      "lambda_target": star, "grad_gamma": torch.empty(n * N, dtype=td, device=d),
                      "grad_S": torch.full_like(S, float("nan")), "n": n, "N": N})
    pf = gb.Plan(h, [{k: v for k, v in f.items() if k != "star"} for f in fwd], layout, cfg)
    pf.execute()
    rf = pf.results()
    for f in fwd:
        gl = f["lambda"] - f["star"]
        adj.append({"S": f["S"], "Pinv": f["Pinv"], "gamma": gl, "lambda": torch.empty_like(gl),
                    "lambda_fwd": f["lambda"], "dS": torch.empty_like(f["S"]), "n": n, "N": N})
    pa = gb.Plan(h, adj, layout, cfg)
    pa.execute()
    ra = pa.results()
    pj = gb.Plan.forward_adjoint(h, fused, layout, cfg)
    assert [l["storage"] for l in pj.launches()] == [l["storage"] for l in pf.launches()]
    pj.execute()
    rj = pj.results()
    torch.cuda.synchronize()
    assert len(rj) == 2 * B
    for b in range(B):
        assert rj[b].status == rf[b].status == gb.CONVERGED and rj[b].iters == rf[b].iters
        assert rj[B + b].status == ra[b].status == gb.CONVERGED and rj[B + b].iters == ra[b].iters
        assert fused[b]["lambda"].cpu().numpy().tobytes() == fwd[b]["lambda"].cpu().numpy().tobytes()
        assert fused[b]["grad_gamma"].cpu().numpy().tobytes() == adj[b]["lambda"].cpu().numpy().tobytes()
        assert fused[b]["grad_S"].cpu().numpy().tobytes() == adj[b]["dS"].cpu().numpy().tobytes()
    for p in (pf, pa, pj):
        p.close()
    h.close()


def test_fused_forward_adjoint_rejects_streamed_sizes(gb, handle):
    """A pair whose rows do not fit on chip (n = 14, N = 20000) is refused at
    plan creation, before anything is launched."""
    import torch
    n, N = 14, 20000
    d = torch.device("cuda:0")
    t = torch.zeros(3 * n * n * N, device=d)
    v = torch.zeros(n * N, device=d)
    with pytest.raises(gb.GbdpcgError) as e:
        gb.Plan.forward_adjoint(handle, [{"S": t, "Pinv": t, "gamma": v, "lambda": v, "lambda_target": v,
                                          "grad_gamma": v, "grad_S": t, "n": n, "N": N}], gb.PINV_BLOCKDIAG,
                                gb.config())
    assert e.value.code == gb.ERR_UNSUPPORTED
