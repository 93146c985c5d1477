"""The steps around the solve on the GPU (csrc/kkt.cu): Schur-complement
formation and KKT back-substitution against their FP64 numpy references
(oracle.form_schur / oracle.kkt_backsub), and the whole chain form -> PCG ->
back-substitute against the dense KKT system."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def relerr(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _dev(P, dt):
    import torch
    return {k: torch.from_numpy(v).to("cuda:0") for k, v in P.items()}


CASES = [(14, 32), (24, 40), (6, 1), (7, 9), (32, 5)]


@pytest.mark.parametrize("dt,tol", [(np.float64, 1e-13), (np.float32, 2e-6)])
@pytest.mark.parametrize("n,N", CASES)
def test_form_schur(gb, oracle_mod, handle, dt, tol, n, N):
    import torch
    O = oracle_mod
    P = O.generate_problem(n, N, 21)
    S_o, g_o = O.form_schur(P)
    d = _dev(O.problem_device_layout(P, dt), dt)
    tdt = torch.float64 if dt == np.float64 else torch.float32
    S = torch.full((3 * n * n * N,), 9.0, dtype=tdt, device="cuda:0")
    g = torch.empty(n * N, dtype=tdt, device="cuda:0")
    gb.form_schur(d["A"], d["B"], d["Qd"], d["Rd"], d["q"], d["r"], d["c"], n, P["m"], N, S, g)
    Sh = S.cpu().numpy()
    assert relerr(Sh, S_o) < tol and relerr(g.cpu().numpy(), g_o) < tol
    # diagonal blocks exactly symmetric; padding blocks zero
    Sc = Sh.reshape(N, 3 * n, n)
    Dk = Sc[:, n:2 * n, :]
    assert np.array_equal(Dk, Dk.transpose(0, 2, 1))
    assert not Sc[0, 0:n].any() and not Sc[N - 1, 2 * n:].any()


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n,N", CASES + [(12, 7)])
def test_form_schur_fused_pinv_matches_builder(gb, oracle_mod, handle, dt, n, N):
    """form_schur_pinv writes the same S and gamma as form_schur, and a
    Phi^-1 bit for bit equal to the block-Jacobi builder's on that S (same
    symmetrised S_kk, same Gauss-Jordan routine; n = 12 pads to 16 in the
    formation and to 12 in the builder)."""
    import torch
    O = oracle_mod
    P = O.generate_problem(n, N, 24)
    d = _dev(O.problem_device_layout(P, dt), dt)
    tdt = torch.float64 if dt == np.float64 else torch.float32
    m = P["m"]
    S1 = torch.full((3 * n * n * N,), 9.0, dtype=tdt, device="cuda:0")
    g1 = torch.empty(n * N, dtype=tdt, device="cuda:0")
    gb.form_schur(d["A"], d["B"], d["Qd"], d["Rd"], d["q"], d["r"], d["c"], n, m, N, S1, g1)
    S2 = torch.full_like(S1, 5.0)
    g2 = torch.empty_like(g1)
    Pf = torch.full((n * n * N,), 3.0, dtype=tdt, device="cuda:0")
    gb.form_schur(d["A"], d["B"], d["Qd"], d["Rd"], d["q"], d["r"], d["c"], n, m, N, S2, g2, Pinv_out=Pf)
    assert torch.equal(S1, S2) and torch.equal(g1, g2)
    Pb = torch.empty_like(Pf)
    handle.block_jacobi(S1, Pb, n, N, gb.PINV_BLOCKDIAG)
    torch.cuda.synchronize()
    assert Pf.cpu().numpy().tobytes() == Pb.cpu().numpy().tobytes()


@pytest.mark.parametrize("dt,tol", [(np.float64, 1e-13), (np.float32, 2e-6)])
@pytest.mark.parametrize("n,N", CASES)
def test_kkt_backsub(gb, oracle_mod, handle, dt, tol, n, N):
    import torch
    O = oracle_mod
    P = O.generate_problem(n, N, 22)
    lam = np.random.default_rng(5).standard_normal(n * N)
    x_o, u_o = O.kkt_backsub(P, lam)
    d = _dev(O.problem_device_layout(P, dt), dt)
    tdt = torch.float64 if dt == np.float64 else torch.float32
    x = torch.empty(n * (N + 1), dtype=tdt, device="cuda:0")
    u = torch.empty(P["m"] * N, dtype=tdt, device="cuda:0")
    gb.kkt_backsub(d["A"], d["B"], d["Qd"], d["Rd"], d["q"], d["r"], torch.from_numpy(lam.astype(dt)).to("cuda:0"),
                   n, P["m"], N, x, u)
    assert relerr(x.cpu().numpy(), x_o.reshape(-1)) < tol and relerr(u.cpu().numpy(), u_o.reshape(-1)) < tol


@pytest.mark.parametrize("n,N", [(14, 64), (24, 100)])
def test_form_solve_backsub_satisfies_kkt(gb, oracle_mod, handle, n, N):
    """FP64 end to end on the GPU: form S, gamma and the block-Jacobi Phi^-1
    in one pass, PCG to 1e-12, back-substitute; the dense KKT residual is at
    the PCG tolerance's level."""
    import torch
    O = oracle_mod
    P = O.generate_problem(n, N, 23)
    m = P["m"]
    d = _dev(O.problem_device_layout(P, np.float64), np.float64)
    f64 = dict(dtype=torch.float64, device="cuda:0")
    S = torch.empty(3 * n * n * N, **f64)
    g = torch.empty(n * N, **f64)
    Pinv = torch.empty(n * n * N, **f64)
    gb.form_schur(d["A"], d["B"], d["Qd"], d["Rd"], d["q"], d["r"], d["c"], n, m, N, S, g, Pinv_out=Pinv)
    lam = torch.zeros(n * N, **f64)
    r = handle.solve(S, Pinv, g, lam, n, N, gb.PINV_BLOCKDIAG,
                     gb.config(max_iter=2000, exit_tol=1e-12, exit_mode=gb.EXIT_RELRES))
    assert r.status == gb.CONVERGED
    x = torch.empty(n * (N + 1), **f64)
    u = torch.empty(m * N, **f64)
    gb.kkt_backsub(d["A"], d["B"], d["Qd"], d["Rd"], d["q"], d["r"], lam, n, m, N, x, u)
    K, rhs = O.kkt_dense(P)
    sol = np.concatenate([x.cpu().numpy(), u.cpu().numpy(), lam.cpu().numpy()])
    assert np.linalg.norm(K @ sol - rhs) <= 1e-9 * np.linalg.norm(rhs)
