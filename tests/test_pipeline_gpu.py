"""End-to-end solves of packed plans from host arenas (gbdpcg_plan_execute_host).

With more than one piece, copies of piece i+1 overlap the solve of piece i.
Every system keeps its launch shape (the shape depends on the system and the
config, or on the handle's tuning table, not on the batch), so the pipelined
path must give the same bits as the unpipelined one and as a device-side
execution of the whole plan."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _packed(gb, count, seed0):
    from gbdpcg.workload import packed_batch
    return packed_batch(range(seed0, seed0 + count), np.float32, workers=1, pinv_layout=1)


def _run_host(gb, handle, descs, Sa, Pa, ga, pieces, tune=False):
    import torch
    d = torch.device("cuda:0")
    dS = torch.zeros(Sa.size, device=d)
    dP = torch.zeros(Pa.size, device=d)
    dg = torch.zeros(ga.size, device=d)
    dl = torch.zeros(ga.size, device=d)
    cfg = gb.config(max_iter=300, exit_tol=1e-6, exit_mode=gb.EXIT_RELRES, zero_guess=1, host_pieces=pieces)
    plan = gb.Plan(handle, layout=gb.PINV_BLOCKDIAG, cfg=cfg, packed=(descs, dS, dP, dg, dl))
    hS = torch.from_numpy(Sa).pin_memory()
    hP = torch.from_numpy(Pa).pin_memory()
    hg = torch.from_numpy(ga).pin_memory()
    hl = torch.full((ga.size,), 9.0).pin_memory()
    if tune:
        dS.copy_(hS)
        dP.copy_(hP)
        dg.copy_(hg)
        plan.autotune(reps=1)
    res = plan.execute_host(hS, hP, hg, hl, with_results=True)
    res2 = plan.results()
    out = hl.numpy().copy()
    # the device-side execution of the same plan on the arenas execute_host filled
    dl.zero_()
    plan.execute()
    torch.cuda.synchronize()
    dev = dl.cpu().numpy()
    plan.close()
    return out, [(r.iters, r.status, r.relres) for r in res], [(r.iters, r.status, r.relres) for r in res2], dev


def _pinv(O, descs, Sa, nP):
    Pa = np.zeros(nP, np.float32)
    for (n, N, oS, oP, oV) in descs:
        _, di, _ = O.unpack_cbtd(Sa[oS:oS + 3 * n * n * N], n, N)
        Pa[oP:oP + n * n * N] = O.block_jacobi(di, "compact").astype(np.float32)
    return Pa


@pytest.mark.parametrize("tune", [False, True])
def test_pipelined_execute_host_matches(gb, oracle_mod, handle, tune):
    O = oracle_mod
    descs, Sa, ga, nP = _packed(gb, 240, 4000)
    Pa = _pinv(O, descs, Sa, nP)
    handle.tune_clear()
    l1, r1, q1, d1 = _run_host(gb, handle, descs, Sa, Pa, ga, pieces=1, tune=tune)
    l4, r4, q4, d4 = _run_host(gb, handle, descs, Sa, Pa, ga, pieces=4, tune=tune)
    assert all(s == 0 for _, s, _ in r1) and all(s == 0 for _, s, _ in r4)
    # within a plan: the pipelined host path, its results and the device path agree bit for bit
    assert q1 == r1 and q4 == r4
    assert d1.tobytes() == l1.tobytes() and d4.tobytes() == l4.tobytes()
    if not tune:  # same shapes in both plans: same bits across them too
        assert r1 == r4 and l1.tobytes() == l4.tobytes()
    for (n, N, oS, oP, oV), (it, st, rr) in list(zip(descs, r1))[::17]:
        assert rr <= 1e-6 * (1 + 1e-6)
        assert O.relres(Sa[oS:oS + 3 * n * n * N], l1[oV:oV + n * N], ga[oV:oV + n * N], n, N) < 1e-3
    handle.tune_clear()


def test_out_of_order_arenas_fall_back(gb, oracle_mod, handle):
    """Offsets that do not increase with the system index: execute_host copies
    the arenas whole and still solves every system."""
    O = oracle_mod
    descs, Sa, ga, nP = _packed(gb, 40, 4500)
    Pa = _pinv(O, descs, Sa, nP)
    rev = list(reversed(descs))
    l_rev, r_rev, _, _ = _run_host(gb, handle, rev, Sa, Pa, ga, pieces=4)
    l_fwd, r_fwd, _, _ = _run_host(gb, handle, descs, Sa, Pa, ga, pieces=4)
    assert r_rev == list(reversed(r_fwd))
    assert l_rev.tobytes() == l_fwd.tobytes()


@pytest.mark.parametrize("pieces", [1, 4])
def test_solve_host_builds_pinv_on_device(gb, oracle_mod, handle, pieces):
    """The batched pcg_solve (S and gamma from the host, block-Jacobi Phi^-1
    built on the device) gives the bits of building Phi^-1 on the device and
    executing the plan there."""
    import torch
    O = oracle_mod
    descs, Sa, ga, nP = _packed(gb, 120, 4700)
    d = torch.device("cuda:0")
    handle.tune_clear()
    cfg = gb.config(max_iter=300, exit_tol=1e-6, exit_mode=gb.EXIT_RELRES, zero_guess=1, host_pieces=pieces)
    dS = torch.zeros(Sa.size, device=d)
    dP = torch.full((nP,), float("nan"), device=d)  # nothing may read a Phi^-1 the call did not build
    dg = torch.zeros(ga.size, device=d)
    dl = torch.zeros(ga.size, device=d)
    plan = gb.Plan(handle, layout=gb.PINV_BLOCKDIAG, cfg=cfg, packed=(descs, dS, dP, dg, dl))
    hS = torch.from_numpy(Sa).pin_memory()
    hg = torch.from_numpy(ga).pin_memory()
    hl = torch.full((ga.size,), 9.0).pin_memory()
    res = plan.solve_host(hS, hg, hl, with_results=True)
    out = hl.numpy().copy()
    assert all(r.status == gb.CONVERGED for r in res)
    dl.zero_()
    plan.build_block_jacobi()
    plan.execute()
    torch.cuda.synchronize()
    assert dl.cpu().numpy().tobytes() == out.tobytes()
    for (n, N, oS, oP, oV) in descs[::13]:
        assert O.relres(Sa[oS:oS + 3 * n * n * N], out[oV:oV + n * N], ga[oV:oV + n * N], n, N) < 1e-3
    plan.close()
