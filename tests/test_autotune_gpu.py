"""Autotuner of batched plans (gbdpcg_plan_autotune) and the handle's tuning
table (gbdpcg_tune_export / _import / _clear).

The tuner re-times each launch class with other storages, cluster sizes and
CTA sizes.  Those shapes reduce in a different order, so tuned results are
checked against the oracle's product iteration with the cluster solver's bar
for mixed sizes: at most one pass apart, and lambda within 1e-5 relative of
the oracle's or no less accurate than 1.5x the oracle's error against the
FP64 block-Cholesky solution (two CPU summation orders already differ by
more than 1e-5 on some of these sizes)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - np.asarray(b, np.float64)) /
                 max(np.linalg.norm(np.asarray(b, np.float64)), 1e-300))


def _batch(O, seeds, d):
    import torch
    systems, host = [], []
    for seed in seeds:
        s = O.generate_mixed(seed)
        S = s.cbtd(np.float32)
        P = O.block_jacobi(s.D, "compact").astype(np.float32)
        g = s.gamma.astype(np.float32)
        systems.append({"S": torch.from_numpy(S).to(d), "Pinv": torch.from_numpy(P).to(d),
                        "gamma": torch.from_numpy(g).to(d), "lambda": torch.zeros(s.n * s.N, device=d),
                        "n": s.n, "N": s.N})
        host.append((S, P, g, s.n, s.N))
    return systems, host


def _cfg(gb, **kw):
    return gb.config(max_iter=300, exit_tol=1e-6, exit_mode=gb.EXIT_RELRES, **kw)


@pytest.mark.parametrize("flags", ["shapes", "whole-plan"])
def test_autotuned_plan_matches_oracle(gb, oracle_mod, handle, flags):
    """Tuned shapes solve like the oracle; the whole-plan pass (the plan timed
    as it runs, solving into scratch) leaves the plan's buffers alone too."""
    import torch
    O = oracle_mod
    d = torch.device("cuda:0")
    handle.tune_clear()
    systems, host = _batch(O, range(300, 396), d)
    plan = gb.Plan(handle, systems, gb.PINV_BLOCKDIAG, _cfg(gb))
    before = plan.launches()
    for s in systems:
        s["lambda"].fill_(7.0)  # the tuner must not touch the plan's buffers
    after = plan.autotune(reps=1, flags=0 if flags == "shapes" else gb.TUNE_WHOLE_PLAN)
    assert sum(l["systems"] for l in after) == len(systems)
    assert len(after) <= len(before)
    for l in after:
        assert 1 <= l["cluster"] <= 16 and l["threads"] % 32 == 0 and l["storage"] in (0, 1, 2, 3, 4)
    for s in systems:
        assert bool((s["lambda"] == 7.0).all())
        s["lambda"].zero_()
    plan.execute()
    res = plan.results()
    for s, r, (S, P, g, n, N) in zip(systems, res, host):
        lam_o, it_o, st_o, _, _ = O.pcg(S, P, g, np.zeros(n * N, np.float32), n, N, 300, 1e-6,
                                        flags=O.PINV_BLOCKDIAG | O.EXIT_RELRES)
        assert r.status == gb.CONVERGED
        assert abs(int(r.iters) - it_o) <= 1, (n, N, r.iters, it_o)
        lam = s["lambda"].cpu().numpy()
        if relerr(lam, lam_o) >= 1e-5:
            x = O.block_cholesky_solve(S.astype(np.float64), n, N, g.astype(np.float64))
            assert relerr(lam, x) <= 1.5 * relerr(lam_o, x) + 1e-6, (n, N)
    plan.close()


def test_tuning_table_round_trip(gb, oracle_mod, handle):
    import torch
    O = oracle_mod
    d = torch.device("cuda:0")
    handle.tune_clear()
    assert handle.tune_export() == ""
    systems, _ = _batch(O, range(500, 540), d)
    plan = gb.Plan(handle, systems, gb.PINV_BLOCKDIAG, _cfg(gb, zero_guess=1))
    tuned = plan.autotune(flags=gb.TUNE_RECURRENCE, reps=1)
    text = handle.tune_export()
    lines = [l for l in text.splitlines() if l]
    assert len(lines) == len({(s["n"], s["N"]) for s in systems})
    # a plan on a fresh handle that imported the table gets the tuned launches
    h2 = gb.Handle(0)
    try:
        h2.tune_import(text)
        assert h2.tune_export() == text
        p2 = gb.Plan(h2, systems, gb.PINV_BLOCKDIAG, _cfg(gb, zero_guess=1))
        key = lambda ls: sorted((l["cluster"], l["threads"], l["storage"], l["rows_per_thread"], l["algorithm"],
                                 l["systems"]) for l in ls)
        assert key(p2.launches()) == key(tuned)
        # a pinned cluster size bypasses the table
        p3 = gb.Plan(h2, systems, gb.PINV_BLOCKDIAG, _cfg(gb, zero_guess=1, cluster_size=8))
        assert all(l["cluster"] == 8 for l in p3.launches())
        p2.close()
        p3.close()
        h2.tune_clear()
        assert h2.tune_export() == ""
    finally:
        h2.close()
    # the same handle's later plans use its own table
    p4 = gb.Plan(handle, systems, gb.PINV_BLOCKDIAG, _cfg(gb, zero_guess=1))
    assert key(p4.launches()) == key(tuned)
    p4.execute()
    assert all(r.status == gb.CONVERGED for r in p4.results())
    p4.close()
    plan.close()


@pytest.mark.parametrize("text", ["1 2 3", "0 0 0 0 0 0 0 14 32 : 1 2 0 1 100",
                                  "0 0 0 0 0 0 0 14 32 : 9 1 0 1 128", "0 0 0 0 0 9 0 14 32 : 1 2 0 1 128"])
def test_tuning_table_rejects_bad_lines(gb, handle, text):
    handle.tune_clear()
    with pytest.raises(gb.GbdpcgError):
        handle.tune_import(text)
    assert handle.tune_export() == ""


def test_autotune_adjoint_plan_leaves_outputs(gb, oracle_mod, handle):
    """Tuning an adjoint plan solves into scratch: lambda (dL/dgamma) and dS keep
    what they held."""
    import torch
    O = oracle_mod
    d = torch.device("cuda:0")
    handle.tune_clear()
    systems, _ = _batch(O, range(700, 716), d)
    fwd = gb.Plan(handle, systems, gb.PINV_BLOCKDIAG, _cfg(gb, zero_guess=1))
    fwd.execute()
    torch.cuda.synchronize()
    adj = []
    for s in systems:
        adj.append({"S": s["S"], "Pinv": s["Pinv"], "gamma": torch.randn_like(s["gamma"]),
                    "lambda": torch.full_like(s["gamma"], 3.0), "lambda_fwd": s["lambda"],
                    "dS": torch.full_like(s["S"], 5.0), "n": s["n"], "N": s["N"]})
    pa = gb.Plan(handle, adj, gb.PINV_BLOCKDIAG, _cfg(gb))
    pa.autotune(reps=1)
    torch.cuda.synchronize()
    for a in adj:
        assert bool((a["lambda"] == 3.0).all()) and bool((a["dS"] == 5.0).all())
    pa.execute()
    res = pa.results()
    assert all(r.status == gb.CONVERGED for r in res)
    for a in adj:
        assert not bool((a["dS"] == 5.0).all())
    pa.close()
    fwd.close()
    handle.tune_clear()
