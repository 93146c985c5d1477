"""The measurement entry points: a plan's per-system timeline
(gbdpcg_plan_timeline / _read) and the latency probes of the synchronisation
primitives (gbdpcg_probe_primitives) and of the bounded wait's failure path
(gbdpcg_probe_timeout)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _plan(gb, O, handle, seeds, algorithm=0):
    import torch
    d = torch.device("cuda:0")
    systems = []
    for seed in seeds:
        s = O.generate_mixed(seed)
        systems.append({"S": torch.from_numpy(s.cbtd(np.float32)).to(d),
                        "Pinv": torch.from_numpy(O.block_jacobi(s.D, "compact").astype(np.float32)).to(d),
                        "gamma": torch.from_numpy(s.gamma.astype(np.float32)).to(d),
                        "lambda": torch.zeros(s.n * s.N, device=d), "n": s.n, "N": s.N})
    cfg = gb.config(max_iter=300, exit_mode=gb.EXIT_RELRES, zero_guess=1, algorithm=algorithm)
    return gb.Plan(handle, systems, gb.PINV_BLOCKDIAG, cfg), systems


@pytest.mark.parametrize("algorithm", ["standard", "recurrence", "single-reduction"])
def test_timeline_records_every_system(gb, oracle_mod, handle, algorithm):
    """One record per system: ordered times, the plan's own iteration counts,
    valid SMs; switching the timeline on and off leaves the solution bits as
    they are."""
    import torch
    algo = {"standard": gb.ALGO_CLUSTER, "recurrence": gb.ALGO_RECURRENCE,
            "single-reduction": gb.ALGO_SINGLE_REDUCTION}[algorithm]
    plan, systems = _plan(gb, oracle_mod, handle, range(40), algo)
    plan.execute()
    torch.cuda.synchronize()
    ref = [s["lambda"].cpu().numpy().tobytes() for s in systems]
    plan.timeline(True)
    plan.execute()
    st, sms = plan.timeline_read()
    res = plan.results()
    launches = plan.launches()
    assert len(st) == 40 and sorted(st["system"]) == list(range(40))
    assert (st["t_pop"] <= st["t_staged"]).all() and (st["t_staged"] <= st["t_solved"]).all()
    assert (st["t_solved"] <= st["t_done"]).all() and (st["t_pop"] > 0).all()
    for rec in st:
        assert rec["iters"] == res[rec["system"]].iters > 0
        assert rec["launch"] < len(launches)
        assert rec["cluster"] < launches[rec["launch"]]["ctas"] // launches[rec["launch"]]["cluster"]
    assert len(sms) == sum(l["ctas"] for l in launches)
    assert (sms < torch.cuda.get_device_properties(0).multi_processor_count).all()
    assert [s["lambda"].cpu().numpy().tobytes() for s in systems] == ref
    plan.timeline(False)
    plan.execute()
    torch.cuda.synchronize()
    assert [s["lambda"].cpu().numpy().tobytes() for s in systems] == ref
    with pytest.raises(gb.GbdpcgError):
        plan.timeline_read()
    plan.close()


@pytest.mark.parametrize("C,threads", [(1, 128), (4, 384), (16, 256)])
def test_probe_primitives(gb, handle, C, threads):
    p = gb.probe_primitives(0, C, threads, clusters=1, reps=20000)
    assert p["syncthreads_ns"] > 0 and p["loop_ns"] > 0
    assert all(x > 0 for x in p["allreduce_ns"])
    if C == 1:
        assert p["cluster_barrier_ns"] == 0 and p["dsmem_store_barrier_ns"] == 0
    else:
        assert p["cluster_barrier_ns"] > 0 and p["dsmem_store_barrier_ns"] > 0
        # a reduction contains a cluster barrier
        assert p["allreduce_ns"][0] >= 0.5 * p["cluster_barrier_ns"]
        # the transaction-counted form completes (a wait that gave up raises)
        assert all(x > 0 for x in p["allreduce_tx_ns"])
    with pytest.raises(gb.GbdpcgError):
        gb.probe_primitives(0, 17, threads, 1, 10)


@pytest.mark.parametrize("C", [1, 2, 8])
def test_bounded_wait_gives_up_and_the_context_stays_usable(gb, oracle_mod, handle, C):
    """The solver's failure path, made without a fault: a wait that nothing
    completes (for C >= 2 a cluster reduction whose receivers also expect halo
    bytes no neighbour sends) gives up after about a second with
    GBDPCG_TIMEOUT, and the same context then solves a batch (true relative
    residual within 1e-4 by the oracle's FP64 product)."""
    import torch
    st, ms = gb.probe_timeout(0, C)
    assert st == gb.TIMEOUT
    assert 900.0 <= ms <= 10000.0
    plan, systems = _plan(gb, oracle_mod, handle, range(8))
    plan.execute()
    torch.cuda.synchronize()
    res = plan.results()
    assert all(r.status == gb.CONVERGED for r in res)
    for i, s in enumerate(systems):
        sy = oracle_mod.generate_mixed(i)
        assert oracle_mod.relres(sy.cbtd(np.float64), s["lambda"].cpu().numpy(), sy.gamma, sy.n, sy.N) <= 1e-4
    with pytest.raises(gb.GbdpcgError):
        gb.probe_timeout(0, 17)
    plan.close()
