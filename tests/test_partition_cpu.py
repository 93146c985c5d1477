"""One batch over several GPUs (gbdpcg_partition, gbdpcg.distributed): the
batch split by estimated cost, each rank solving its own part, the results
gathered in input order.  Runs on the host: the split is host code, and the
two ranks are gloo processes that solve their parts with the oracle's CPU
PCG (the CUDA solver's GPU runs are covered by the -m gpu tests)."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _sizes(count):
    from gbdpcg.workload import mixed_size
    return np.array([mixed_size(s) for s in range(count)], np.uint32)


@pytest.mark.parametrize("parts", [2, 4, 8])
def test_partition_balances_the_mixed_batch(gb, parts):
    """The 4096-system mixed batch's cost model (n^2 N, and n^2 N x a per-system
    iteration estimate): every part within 5% of the mean, every system in
    exactly one part, the same split on every call."""
    from gbdpcg import distributed as D
    sz = _sizes(4096)
    for iters in (None, np.random.default_rng(parts).uniform(10, 60, 4096).astype(np.float32)):
        part_of, cost = D.partition(sz[:, 0], sz[:, 1], parts, iters)
        assert part_of.max() < parts and len(part_of) == 4096
        w = (sz[:, 0].astype(np.float64) ** 2) * sz[:, 1] * (1 if iters is None else iters)
        assert np.allclose([w[part_of == p].sum() for p in range(parts)], cost)
        assert cost.max() <= 1.05 * cost.mean()
        again, _ = D.partition(sz[:, 0], sz[:, 1], parts, iters)
        assert (again == part_of).all()
        assert sorted(np.concatenate([D.rank_items(part_of, p) for p in range(parts)])) == list(range(4096))


def test_partition_rejects_bad_arguments(gb):
    from gbdpcg import distributed as D
    with pytest.raises(gb.GbdpcgError):
        D.partition([4, 0], [8, 8], 2)
    with pytest.raises(gb.GbdpcgError):
        D.partition([4], [8], 0)
    with pytest.raises(ValueError):
        D.partition([4, 5], [8], 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _small_batch(count):
    """Small systems the CPU PCG solves in milliseconds: n in {3, 4, 6}, N in 4..12."""
    from oracle import oracle as O
    rng = np.random.default_rng(77)
    out = []
    for i in range(count):
        n, N = int(rng.choice([3, 4, 6])), int(rng.integers(4, 13))
        sy = O.generate(n, N, 500 + i)
        out.append((n, N, sy.cbtd(np.float32), O.block_jacobi(sy.D, "compact").astype(np.float32),
                    sy.gamma.astype(np.float32)))
    return out


def _solve(O, sys_):
    n, N, S, P, g = sys_
    lam, it, st, _, _ = O.pcg(S, P, g, np.zeros(n * N, np.float32), n, N, 200, 1e-6,
                              flags=O.PINV_BLOCKDIAG | O.EXIT_RELRES)
    return lam.tobytes().hex(), int(it)


def _rank_main(rank, world, port, out_dir):
    for p in (ROOT, os.path.join(ROOT, "gbd-pcg_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch.distributed as dist
    from gbdpcg import distributed as D
    from oracle import oracle as O
    O.lib()
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        batch = _small_batch(40)
        part_of, cost = D.partition([b[0] for b in batch], [b[1] for b in batch], world)
        mine = D.rank_items(part_of, rank)
        values = [_solve(O, batch[i]) for i in mine]   # each rank solves only its part
        allv = D.gather_in_order(mine, values, len(batch))
        np.save(os.path.join(out_dir, f"rank{rank}.npy"),
                np.array([len(mine), cost[rank]], np.float64))
        with open(os.path.join(out_dir, f"gathered{rank}.txt"), "w") as f:
            f.write("\n".join(f"{h} {it}" for h, it in allv))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_solve_their_parts_and_gather_in_order(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    for p in (ROOT, os.path.join(ROOT, "gbd-pcg_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    from oracle import build_oracle
    build_oracle.build()
    from oracle import oracle as O
    O.lib()
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn", join=True)
    serial = [_solve(O, s) for s in _small_batch(40)]
    for r in range(world):
        got = open(tmp_path / f"gathered{r}.txt").read().split("\n")
        assert got == [f"{h} {it}" for h, it in serial]   # every rank: all results, input order
    counts = [np.load(tmp_path / f"rank{r}.npy") for r in range(world)]
    assert sum(int(c[0]) for c in counts) == 40 and all(c[0] > 0 for c in counts)
    costs = [c[1] for c in counts]
    assert max(costs) <= 1.05 * (sum(costs) / world)
