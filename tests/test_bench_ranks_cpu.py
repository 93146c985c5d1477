"""Multi-rank pieces of bench.py on CPU ranks (gloo, world size 2).

A multi-GPU bench run is one process per GPU; the job's batch is split over
the ranks by estimated cost with the library's partitioner, each rank solving
its own part (no exchange of data between ranks: the systems are
independent), timed between barriers, with the slowest rank's time taken as
the job's and the whole-job rate = the job's systems / that time.  These
tests run the same helpers on two gloo ranks on the host.
"""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    for p in (ROOT, os.path.join(ROOT, "gbd-pcg_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        count = 6
        seeds = list(bench.rank_seeds(rank, count, world))
        descs, Sa, ga, nP = bench.build_batch(rank, count, 1, world)
        all_seeds = [None] * world
        dist.all_gather_object(all_seeds, seeds)
        digests = [None] * world
        dist.all_gather_object(digests, float(np.abs(ga).sum()))
        dist.barrier()
        elapsed = 0.25 * (rank + 1)  # rank r "took" 0.25 (r + 1) s
        slowest = bench.max_over_ranks(elapsed, world)
        rate = bench.whole_job_rate(world * count, 4, slowest)
        np.save(os.path.join(out_dir, f"rank{rank}.npy"),
                np.array([slowest, rate, len(descs)], np.float64))
        if rank == 0:
            np.save(os.path.join(out_dir, "seeds.npy"), np.array(sum(all_seeds, [])))
            np.save(os.path.join(out_dir, "split.npy"), np.array([len(x) for x in all_seeds]))
            np.save(os.path.join(out_dir, "digests.npy"), np.array(digests))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_weak_scaling(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn", join=True)
    seeds = np.load(tmp_path / "seeds.npy")
    split = np.load(tmp_path / "split.npy")
    assert sorted(seeds) == list(range(12))            # the job's batch, each system on one rank
    assert split.sum() == 12 and (split > 0).all()
    d = np.load(tmp_path / "digests.npy")
    assert d[0] != d[1]                                # different data, no replica
    for r in range(world):
        slowest, rate, ndesc = np.load(tmp_path / f"rank{r}.npy")
        assert slowest == pytest.approx(0.5)          # the max over ranks, seen by every rank
        assert rate == pytest.approx(2 * 6 * 4 / 0.5)  # all ranks' systems / slowest time
        assert ndesc == split[r]


def test_single_rank_helpers_need_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert list(bench.rank_seeds(0, 4)) == [0, 1, 2, 3]
    assert bench.whole_job_rate(4096, 20, 2.0) == pytest.approx(40960.0)


def test_reference_arm_other_ranks_do_no_work(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(bench, "build_batch", lambda *a, **k: pytest.fail("rank 1 built a batch"))

    class A:
        systems, steps, warmup = 8, 1, 1
    assert bench.run_reference(A()) is None
