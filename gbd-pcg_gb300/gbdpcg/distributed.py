"""One batch of independent systems over several GPUs: one process (rank) per
GPU, each solving its own part with its own plan, no exchange of data while
they solve; the per-system results are gathered in input order afterwards.

  partition(n, N, parts, iters=None)  gbdpcg_partition: the batch split by
      estimated cost n^2 N iters (greedy longest-processing-time);
  rank_items(part_of, rank)           the input indices rank `rank` solves, in
      input order;
  gather_in_order(items, values, count, group=None)
      every rank's (indices, per-system values) gathered with
      torch.distributed.all_gather_object (host objects: results, not the
      systems' data), returned in input order on every rank.
"""
from __future__ import annotations

import ctypes

import numpy as np


def partition(n, N, parts: int, iters=None):
    """(part_of, part_cost): the part of each system and each part's cost."""
    from . import lib, _check
    n = np.ascontiguousarray(n, np.uint32)
    N = np.ascontiguousarray(N, np.uint32)
    if n.shape != N.shape or n.ndim != 1:
        raise ValueError("n and N must be 1-D arrays of the same length")
    it = None if iters is None else np.ascontiguousarray(iters, np.float32)
    if it is not None and it.shape != n.shape:
        raise ValueError("iters must have one entry per system")
    part_of = np.zeros(n.size, np.uint32)
    cost = np.zeros(parts, np.float64)
    P = ctypes.c_void_p
    _check(lib().gbdpcg_partition(n.ctypes.data_as(P), N.ctypes.data_as(P),
                                  None if it is None else it.ctypes.data_as(P), n.size, parts,
                                  part_of.ctypes.data_as(P), cost.ctypes.data_as(P)), "gbdpcg_partition")
    return part_of, cost


def rank_items(part_of, rank: int) -> np.ndarray:
    """Input indices of the systems part `rank` solves, ascending."""
    return np.flatnonzero(np.asarray(part_of) == rank)


def gather_in_order(items, values, count: int, group=None) -> list:
    """Every rank passes the input indices it solved and one value per index;
    every rank gets the list of all `count` values in input order."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    got = [None] * world
    dist.all_gather_object(got, (list(map(int, items)), list(values)), group=group)
    out = [None] * count
    for idx, vals in got:
        if len(idx) != len(vals):
            raise ValueError("one value per index")
        for i, v in zip(idx, vals):
            if out[i] is not None:
                raise ValueError(f"system {i} solved by two ranks")
            out[i] = v
    missing = [i for i, v in enumerate(out) if v is None]
    if missing:
        raise ValueError(f"systems not solved by any rank: {missing[:8]}")
    return out
