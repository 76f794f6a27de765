"""Replicas across GPUs: one process per GPU, each aligning its own share of
independent pairs.  Pairs never depend on one another, so there is no data-path
collective; the only communication is the timing and count reduction after the
timed region.

* ``shard_by_cells(cells, world)``: per-rank pair indices, balanced by cells
  (longest first onto the least-loaded rank), each rank's list in input order.
* ``aggregate(t_local, units_local)``: the job's wall time (max over ranks) and
  total work (sum over ranks) through ``torch.distributed``; with one process it
  returns the local values.
"""
from __future__ import annotations

import heapq

import numpy as np


def shard_by_cells(cells, world: int):
    """Indices of the pairs each of `world` ranks takes, balancing the sum of cells."""
    cells = np.asarray(cells, dtype=np.float64)
    if world < 1:
        raise ValueError("world must be >= 1")
    heap = [(0.0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for i in np.argsort(-cells, kind="stable"):
        load, r = heapq.heappop(heap)
        parts[r].append(int(i))
        heapq.heappush(heap, (load + float(cells[i]), r))
    return [np.sort(np.asarray(p, dtype=np.int64)) for p in parts]


def aggregate(t_local: float, units_local: float, device=None):
    """(max over ranks of t_local, sum over ranks of units_local)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(t_local), float(units_local)
    t = torch.tensor([float(t_local)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units_local)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())
