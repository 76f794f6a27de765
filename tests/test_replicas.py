"""Replicas across ranks without a GPU: cell-balanced sharding of independent pairs,
and the timing/work reduction over two gloo ranks (the multi-GPU path's host logic)."""
import os
import socket

import numpy as np
import pytest

from gpumemefficient_gb300.replicas import shard_by_cells


def test_shard_by_cells_covers_and_balances():
    rng = np.random.default_rng(3)
    cells = np.exp(rng.uniform(np.log(64), np.log(4096), 5000)).astype(int) ** 2
    for world in (1, 2, 3, 8):
        parts = shard_by_cells(cells, world)
        allidx = np.sort(np.concatenate(parts))
        assert (allidx == np.arange(len(cells))).all()
        loads = [cells[p].sum() for p in parts]
        assert max(loads) - min(loads) <= cells.max()
        assert all((np.diff(p) > 0).all() for p in parts)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    from gpumemefficient_gb300.replicas import aggregate, shard_by_cells
    from oracle import oracle as O
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(11)  # every rank draws the same job
    n = 60
    kinds = rng.integers(0, 3, n)
    sa = [rng.integers(0, 4, int(k)) for k in rng.integers(1, 300, n)]
    sb = [rng.integers(0, 4, int(k)) for k in rng.integers(1, 300, n)]
    cells = np.array([len(a) * len(b) for a, b in zip(sa, sb)])
    mine = shard_by_cells(cells, world)[rank]
    res = O.align_batch(kinds[mine], [sa[i] for i in mine], [sb[i] for i in mine], threads=1)
    t, units = aggregate(0.5 + rank, float(cells[mine].sum()))
    q.put((rank, mine.tolist(), res["score"].tolist(), t, units))
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_aggregate():
    import multiprocessing as mp
    from oracle import oracle as O
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    rng = np.random.default_rng(11)
    n = 60
    kinds = rng.integers(0, 3, n)
    sa = [rng.integers(0, 4, int(k)) for k in rng.integers(1, 300, n)]
    sb = [rng.integers(0, 4, int(k)) for k in rng.integers(1, 300, n)]
    whole = O.align_batch(kinds, sa, sb, threads=1)["score"]
    cells = np.array([len(a) * len(b) for a, b in zip(sa, sb)])
    got = np.zeros(n, np.int64)
    for rank, idx, scores, t, units in out:
        got[idx] = scores
        assert t == pytest.approx(1.5)              # max over ranks
        assert units == pytest.approx(cells.sum())  # sum over ranks
    assert (got == whole).all()
