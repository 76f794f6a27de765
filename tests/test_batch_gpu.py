"""Parity of the batched path (one launch, many uneven mixed pairs) with the oracle."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def check_batch(ctx, kinds, sa, sb, rule=0, sc=None):
    import gpumemefficient_gb300 as g
    sc = sc or g.scoring(ed_boundary=rule)
    res = ctx.align_batch(kinds, sa, sb, sc=sc)
    o = O.align_batch(kinds, sa, sb, rule=rule, match=sc.match, mismatch=sc.mismatch, gap=sc.gap)
    np.testing.assert_array_equal(res["status"], 0)
    np.testing.assert_array_equal(res["score"], o["score"])
    sw = np.asarray(kinds) == 2
    np.testing.assert_array_equal(res["sw_max"][sw], o["sw_max"][sw])
    np.testing.assert_array_equal(res["sw_max_y"][sw], o["sw_y"][sw])
    np.testing.assert_array_equal(res["sw_max_x"][sw], o["sw_x"][sw])
    return res


@pytest.mark.parametrize("nw", [4, 8])
def test_mixed_uneven(gme_ctx, nw):
    rng = np.random.default_rng(31 + nw)
    n = 600
    kinds = rng.integers(0, 3, n)
    la = np.exp(rng.uniform(np.log(1), np.log(3000), n)).astype(int)
    lb = np.exp(rng.uniform(np.log(1), np.log(3000), n)).astype(int)
    sa = [rng.integers(0, 4, k) for k in la]
    sb = [rng.integers(0, 4, k) for k in lb]
    gme_ctx.set_batch_config(warps_per_block=nw, block_min_cells=1 << 18)
    try:
        check_batch(gme_ctx, kinds, sa, sb, rule=0)
        check_batch(gme_ctx, kinds, sa, sb, rule=1)
        st = gme_ctx.batch_stats()
        assert st["block_jobs"] > 0 and st["warp_jobs"] > 0
    finally:
        gme_ctx.set_batch_config()


def test_shapes_edges(gme_ctx):
    rng = np.random.default_rng(77)
    shapes = [(1, 1), (1, 5), (5, 1), (0, 4), (4, 0), (0, 0), (1024, 512), (1025, 513), (4096, 4096),
              (4097, 100), (100, 4097), (513, 2000), (2000, 513), (128, 128), (129, 127), (7000, 300),
              (16384, 700), (16385, 40), (16000, 1500)]
    kinds, sa, sb = [], [], []
    for i, (n1, n2) in enumerate(shapes):
        for k in range(3):
            kinds.append(k)
            sa.append(rng.integers(0, 20, n1))
            sb.append(rng.integers(0, 20, n2))
    check_batch(gme_ctx, kinds, sa, sb)
    st = gme_ctx.batch_stats()
    assert st["long_jobs"] > 0


@pytest.mark.parametrize("nw", [4, 8])
def test_wide_pairs(gme_ctx, nw):
    """Rows of 4097..16384 columns: block jobs (tagged wrap rows in global memory) and warp jobs."""
    rng = np.random.default_rng(101 + nw)
    n = 60
    kinds = rng.integers(0, 3, n)
    la = rng.integers(4097, 16385, n)
    lb = np.exp(rng.uniform(np.log(1), np.log(3000), n)).astype(int)
    sa = [rng.integers(0, 4, k) for k in la]
    sb = [rng.integers(0, 4, k) for k in lb]
    gme_ctx.set_batch_config(warps_per_block=nw, block_min_cells=1 << 20)
    try:
        for _ in range(2):  # the second run reuses the wrap rows with newer tags
            check_batch(gme_ctx, kinds, sa, sb, rule=0)
        st = gme_ctx.batch_stats()
        assert st["block_jobs"] > 0 and st["warp_jobs"] > 0 and st["long_jobs"] == 0
    finally:
        gme_ctx.set_batch_config()


@pytest.mark.parametrize("nw", [4, 8])
def test_team_jobs(gme_ctx, nw):
    """Pairs shared by teams of CTAs (every T-th band group per CTA, rows handed over
    through global tagged rows); SW maxima with ties combined across the team."""
    rng = np.random.default_rng(202 + nw)
    kinds, sa, sb = [], [], []
    for i in range(24):
        n1 = int(rng.integers(100, 16385))
        n2 = int(rng.integers(2048 if nw == 4 else 4096, 9000))
        kinds.append(i % 3)
        sa.append(rng.integers(0, 4, n1))
        sb.append(rng.integers(0, 4, n2))
    # equal SW maxima in several rows and columns: the first in row-major order wins
    a = rng.integers(0, 20, 9000)
    seg = a[1000:1400]
    for reps in (6, 11):
        kinds.append(2)
        sa.append(a)
        sb.append(np.concatenate([seg] * reps + [rng.integers(0, 20, 300)]))
    kinds.append(2)
    sa.append(np.concatenate([seg, seg, seg]))
    sb.append(np.concatenate([seg] * 12))
    # small pairs beside them: one per warp and one per CTA
    for i in range(60):
        kinds.append(i % 3)
        sa.append(rng.integers(0, 4, int(rng.integers(1, 3000))))
        sb.append(rng.integers(0, 4, int(rng.integers(1, 3000))))
    gme_ctx.set_batch_config(warps_per_block=nw, team_min_cells=1 << 18, long_min_cells=-1,
                             block_min_cells=1 << 20)
    try:
        for _ in range(2):
            check_batch(gme_ctx, kinds, sa, sb, rule=1)
        st = gme_ctx.batch_stats()
        assert st["team_jobs"] > 20 and st["block_jobs"] > 0 and st["warp_jobs"] > 0
        assert st["long_jobs"] == 0
    finally:
        gme_ctx.set_batch_config()


def test_identical_and_disjoint(gme_ctx):
    rng = np.random.default_rng(5)
    kinds, sa, sb = [], [], []
    for n in (100, 700, 2500):
        a = rng.integers(0, 4, n)
        for k in range(3):
            kinds += [k, k]
            sa += [a, np.zeros(n, int)]
            sb += [a.copy(), np.ones(n + 3, int)]
    check_batch(gme_ctx, kinds, sa, sb)


def test_batch_sw_scoring(gme_ctx):
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(9)
    kinds = [2] * 40
    sa = [rng.integers(0, 6, rng.integers(50, 1500)) for _ in kinds]
    sb = [rng.integers(0, 6, rng.integers(50, 1500)) for _ in kinds]
    check_batch(gme_ctx, kinds, sa, sb, sc=g.scoring(5, -4, -7))


def test_block_cutoffs(gme_ctx):
    rng = np.random.default_rng(12)
    kinds = rng.integers(0, 3, 200)
    sa = [rng.integers(0, 4, rng.integers(10, 2100)) for _ in kinds]
    sb = [rng.integers(0, 4, rng.integers(10, 2100)) for _ in kinds]
    for cells in [1, 1 << 16, 1 << 20, 1 << 30]:
        gme_ctx.set_batch_config(block_min_cells=cells)
        try:
            check_batch(gme_ctx, kinds, sa, sb)
        finally:
            gme_ctx.set_batch_config()


def test_plan_graph_replay(gme_ctx):
    """A planned batch run three times: uncaptured, first graph run (captures), replay."""
    import torch
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(21)
    n = 300
    kinds = rng.integers(0, 3, n)
    sa = [rng.integers(0, 4, k) for k in np.exp(rng.uniform(0, np.log(2500), n)).astype(int)]
    sb = [rng.integers(0, 4, k) for k in np.exp(rng.uniform(0, np.log(2500), n)).astype(int)]
    sa[3] = rng.integers(0, 4, 17000)  # one pair for the plain path (n1 > 16384)
    symbols, pairs = g.pack_batch(kinds, sa, sb)
    o = O.align_batch(kinds, sa, sb)
    dev = torch.device("cuda", 0)
    d_sym = torch.from_numpy(symbols).to(dev)
    d_res = torch.zeros(n * g.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    plan = g.BatchPlan(gme_ctx, pairs, len(symbols))
    try:
        for use_graph in (False, True, True, True):
            d_res.zero_()
            torch.cuda.synchronize()
            plan.run(d_sym.data_ptr(), d_res.data_ptr(), use_graph=use_graph)
            torch.cuda.synchronize()
            res = np.frombuffer(d_res.cpu().numpy().tobytes(), g.RESULT_DTYPE)
            np.testing.assert_array_equal(res["status"], 0)
            np.testing.assert_array_equal(res["score"], o["score"])
    finally:
        plan.close()
