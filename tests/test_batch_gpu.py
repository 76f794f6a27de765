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


@pytest.mark.parametrize("nw,packed16,rows", [(4, -1, 4), (8, -1, 4), (4, 1, 4), (8, 1, 4), (8, -1, 2),
                                              (8, 1, 2)])
def test_mixed_uneven(gme_ctx, nw, packed16, rows):
    rng = np.random.default_rng(31 + nw)
    n = 600
    kinds = rng.integers(0, 3, n)
    la = np.exp(rng.uniform(np.log(1), np.log(3000), n)).astype(int)
    lb = np.exp(rng.uniform(np.log(1), np.log(3000), n)).astype(int)
    sa = [rng.integers(0, 4, k) for k in la]
    sb = [rng.integers(0, 4, k) for k in lb]
    # at 2 rows per lane the packed engine does not exist: packed16=1 runs int32
    gme_ctx.set_batch_config(warps_per_block=nw, block_min_cells=1 << 18, packed16=packed16, rows_per_lane=rows)
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


@pytest.mark.parametrize("nw,rows", [(4, 4), (8, 4), (8, 2)])
def test_wide_pairs(gme_ctx, nw, rows):
    """Rows of 4097..16384 columns: block jobs (tagged wrap rows in global memory) and warp jobs."""
    rng = np.random.default_rng(101 + nw)
    n = 60
    kinds = rng.integers(0, 3, n)
    la = rng.integers(4097, 16385, n)
    lb = np.exp(rng.uniform(np.log(1), np.log(3000), n)).astype(int)
    sa = [rng.integers(0, 4, k) for k in la]
    sb = [rng.integers(0, 4, k) for k in lb]
    gme_ctx.set_batch_config(warps_per_block=nw, block_min_cells=1 << 20, rows_per_lane=rows)
    try:
        for _ in range(2):  # the second run reuses the wrap rows with newer tags
            check_batch(gme_ctx, kinds, sa, sb, rule=0)
        st = gme_ctx.batch_stats()
        assert st["block_jobs"] > 0 and st["warp_jobs"] > 0 and st["long_jobs"] == 0
    finally:
        gme_ctx.set_batch_config()


@pytest.mark.parametrize("nw,split,rows", [(4, 2, 4), (8, 2, 4), (4, 3, 4), (4, 1, 4), (8, 2, 2), (8, 3, 2)])
def test_team_jobs(gme_ctx, nw, split, rows):
    """Pairs shared by teams of CTAs (every T-th band group per CTA, rows handed over
    through global tagged rows, T = groups / split in 2..8); SW maxima with ties
    combined across the team."""
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
                             block_min_cells=1 << 20, packed16=1 if nw == 4 else -1, team_split=split,
                             rows_per_lane=rows)
    try:
        for _ in range(2):
            check_batch(gme_ctx, kinds, sa, sb, rule=1)
        st = gme_ctx.batch_stats()
        assert st["team_jobs"] > 20 and st["block_jobs"] > 0 and st["warp_jobs"] > 0
        assert st["long_jobs"] == 0
    finally:
        gme_ctx.set_batch_config()


@pytest.mark.parametrize("packed16", [-1, 1])
def test_engine_selection(gme_ctx, packed16):
    """Pairs on the packed 16-bit engine beside pairs that must stay on int32: symbols
    outside [0, 65535], and SW scorings whose maxima could leave 16 bits."""
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(404)
    kinds, sa, sb = [], [], []
    for i in range(90):
        n1, n2 = int(rng.integers(1, 2500)), int(rng.integers(1, 2500))
        if i % 3 == 0:    # full int32 range in one sequence: int32 engine
            a = rng.integers(-2**31, 2**31 - 1, n1)
            b = a[:n2].copy() if n2 <= n1 else rng.integers(-2**31, 2**31 - 1, n2)
        elif i % 3 == 1:  # just above the 16-bit engine's symbol range
            a = rng.integers(32760, 32775, n1)
            b = rng.integers(32760, 32775, n2)
        else:             # small alphabet: packed engine
            a = rng.integers(0, 4, n1)
            b = rng.integers(0, 4, n2)
        kinds.append(i % 3 if i < 60 else 2)
        sa.append(a)
        sb.append(b)
    gme_ctx.set_batch_config(packed16=packed16, block_min_cells=1 << 21)
    try:
        for rule in (0, 1):
            check_batch(gme_ctx, kinds, sa, sb, rule=rule)
        # SW maxima near and beyond the 16-bit bound (match 40: 40 x 800 = 32000)
        sk = [2] * 12
        sa2 = [np.zeros(n, int) for n in (700, 790, 801, 900, 2000, 3000)] * 2
        sb2 = [np.zeros(n, int) for n in (700, 790, 801, 900, 2000, 3000)] * 2
        check_batch(gme_ctx, sk, sa2, sb2, sc=g.scoring(40, -40, -40))
        check_batch(gme_ctx, sk, sa2, sb2, sc=g.scoring(3, -3, -2))
        # ED and LCS at the 16-bit bound (n1 + n2 = 32000 and just above), as block jobs
        kinds3 = [1, 1, 0, 0]
        sa3 = [rng.integers(0, 4, 16000), rng.integers(0, 4, 16001), rng.integers(0, 4, 16000), np.zeros(9000, int)]
        sb3 = [rng.integers(0, 4, 16000), rng.integers(0, 4, 16000), rng.integers(0, 4, 500), np.zeros(8000, int)]
        check_batch(gme_ctx, kinds3, sa3, sb3, rule=1)
    finally:
        gme_ctx.set_batch_config()


@pytest.mark.parametrize("rule,packed16", [(0, 1), (1, 1), (1, -1)])
def test_batch_last_rows_and_columns(gme_ctx, rule, packed16):
    """Each pair's last row and last column from one batch, as the plain path gives them:
    warp, block and team jobs, both engines, pairs on the plain path, pairs skipped."""
    import torch
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(808 + rule)
    kinds, sa, sb = [], [], []
    shapes = [(int(rng.integers(1, 3000)), int(rng.integers(1, 3000))) for _ in range(80)]
    shapes += [(16384, 300), (17000, 100), (9000, 4000), (0, 5), (6, 0), (3000, 9000)]
    for i, (n1, n2) in enumerate(shapes):
        kinds.append(i % 3)
        sa.append(rng.integers(0, 4, n1))
        sb.append(rng.integers(0, 4, n2))
    symbols, pairs = g.pack_batch(kinds, sa, sb)
    n = len(pairs)
    row_off = np.full(n, -1, np.int64)
    col_off = np.full(n, -1, np.int64)
    r = c = 0
    for i in range(n):
        if i % 7 != 3:
            row_off[i] = r
            r += len(sa[i]) + 1
        if i % 5 != 2:
            col_off[i] = c
            c += len(sb[i]) + 1
    dev = torch.device("cuda", 0)
    d_sym = torch.from_numpy(symbols).to(dev)
    d_res = torch.zeros(n * g.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    d_rows = torch.full((max(r, 1),), -7, dtype=torch.int32, device=dev)
    d_cols = torch.full((max(c, 1),), -7, dtype=torch.int32, device=dev)
    sc = g.scoring(ed_boundary=rule)
    gme_ctx.set_batch_config(team_min_cells=1 << 20, block_min_cells=1 << 20, packed16=packed16)
    try:
        gme_ctx.align_batch_device_rows(d_sym.data_ptr(), len(symbols), pairs, d_res.data_ptr(),
                                        d_rows.data_ptr(), row_off, d_cols.data_ptr(), col_off, sc=sc)
        torch.cuda.synchronize()
        st = gme_ctx.batch_stats()
    finally:
        gme_ctx.set_batch_config()
    assert st["team_jobs"] > 0 and st["block_jobs"] > 0 and st["warp_jobs"] > 0 and st["long_jobs"] > 0
    res = np.frombuffer(d_res.cpu().numpy().tobytes(), g.RESULT_DTYPE)
    rows = d_rows.cpu().numpy()
    cols = d_cols.cpu().numpy()
    for i in range(n):
        o = O.align(kinds[i], sa[i], sb[i], rule=rule)
        assert res["status"][i] == 0 and res["score"][i] == o["score"], i
        if row_off[i] >= 0:
            np.testing.assert_array_equal(rows[row_off[i]:row_off[i] + len(sa[i]) + 1], o["last_row"],
                                          err_msg=f"pair {i} row")
        if col_off[i] >= 0:
            np.testing.assert_array_equal(cols[col_off[i]:col_off[i] + len(sb[i]) + 1], o["last_col"],
                                          err_msg=f"pair {i} col")
    # skipped pairs leave the buffers alone
    used_r = np.zeros(len(rows), bool)
    for i in range(n):
        if row_off[i] >= 0:
            used_r[row_off[i]:row_off[i] + len(sa[i]) + 1] = True
    assert (rows[~used_r] == -7).all()


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


def test_fill_teams(gme_ctx):
    """A planned batch of a few large pairs, too few to fill the grid one pair per CTA:
    the plan shares them among teams sized to the grid, and pairs with a single band
    group stay on one CTA; results as the oracle's, SW positions included."""
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(515)
    kinds = list(rng.integers(0, 3, 12)) + [0, 1, 2]
    sa = [rng.integers(0, 4, int(k)) for k in rng.integers(2000, 4100, 12)] + \
         [rng.integers(0, 4, 9000) for _ in range(3)]
    sb = [rng.integers(0, 4, int(k)) for k in rng.integers(2000, 4100, 12)] + \
         [rng.integers(0, 4, 1000) for _ in range(3)]
    gme_ctx.set_batch_config()
    for rule in (0, 1):
        check_batch(gme_ctx, kinds, sa, sb, rule=rule)
        st = gme_ctx.batch_stats()
        assert st["team_jobs"] >= 10 and st["long_jobs"] == 0
    check_batch(gme_ctx, kinds, sa, sb, sc=g.scoring(5, -4, -7))


def test_rows_per_lane_config(gme_ctx):
    """2 rows per lane runs with 8 warps per CTA only: asked with 4 it is refused, and
    asked alone it takes 8; other values are refused."""
    import gpumemefficient_gb300 as g
    for bad in (dict(rows_per_lane=2, warps_per_block=4), dict(rows_per_lane=3), dict(rows_per_lane=8)):
        with pytest.raises(g.GmeError):
            gme_ctx.set_batch_config(**bad)
    rng = np.random.default_rng(91)
    kinds = rng.integers(0, 3, 40)
    sa = [rng.integers(0, 4, int(k)) for k in rng.integers(1, 2500, 40)]
    sb = [rng.integers(0, 4, int(k)) for k in rng.integers(500, 2500, 40)]
    gme_ctx.set_batch_config(rows_per_lane=2, block_min_cells=1 << 18)
    try:
        check_batch(gme_ctx, kinds, sa, sb)
        assert gme_ctx.batch_stats()["block_jobs"] > 0
    finally:
        gme_ctx.set_batch_config()
