"""The comparison baselines (the reference's table-based strategies on the GPU:
one launch per anti-diagonal of tiles, or of cells) against the oracle: every kind,
both ED borders, ragged shapes around the tile sizes, SW maxima with ties."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1), (5, 300), (300, 5), (64, 128), (65, 129), (129, 257), (1000, 777), (777, 1000)]


def _run(ctx, strategy, kind, a, b, sc, tile_x=64, tile_y=128):
    import torch
    import gpumemefficient_gb300 as g
    da = torch.from_numpy(np.ascontiguousarray(a, np.int32)).cuda()
    db = torch.from_numpy(np.ascontiguousarray(b, np.int32)).cuda()
    table = torch.empty((len(b) + 1) * (len(a) + 1), dtype=torch.int32, device="cuda")
    out = torch.zeros(g.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    ctx.baseline_align_device(strategy, kind, da.data_ptr(), len(a), db.data_ptr(), len(b), table.data_ptr(),
                              out.data_ptr(), tile_x=tile_x, tile_y=tile_y, sc=sc,
                              stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return np.frombuffer(out.cpu().numpy().tobytes(), g.RESULT_DTYPE)[0]


@pytest.mark.parametrize("strategy,tile", [(0, (64, 128)), (0, (37, 50)), (0, (128, 32)), (1, (0, 0))])
@pytest.mark.parametrize("rule", [0, 1])
def test_baselines_match_oracle(gme_ctx, strategy, tile, rule):
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(strategy * 10 + tile[0] + rule)
    sc = g.scoring(4, -3, -5, ed_boundary=rule)
    for n1, n2 in SHAPES:
        for kind in range(3):
            a = rng.integers(0, 4, n1)
            b = rng.integers(0, 4, n2)
            r = _run(gme_ctx, strategy, kind, a, b, sc, *tile) if strategy == 0 else _run(gme_ctx, strategy, kind, a, b, sc)
            o = O.align(kind, a, b, rule=rule, match=4, mismatch=-3, gap=-5)
            assert r["score"] == o["score"], (strategy, tile, kind, n1, n2)
            if kind == 2:
                assert (r["sw_max"], r["sw_max_y"], r["sw_max_x"]) == (o["sw_max"], o["sw_y"], o["sw_x"])


def test_baselines_sw_ties_and_planted(gme_ctx):
    """Equal SW maxima in many rows and tiles: the first in row-major order wins."""
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(3)
    seg = rng.integers(0, 20, 300)
    a = np.concatenate([rng.integers(0, 20, 500), seg, rng.integers(0, 20, 400), seg])
    b = np.concatenate([seg, rng.integers(0, 20, 700), seg, seg])
    sc = g.scoring()
    o = O.align(2, a, b)
    for strategy in (0, 1):
        r = _run(gme_ctx, strategy, 2, a, b, sc)
        assert (r["score"], r["sw_max"], r["sw_max_y"], r["sw_max_x"]) == (o["score"], o["sw_max"], o["sw_y"], o["sw_x"])


def test_baseline_arguments_checked(gme_ctx):
    import torch
    import gpumemefficient_gb300 as g
    d = torch.zeros(16, dtype=torch.int32, device="cuda")
    out = torch.zeros(g.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    with pytest.raises(g.GmeError):  # a tile of more rows than a CTA has threads
        gme_ctx.baseline_align_device(0, 0, d.data_ptr(), 3, d.data_ptr(), 3, d.data_ptr(), out.data_ptr(),
                                      tile_x=4, tile_y=2048)
    with pytest.raises(g.GmeError):  # empty sequences have no table to sweep
        gme_ctx.baseline_align_device(1, 0, d.data_ptr(), 0, d.data_ptr(), 3, d.data_ptr(), out.data_ptr())
