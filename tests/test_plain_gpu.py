"""Parity of the plain (one pair per call) CUDA path with the oracle, through the C ABI."""
import numpy as np
import pytest

from conftest import load_random_cases
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CONFIGS = [(4, 4), (4, 8), (2, 4), (2, 8)]


def check(ctx, kind, a, b, rule=0, sc=None):
    import gpumemefficient_gb300 as g
    sc = sc or g.scoring(ed_boundary=rule)
    r = ctx.align(kind, a, b, sc=sc, last_row=True, last_col=True)
    o = O.align(kind, a, b, rule=rule, match=sc.match, mismatch=sc.mismatch, gap=sc.gap,
                threads=8 if len(a) * len(b) > 4e6 else 1)
    assert r.score == o["score"], (kind, len(a), len(b))
    np.testing.assert_array_equal(r.last_row, o["last_row"])
    np.testing.assert_array_equal(r.last_col, o["last_col"])
    if kind == 2:
        assert (r.sw_max, r.sw_max_y, r.sw_max_x) == (o["sw_max"], o["sw_y"], o["sw_x"])
    return r


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_reference_kats(gme_ctx, kind, kat, fixture_seqs):
    a, b = fixture_seqs
    key = ["lcs", "ed", "sw_corner"][kind]
    for case in kat["cases"]:
        n = case["n"]
        r = gme_ctx.align(kind, a[:n], b[:n])
        assert r.score == case[key], (kind, n)


def test_reference_random_golden(gme_ctx):
    for c in load_random_cases():
        a, b = np.array(c["a"]), np.array(c["b"])
        assert gme_ctx.align(0, a, b).score == c["lcs"]
        assert gme_ctx.align(1, a, b).score == c["ed"]
        assert gme_ctx.align(2, a, b).score == c["sw_corner"]


@pytest.mark.parametrize("cfg", CONFIGS)
@pytest.mark.parametrize("kind", [0, 1, 2])
def test_random_shapes(gme_ctx, kind, cfg):
    rng = np.random.default_rng(100 * kind + cfg[0] + cfg[1])
    gme_ctx.set_plain_config(*cfg)
    try:
        shapes = [(1, 1), (1, 7), (7, 1), (3, 300), (300, 3), (129, 257), (1000, 999),
                  (5, 2000), (2000, 5), (4096, 300)]
        shapes += [tuple(rng.integers(1, 700, 2)) for _ in range(6)]
        for n1, n2 in shapes:
            alpha = int(rng.choice([2, 4, 20]))
            a = rng.integers(0, alpha, n1)
            b = rng.integers(0, alpha, n2)
            check(gme_ctx, kind, a, b, rule=int(rng.integers(0, 2)))
    finally:
        gme_ctx.set_plain_config(0, 0, 0)


@pytest.mark.parametrize("cfg", CONFIGS)
def test_chunk_boundaries(gme_ctx, cfg):
    """Widths around the chunk length (16 and 32 columns), the 32R-column skew of a
    warp's output (64, 128) and their sums, against heights around the band heights
    (256, 512, 1024 rows); all kinds, table and compare forms."""
    rng = np.random.default_rng(900 + cfg[0] * 10 + cfg[1])
    widths = [1, 2, 3, 4, 5, 15, 16, 17, 31, 32, 33, 63, 64, 65, 95, 96, 97, 127, 128, 129, 159, 160, 161,
              191, 192, 193, 255, 256, 257]
    heights = [1, 63, 255, 257, 511, 1025]
    gme_ctx.set_plain_config(*cfg)
    try:
        for i, n1 in enumerate(widths):
            for j, n2 in enumerate(heights):
                alpha = 4 if (i + j) % 2 == 0 else 20
                a = rng.integers(0, alpha, n1)
                b = rng.integers(0, alpha, n2)
                for kind in (0, 1, 2):
                    check(gme_ctx, kind, a, b, rule=(i + j + kind) % 2)
    finally:
        gme_ctx.set_plain_config(0, 0, 0)


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_extremes(gme_ctx, kind):
    rng = np.random.default_rng(7)
    a = rng.integers(0, 4, 1500)
    check(gme_ctx, kind, a, a.copy())                       # identical
    check(gme_ctx, kind, np.zeros(1500, int), np.ones(1300, int))  # no match at all
    check(gme_ctx, kind, np.full(800, 5), np.full(900, 5))   # all match
    big = np.array([2 ** 31 - 1, -2 ** 31, 0, 7] * 50)       # full int32 symbol range
    check(gme_ctx, kind, big, big[::-1].copy())


def test_empty_inputs(gme_ctx):
    for kind in (0, 1, 2):
        for rule in (0, 1):
            for n1, n2 in [(0, 0), (0, 5), (6, 0)]:
                check(gme_ctx, kind, np.arange(n1), np.arange(n2), rule=rule)


def test_sw_scoring_constants(gme_ctx):
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(3)
    a = rng.integers(0, 20, 3000)
    b = rng.integers(0, 20, 2500)
    for m, mm, gp in [(3, -3, -2), (5, -4, -7), (1, -1, -1), (2, 0, -1)]:
        check(gme_ctx, 2, a, b, sc=g.scoring(m, mm, gp))


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_large_square(gme_ctx, kind, fixture_seqs):
    a, b = fixture_seqs
    for cfg in [(0, 0), (4, 4), (4, 8)]:
        gme_ctx.set_plain_config(*cfg)
        try:
            check(gme_ctx, kind, a[:8192], b[:8192])
        finally:
            gme_ctx.set_plain_config(0, 0, 0)


def test_repeated_calls_reuse_workspace(gme_ctx):
    rng = np.random.default_rng(11)
    for i in range(30):
        n1, n2 = (int(x) for x in rng.integers(50, 3000, 2))
        kind = i % 3
        check(gme_ctx, kind, rng.integers(0, 4, n1), rng.integers(0, 4, n2), rule=i % 2)


def test_reference_signatures(gme_ctx, fixture_seqs):
    import gpumemefficient_gb300 as g
    a, b = fixture_seqs
    n = 2048
    assert g.LCS(n, n, a, b, 3, 1, None) == O.align(0, a[:n], b[:n])["score"]
    assert g.ED(n, n, a, b, 3, 1, None, 32, 128) == O.align(1, a[:n], b[:n], rule=1)["score"]
    assert g.SW(n, n, a, b, 3, 1, None, 32, 128) == O.align(2, a[:n], b[:n])["score"]
    # the C-callable forms of the reference signatures
    L = g.lib()
    aa = np.ascontiguousarray(a[:n], np.int32)
    bb = np.ascontiguousarray(b[:n], np.int32)
    assert L.gme_ref_ed(n, n, aa.ctypes.data, bb.ctypes.data) == O.align(1, aa, bb, rule=1)["score"]


@pytest.mark.parametrize("cfg", [(0, 0), (4, 4), (2, 8)])
def test_cost_forms(gme_ctx, cfg):
    """The plain kernel stages a pair either as PRMT cost tables (every symbol within 7
    consecutive values, scoring constants in signed bytes, SW gap <= 0) or as the
    symbols themselves; both must match the oracle, including at the boundary of the
    choice and for symbol ranges anywhere in int32."""
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(77 + cfg[0] + cfg[1])
    gme_ctx.set_plain_config(*cfg)
    try:
        ranges = [(0, 7), (0, 8), (100, 107), (-3, 4), (-2 ** 31, -2 ** 31 + 7),
                  (2 ** 31 - 7, 2 ** 31), (2 ** 31 - 8, 2 ** 31), (5, 6)]
        for lo, hi in ranges:
            n1, n2 = int(rng.integers(200, 900)), int(rng.integers(200, 900))
            a = rng.integers(lo, hi, n1, dtype=np.int64).astype(np.int32)
            b = rng.integers(lo, hi, n2, dtype=np.int64).astype(np.int32)
            for kind in (0, 1, 2):
                check(gme_ctx, kind, a, b, rule=int(rng.integers(0, 2)))
        # SW scorings the byte tables cannot hold (or whose ramp needs gap <= 0)
        a = rng.integers(0, 4, 700).astype(np.int32)
        b = rng.integers(0, 4, 650).astype(np.int32)
        for m, mm, gp in [(200, -3, -2), (3, -130, -2), (1, -1, 1), (127, -128, 0)]:
            check(gme_ctx, 2, a, b, sc=g.scoring(m, mm, gp))
    finally:
        gme_ctx.set_plain_config(0, 0, 0)
