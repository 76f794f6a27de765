"""Alignment paths (Hirschberg on the GPU): every script is a valid alignment whose
cost equals the oracle's optimal score."""
import numpy as np
import pytest

from conftest import load_fixture
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def check_path(ctx, kind, a, b):
    score, ops = ctx.align_path(kind, a, b)
    a = np.asarray(a)
    b = np.asarray(b)
    assert set(ops) <= {"M", "D", "I"}
    assert ops.count("M") + ops.count("D") == len(a)
    assert ops.count("M") + ops.count("I") == len(b)
    i = j = cost = 0
    for c in ops:
        if c == "M":
            if kind == 0:
                assert a[i] == b[j]  # LCS aligns equal symbols only
                cost += 1
            else:
                cost += int(a[i] != b[j])
            i += 1
            j += 1
        elif c == "D":
            cost += kind == 1
            i += 1
        else:
            cost += kind == 1
            j += 1
    want = O.align(kind, a, b, rule=O.ED_STANDARD, threads=8)["score"]
    assert score == want
    assert cost == want
    return ops


@pytest.mark.parametrize("kind", [0, 1])
def test_paths_small_and_degenerate(gme_ctx, kind):
    rng = np.random.default_rng(61 + kind)
    shapes = [(0, 0), (0, 7), (9, 0), (1, 1), (1, 50), (50, 1), (17, 300), (300, 17), (256, 256),
              (257, 255), (700, 2048), (3000, 1000), (1000, 3000), (5, 4000)]
    for n1, n2 in shapes:
        for alphabet in (2, 4, 20):
            a = rng.integers(0, alphabet, n1)
            b = rng.integers(0, alphabet, n2)
            check_path(gme_ctx, kind, a, b)


@pytest.mark.parametrize("kind", [0, 1])
def test_paths_related_and_large(gme_ctx, kind):
    from gpumemefficient_gb300 import synth
    a, b = synth.ed_pair(12000, rate=0.1, seed=77 + kind)
    ops = check_path(gme_ctx, kind, a, b[:11000])
    assert ops.count("M") > 9000  # a related pair aligns mostly on the diagonal
    check_path(gme_ctx, kind, np.arange(3000) % 7, np.arange(2900) % 5)


def test_lcs_path_on_reference_fixture(gme_ctx):
    # LCS/GPU_Hyperlane_Share.txt:102: "lcs length: 21469" for the 2^15 fixture
    a, b = load_fixture()
    ops = check_path(gme_ctx, 0, a, b)
    assert ops.count("M") == 21469


def test_path_rejects_sw_and_ref_cpu_border(gme_ctx):
    import ctypes
    import gpumemefficient_gb300 as g
    with pytest.raises(g.GmeError):
        gme_ctx.align_path(2, np.arange(10), np.arange(10))
    n = ctypes.c_int64()
    sc = g.scoring(ed_boundary=g.ED_REF_CPU)
    a = np.arange(10, dtype=np.int32)
    st = g.lib().gme_align_path(gme_ctx.handle, 1, a.ctypes.data, 10, a.ctypes.data, 10, ctypes.byref(sc),
                                None, 0, ctypes.byref(n), None)
    assert st == 1
