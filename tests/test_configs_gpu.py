"""The named single-pair workloads at their full sizes on the GPU, bit-exact against the
oracle (its blocked wavefront on all host threads), through the C ABI:

* LCS, one pair 8192 x 8192, i.i.d. uniform over 4 symbols (LCS/LCS.cpp:45-82):
  the LCS length, the last row and the last column;
* edit distance, one pair 65536 x 65536, the second sequence the first with 10% seeded
  edits (EditDistance/ED.cpp:45-80): the score, the last row and the last column, under
  both borders and two kernel shapes;
* Smith-Waterman, one pair 32768 x 32768 over 20 symbols with a 2048-long segment
  planted in both, mutated at 15% (SmithWaterman/SW.cpp:45-83, +3/-3/-2): the corner
  cell, the maximum and its cell (first in row-major order), the last row and column.

These are the shapes the benchmark lines are quoted on, so a green run here means the
numbers there come from correct results."""
import os

import numpy as np
import pytest

from gpumemefficient_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def _check(r, o, kind):
    assert r.score == o["score"]
    np.testing.assert_array_equal(r.last_row, o["last_row"])
    np.testing.assert_array_equal(r.last_col, o["last_col"])
    if kind == O.SW:
        assert (r.sw_max, r.sw_max_y, r.sw_max_x) == (o["sw_max"], o["sw_y"], o["sw_x"])


def test_lcs_8192(gme_ctx):
    a, b = synth.lcs_pair(8192)
    o = O.align(O.LCS, a, b, threads=THREADS)
    r = gme_ctx.align("lcs", a, b, last_row=True, last_col=True)
    _check(r, o, O.LCS)


@pytest.fixture(scope="module")
def ed_pair():
    return synth.ed_pair(65536)


@pytest.mark.parametrize("rule", [O.ED_REF_CPU, O.ED_STANDARD])
def test_ed_65536(gme_ctx, ed_pair, rule):
    import gpumemefficient_gb300 as g
    a, b = ed_pair
    o = O.align(O.ED, a, b, rule=rule, threads=THREADS)
    sc = g.scoring(ed_boundary=rule)
    # the automatic (tuned) shape, then a second shape with taller bands
    for shape in ((0, 0), (4, 8)):
        gme_ctx.set_plain_config(*shape)
        try:
            r = gme_ctx.align("ed", a, b, sc=sc, last_row=True, last_col=True)
        finally:
            gme_ctx.set_plain_config()
        _check(r, o, O.ED)


def test_sw_32768_planted(gme_ctx):
    a, b = synth.sw_pair(32768)
    o = O.align(O.SW, a, b, threads=THREADS)
    # the planted segment must dominate: a maximum far above what chance gives
    assert o["sw_max"] > 1000
    r = gme_ctx.align("sw", a, b, last_row=True, last_col=True)
    _check(r, o, O.SW)
