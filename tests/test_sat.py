"""The summed-area-table oracle (CPU only): the C restatement of the reference's
SAT recurrence (SAT/GPU_Hyperlane_Share.cu:169,196,231) against its closed form.

The reference ships no SAT outputs to pin against: its host function never copies
the table back (SAT/GPU_Hyperlane_Share.cu:321), and its GPU kernels cannot run
here.  So the oracle is checked against an independent restatement instead: the
recurrence telescopes to t[y][x] = A[y][0] + A[0][x] - A[0][0] + the sum of the
interior rectangle, evaluated with numpy cumulative sums.
"""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.mark.parametrize("n1,n2,pad", [(1, 1, 3), (2, 5, 3), (31, 33, 3), (256, 32, 3),
                                       (257, 65, 0), (1000, 7, 40), (7, 1000, 1)])
def test_sat_oracle_matches_closed_form(n1, n2, pad):
    rng = np.random.default_rng(n1 * 1009 + n2)
    # the reference's generator: values rand() % 10000 over (n2 + 3) x (n1 + 3)
    t = rng.integers(0, 10000, (n2 + 3, n1 + 1 + pad)).astype(np.int32)
    got = O.sat(t, n1, n2)
    np.testing.assert_array_equal(got, O.sat_py(t, n1, n2))
    # untouched: row 0, column 0, columns beyond n1, rows beyond n2
    np.testing.assert_array_equal(got[0], t[0])
    np.testing.assert_array_equal(got[:, 0], t[:, 0])
    np.testing.assert_array_equal(got[:, n1 + 1:], t[:, n1 + 1:])
    np.testing.assert_array_equal(got[n2 + 1:], t[n2 + 1:])


def test_sat_oracle_wraps_like_int32():
    rng = np.random.default_rng(5)
    t = rng.integers(-2 ** 31, 2 ** 31, (70, 140), dtype=np.int64).astype(np.int32)
    np.testing.assert_array_equal(O.sat(t, 137, 68), O.sat_py(t, 137, 68))


def test_sat_oracle_small_by_hand():
    # the 2 x 2 interior, the recurrence written out cell by cell (left + up + self - up-left)
    t = np.array([[0, 1, 2, 9], [3, 4, 5, 9], [6, 7, 8, 9], [9, 9, 9, 9]], np.int32)
    got = O.sat(t, 2, 2)
    r11 = 3 + 1 + 4 - 0
    r12 = r11 + 2 + 5 - 1
    r21 = 6 + r11 + 7 - 3
    r22 = r21 + r12 + 8 - r11
    np.testing.assert_array_equal(got[1:3, 1:3], [[r11, r12], [r21, r22]])
    np.testing.assert_array_equal(got[:, 3], t[:, 3])


def test_sat_oracle_empty_is_identity():
    t = np.arange(20, dtype=np.int32).reshape(4, 5)
    np.testing.assert_array_equal(O.sat(t, 0, 3), t)
    np.testing.assert_array_equal(O.sat(t, 4, 0), t)


@pytest.mark.parametrize("threads", [1, 3, 8])
def test_sat_oracle_threaded_equals_sequential(threads):
    rng = np.random.default_rng(77 + threads)
    for n1, n2, pad in [(1, 1, 0), (5, 9, 3), (1024, 40, 3), (2500, 33, 7), (3, 2000, 0)]:
        t = rng.integers(-2 ** 31, 2 ** 31, (n2 + 2, n1 + 1 + pad), dtype=np.int64).astype(np.int32)
        np.testing.assert_array_equal(O.sat_mt(t, n1, n2, threads), O.sat(t, n1, n2))
