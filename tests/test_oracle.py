"""The oracle against the reference's own answers (CPU only)."""
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_random_cases
from oracle import oracle as O


def test_fixture_checksum(kat):
    blob = open(os.path.join(GOLDEN, "fixture_2_15.bin"), "rb").read()
    assert hashlib.sha256(blob).hexdigest() == kat["fixture_sha256"]


@pytest.mark.parametrize("n", [256, 512, 1024, 2048, 4096])
def test_kat_small(n, kat, fixture_seqs):
    a, b = fixture_seqs
    case = next(c for c in kat["cases"] if c["n"] == n)
    assert O.align(O.LCS, a[:n], b[:n])["score"] == case["lcs"]
    assert O.align(O.ED, a[:n], b[:n])["score"] == case["ed"]
    assert O.align(O.SW, a[:n], b[:n])["score"] == case["sw_corner"]


def test_kat_large_multithreaded(kat, fixture_seqs):
    a, b = fixture_seqs
    for case in kat["cases"]:
        n = case["n"]
        if n < 8192:
            continue
        assert O.align(O.LCS, a[:n], b[:n], threads=8)["score"] == case["lcs"]
        assert O.align(O.ED, a[:n], b[:n], threads=8)["score"] == case["ed"]
        assert O.align(O.SW, a[:n], b[:n], threads=8)["score"] == case["sw_corner"]
    assert kat["gpu_log_pin"]["lcs"] == next(c for c in kat["cases"] if c["n"] == 32768)["lcs"]


def test_random_cases_match_reference_binaries():
    for c in load_random_cases():
        a, b = np.array(c["a"]), np.array(c["b"])
        assert O.align(O.LCS, a, b)["score"] == c["lcs"]
        assert O.align(O.ED, a, b)["score"] == c["ed"]
        assert O.align(O.SW, a, b)["score"] == c["sw_corner"]


def test_ed_boundary_quirk():
    # ED.cpp:48-54 makes row 0 [0,0,1,2,...]; the GPU_setInit border is [0,1,2,...]
    a = np.array([0, 1, 3, 1, 3, 0])
    b = np.array([3, 2, 3, 0, 2, 3])
    assert O.align(O.ED, a, b, rule=O.ED_REF_CPU)["score"] == 4
    assert O.align(O.ED, a, b, rule=O.ED_STANDARD)["score"] == 5


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_c_matches_python_restatement(kind):
    rng = np.random.default_rng(kind)
    for _ in range(60):
        n1, n2 = rng.integers(0, 14, 2)
        a = rng.integers(0, 3, n1)
        b = rng.integers(0, 3, n2)
        for rule in (0, 1):
            t = O.table(kind, a, b, rule=rule)
            assert (t == np.array(O.table_py(kind, list(a), list(b), rule=rule))).all()
            r = O.align(kind, a, b, rule=rule)
            assert r["score"] == t[-1, -1]
            assert (r["last_row"] == t[-1, :]).all()
            assert (r["last_col"] == t[:, -1]).all()
            if kind == 2:
                m = t[1:, 1:].max() if n1 and n2 else 0
                assert r["sw_max"] == max(m, 0)
                if r["sw_max"] > 0:
                    ys, xs = np.nonzero(t[1:, 1:] == r["sw_max"])
                    assert (r["sw_y"], r["sw_x"]) == (ys[0] + 1, xs[0] + 1)


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_multithreaded_equals_single(kind):
    rng = np.random.default_rng(10 + kind)
    a = rng.integers(0, 4, 2100).astype(np.int32)
    b = rng.integers(0, 4, 1700).astype(np.int32)
    s = O.align(kind, a, b)
    m = O.align(kind, a, b, threads=6, band_rows=97, chunk_cols=61)
    assert s["score"] == m["score"]
    assert (s["last_row"] == m["last_row"]).all() and (s["last_col"] == m["last_col"]).all()
    assert (s["sw_max"], s["sw_y"], s["sw_x"]) == (m["sw_max"], m["sw_y"], m["sw_x"])


def test_batch_matches_single():
    rng = np.random.default_rng(5)
    kinds, sa, sb = [], [], []
    for i in range(40):
        kinds.append(i % 3)
        sa.append(rng.integers(0, 4, rng.integers(1, 200)))
        sb.append(rng.integers(0, 4, rng.integers(1, 200)))
    r = O.align_batch(kinds, sa, sb, threads=4)
    for i in range(40):
        s = O.align(kinds[i], sa[i], sb[i])
        assert r["score"][i] == s["score"]
        if kinds[i] == 2:
            assert (r["sw_max"][i], r["sw_y"][i], r["sw_x"][i]) == (s["sw_max"], s["sw_y"], s["sw_x"])


def test_sw_max_known_cells(fixture_seqs):
    a, b = fixture_seqs
    r = O.align(O.SW, a[:256], b[:256])
    assert (r["sw_max"], r["sw_y"], r["sw_x"]) == (156, 256, 228)
    r = O.align(O.SW, a[:1024], b[:1024])
    assert (r["sw_max"], r["sw_y"], r["sw_x"]) == (733, 1019, 961)
