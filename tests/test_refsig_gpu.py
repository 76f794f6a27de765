"""Every one of the reference's host-function signatures (include/gme_reference.h),
called the way the reference drivers call them, through libgme.so on the GPU: the eight
LCS/ED/SW overloads (paddX = 3, paddY = 1, a caller-owned table, tX = 32, tY = 128, as in
EditDistance/GPU_Hyperlane_Share.cpp:86-108) and SOR on a summed-area-table data file
(SAT/GPU_Hyperlane_Share.cpp), each checked against the oracle."""
import os
import subprocess

import numpy as np
import pytest

from conftest import load_fixture
from oracle import oracle as O
from test_cli import _tools, reference_text

pytestmark = pytest.mark.gpu


def refcheck(seqfile, satfile=None):
    exe = _tools()["gme-refcheck"]
    r = subprocess.run([exe, str(seqfile)] + ([str(satfile)] if satfile else []), capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = {}
    for line in r.stdout.splitlines():
        k, *v = line.split()
        out[k] = [int(x) for x in v]
    return out


def expected(a, b):
    lcs = O.align(O.LCS, a, b)["score"]
    ed = O.align(O.ED, a, b, rule=O.ED_STANDARD)["score"]  # the reference GPU code's border
    sw = O.align(O.SW, a, b)["score"]  # the corner cell, as the reference returns
    return {"LCS/7": lcs, "LCS/4": lcs, "ED/9": ed, "ED/7": ed, "ED/4": ed, "SW/9": sw, "SW/7": sw, "SW/4": sw}


def write_sat(path, t, n1, n2):
    with open(path, "w") as f:
        f.write(f"{n1} {n2}\n")
        for row in t:
            f.write("".join(f"{v} " for v in row) + "\n")


@pytest.mark.parametrize("shape", [(1000, 731), (4096, 4096)])
def test_all_reference_signatures(tmp_path, shape):
    n1, n2 = shape
    if n1 == n2 == 4096:
        a, b = load_fixture()
        a, b = a[:n1], b[:n2]  # a prefix of the reference's own 2^15 fixture
    else:
        rng = np.random.default_rng(n1 + n2)
        a = rng.integers(0, 4, n1).astype(np.int32)
        b = rng.integers(0, 4, n2).astype(np.int32)
    seq = tmp_path / "seq.txt"
    seq.write_bytes(reference_text(a, b))
    s1, s2 = 300, 211
    t = np.random.default_rng(5).integers(0, 10000, (s2 + 3, s1 + 3)).astype(np.int32)
    sat = tmp_path / "sat.txt"
    write_sat(sat, t, s1, s2)
    got = refcheck(seq, sat)
    want = expected(a, b)
    for k, v in want.items():
        assert got[k] == [v], k
    w = O.sat(t, s1, s2)
    total = int(w[1:s2 + 1, 1:s1 + 1].astype(np.uint32).sum(dtype=np.uint64) % (1 << 32))
    assert got["SOR/5"] == [total, int(w[s2, s1])]
    assert got["SOR/3"] == [total, int(w[s2, s1])]
