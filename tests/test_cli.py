"""The data-file tools without a GPU: gme-generate's layout and seeding, the reference
text layout reproduced byte for byte, and gme-align failing loudly (CPU only)."""
import hashlib
import os
import subprocess

import numpy as np

from conftest import load_fixture, load_kat


def _tools():
    from gpumemefficient_gb300 import _build
    import __graft_entry__ as ge
    ge.build_library()
    return _build.build_tools()


def reference_text(a, b) -> bytes:
    """The reference's data-file layout (EditDistance/generator.cpp:50-66)."""
    return (f"{len(a)} {len(b)}\n" + "".join(f"{x} " for x in a) + "\n" +
            "".join(f"{x} " for x in b) + "\n").encode()


def read_text(path):
    lines = open(path).read().split("\n")
    n1, n2 = map(int, lines[0].split())
    a = np.array(lines[1].split(), np.int32)
    b = np.array(lines[2].split(), np.int32)
    assert len(a) == n1 and len(b) == n2
    return a, b


def test_fixture_text_layout():
    """The packed fixture, written in the reference layout, is the shipped file."""
    a, b = load_fixture()
    assert hashlib.sha256(reference_text(a, b)).hexdigest() == load_kat()["fixture_text_sha256"]


def test_generate_layout_prefixes_and_seed(tmp_path):
    gen = _tools()["gme-generate"]
    d1, d2, d3 = (tmp_path / x for x in ("s5", "s5b", "s6"))
    for d, seed in ((d1, 5), (d2, 5), (d3, 6)):
        d.mkdir()
        subprocess.run([gen, "11", "10", "--seed", str(seed), "--dir", str(d)], check=True)
    names = sorted(os.listdir(d1))
    assert names == ["str1_2_10_str2_2_9.txt", "str1_2_11_str2_2_10.txt", "str1_2_8_str2_2_7.txt",
                     "str1_2_9_str2_2_8.txt"]
    a11, b10 = read_text(d1 / "str1_2_11_str2_2_10.txt")
    assert len(a11) == 2048 and len(b10) == 1024 and set(np.unique(a11)) <= {0, 1, 2, 3}
    for e in (10, 9, 8):  # every smaller file holds prefixes of the same sequences
        a, b = read_text(d1 / f"str1_2_{e}_str2_2_{e - 1}.txt")
        assert (a == a11[:len(a)]).all() and (b == b10[:len(b)]).all()
    for n in names:  # the layout byte for byte, and the seed decides the contents
        raw = open(d1 / n, "rb").read()
        assert raw == reference_text(*read_text(d1 / n))
        assert raw == open(d2 / n, "rb").read()
        assert raw != open(d3 / n, "rb").read()


def test_align_cli_errors_without_data(tmp_path):
    exe = _tools()["gme-align"]
    r = subprocess.run([exe, "ED", "12", "12", "--dir", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 1 and "Input file cannot be opened" in r.stdout
    r = subprocess.run([exe, "XX", "12", "12"], capture_output=True, text=True)
    assert r.returncode == 1
    r = subprocess.run([exe, "ED", "12"], capture_output=True, text=True)
    assert r.returncode == 1 and "Incorrect Input Parameters" in r.stdout


def read_sat_text(path):
    lines = open(path).read().split("\n")
    n1, n2 = map(int, lines[0].split())
    rows = [np.array(l.split(), np.int64) for l in lines[1:1 + n2 + 3]]
    assert all(len(r) == n1 + 3 for r in rows) and lines[1].endswith(" ")
    return n1, n2, np.stack(rows)


def test_generate_sat_layout_and_seed(tmp_path):
    """gme-generate --sat: the layout of SAT/generator.cpp (header, n2 + 3 rows of n1 + 3
    values in 0..9999); smaller files hold the first values of the same array."""
    gen = _tools()["gme-generate"]
    for d in ("a", "b"):
        (tmp_path / d).mkdir()
        r = subprocess.run([gen, "--sat", "8", "7", "--min", "6", "--seed", "5", "--dir", str(tmp_path / d)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stdout
    names = sorted(p.name for p in (tmp_path / "a").iterdir())
    assert names == ["x_2_6_y_2_5.txt", "x_2_7_y_2_6.txt", "x_2_8_y_2_7.txt"]
    for nm in names:
        assert (tmp_path / "a" / nm).read_bytes() == (tmp_path / "b" / nm).read_bytes()
    n1, n2, big = read_sat_text(tmp_path / "a" / "x_2_8_y_2_7.txt")
    assert (n1, n2) == (256, 128) and big.min() >= 0 and big.max() <= 9999
    s1, s2, small = read_sat_text(tmp_path / "a" / "x_2_7_y_2_6.txt")
    flat = big.reshape(-1)
    np.testing.assert_array_equal(small.reshape(-1), flat[:(s1 + 3) * (s2 + 3)])


def test_align_sat_missing_file_fails(tmp_path):
    r = subprocess.run([_tools()["gme-align"], "SAT", "9", "9", "32", "128", "1", "--dir", str(tmp_path)],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "cannot be opened" in r.stdout
