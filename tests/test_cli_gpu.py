"""gme-align on the reference's data files: the reference drivers' invocations and
output lines, checked against the oracle and the reference's own GPU log."""
import subprocess

import numpy as np
import pytest

from conftest import load_fixture
from oracle import oracle as O
from test_cli import _tools, reference_text

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def data_dir(tmp_path_factory):
    d = tmp_path_factory.mktemp("Data")
    a, b = load_fixture()
    for k in (15, 12, 10):  # the shipped fixtures are prefixes of the 2^15 one
        (d / f"str1_2_{k}_str2_2_{k}.txt").write_bytes(reference_text(a[:1 << k], b[:1 << k]))
    return d


def run(args, d):
    r = subprocess.run([_tools()["gme-align"], *args, "--dir", str(d)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout.splitlines()


def test_lcs_2_15_matches_reference_gpu_log(data_dir):
    # LCS/GPU_Hyperlane_Share.txt:102 prints "lcs length: 21469" for this file
    out = run(["LCS", "15", "15", "32", "128", "2"], data_dir)
    assert out[0] == "input data loaded"
    assert out[1] == "lcs length: 21469"
    assert out[2].startswith("execution time: ") and out[2].endswith(" ms.")


@pytest.mark.parametrize("kind,name", [(0, "LCS"), (1, "ED"), (2, "SW")])
def test_cpu_and_gpu_forms(data_dir, kind, name):
    a, b = load_fixture()
    a, b = a[:4096], b[:4096]
    # CPU-program form: ED.cpp's border
    out = run([name, "12", "12"], data_dir)
    want = O.align(kind, a, b, rule=O.ED_REF_CPU)["score"]
    assert out[0] == (f"lcs length: {want}" if kind == 0 else f"last: {want}")
    # GPU-driver form: GPU_setInit's border, ITR repetitions
    out = run([name, "12", "12", "32", "128", "3"], data_dir)
    want = O.align(kind, a, b, rule=O.ED_STANDARD)["score"]
    assert out[0] == "input data loaded"
    assert out[1] == (f"lcs length: {want}" if kind == 0 else f"last: {want}")


def test_generated_data_end_to_end(tmp_path):
    t = _tools()
    subprocess.run([t["gme-generate"], "9", "8", "--seed", "77", "--dir", str(tmp_path)], check=True)
    lines = open(tmp_path / "str1_2_9_str2_2_8.txt").read().split("\n")
    a = np.array(lines[1].split(), np.int32)
    b = np.array(lines[2].split(), np.int32)
    out = run(["ED", "9", "8", "--border", "gpu"], tmp_path)
    assert out[0] == f"last: {O.align(1, a, b, rule=O.ED_STANDARD)['score']}"


def test_sat_driver_matches_oracle(tmp_path):
    """gme-align SAT E1 E2 TX TY ITR on a generated file: the reference driver's output
    line, and with --out the table equal to the oracle's."""
    from test_cli import read_sat_text
    tools = _tools()
    r = subprocess.run([tools["gme-generate"], "--sat", "9", "8", "--min", "9", "--seed", "7", "--dir",
                        str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    out = tmp_path / "out.txt"
    r = subprocess.run([tools["gme-align"], "SAT", "9", "8", "16", "64", "3", "--dir", str(tmp_path),
                        "--out", str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.splitlines()
    assert len(lines) == 1 and lines[0].startswith("execution time: ") and lines[0].endswith(" ms.")
    n1, n2, t_in = read_sat_text(tmp_path / "x_2_9_y_2_8.txt")
    _, _, t_out = read_sat_text(out)
    want = O.sat(t_in.astype(np.int32), n1, n2)
    np.testing.assert_array_equal(t_out, want.astype(np.int64))
