"""Regenerates the golden fixtures in this directory from the reference checkout.

Run where the read-only reference checkout exists, never on the GPU host:
    oracle/build_ref.sh [REFERENCE_ROOT] && python tests/golden/make_golden.py [REFERENCE_ROOT]
The checkout is REFERENCE_ROOT, else $GME_REFERENCE_ROOT, else a directory named
`reference` beside this repository's own directory.

Outputs
  fixture_2_15.bin  the reference's square fixture LCS/Data/str1_2_15_str2_2_15.txt
                    (alphabet {0,1,2,3}) packed 2 bits per symbol.  Every smaller
                    square fixture str1_2_k_str2_2_k.txt (k = 8..15) is a prefix of it
                    in both sequences; the script checks that before writing.
  random_cases.json small seeded random square pairs (n = 1..96, alphabets 2, 4
                    and 20) with the answers the same unmodified reference programs
                    print for them; these pin the ED.cpp boundary quirk (row 0 =
                    [0,0,1,2,...]) that the 2^k fixtures do not exercise.
  kat.json          known answers printed by the UNMODIFIED reference CPU programs
                    (LCS/LCS.cpp, EditDistance/ED.cpp, SmithWaterman/SW.cpp, built by
                    oracle/build_ref.sh) on those fixtures, plus the GPU-log pin
                    LCS/GPU_Hyperlane_Share.txt:102 ("lcs length: 21469").
"""
import hashlib
import json
import os
import re
import struct
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def reference_root():
    """The reference checkout: the first argument, $GME_REFERENCE_ROOT, or the
    directory `reference` beside this repository."""
    for cand in (sys.argv[1] if len(sys.argv) > 1 else None, os.environ.get("GME_REFERENCE_ROOT"),
                 os.path.join(os.path.dirname(REPO), "reference")):
        if cand and os.path.isfile(os.path.join(cand, "LCS", "LCS.cpp")):
            return cand
    sys.exit("make_golden: no reference checkout (pass its root or set GME_REFERENCE_ROOT)")


REF = reference_root()
DATA = os.path.join(REF, "LCS", "Data")
REFBIN = os.path.join(REPO, "oracle", "_ref")


def read_fixture(path):
    lines = open(path).read().split("\n")
    n1, n2 = map(int, lines[0].split()[:2])
    a = np.array(lines[1].split(), dtype=np.int32)
    b = np.array(lines[2].split(), dtype=np.int32)
    assert len(a) == n1 and len(b) == n2, path
    return a, b


def pack2(x):
    x = np.asarray(x, np.uint8)
    assert x.max() < 4
    pad = (-len(x)) % 4
    x = np.concatenate([x, np.zeros(pad, np.uint8)]).reshape(-1, 4)
    return (x[:, 0] | (x[:, 1] << 2) | (x[:, 2] << 4) | (x[:, 3] << 6)).astype(np.uint8)


def run_ref(prog, k):
    out = subprocess.run([os.path.join(REFBIN, prog), str(k), str(k)], cwd=os.path.join(REF, "LCS"),
                         capture_output=True, text=True, check=True, timeout=600).stdout
    m = re.search(r"(?:lcs length|last):\s*(-?\d+)", out)
    return int(m.group(1))


def run_ref_dir(prog, workdir, case_id):
    out = subprocess.run([os.path.join(REFBIN, prog), str(case_id), str(case_id)], cwd=workdir,
                         capture_output=True, text=True, check=True, timeout=60).stdout
    return int(re.search(r"(?:lcs length|last):\s*(-?\d+)", out).group(1))


def random_cases():
    import tempfile
    rng = np.random.default_rng(20181021)
    cases = []
    with tempfile.TemporaryDirectory() as td:
        os.makedirs(os.path.join(td, "Data"))
        for cid in range(1, 121):
            n = int(rng.integers(1, 97)) if cid > 12 else cid
            alpha = int(rng.choice([2, 4, 20]))
            a = rng.integers(0, alpha, n).astype(np.int32)
            b = rng.integers(0, alpha, n).astype(np.int32)
            if cid % 17 == 0:
                b = a.copy()                      # all matches
            if cid % 19 == 0:
                a[:] = 0; b[:] = 1                # no matches
            with open(os.path.join(td, "Data", f"str1_2_{cid}_str2_2_{cid}.txt"), "w") as f:
                f.write(f"{n} {n}\n" + " ".join(map(str, a)) + " \n" + " ".join(map(str, b)) + " \n")
            cases.append({"a": a.tolist(), "b": b.tolist(),
                          "lcs": run_ref_dir("LCS", td, cid), "ed": run_ref_dir("ED", td, cid),
                          "sw_corner": run_ref_dir("SW", td, cid)})
    with open(os.path.join(HERE, "random_cases.json"), "w") as f:
        json.dump({"source": "reference CPU programs, unmodified, on seeded random square pairs",
                   "seed": 20181021, "cases": cases}, f)


def main():
    random_cases()
    A, B = read_fixture(os.path.join(DATA, "str1_2_15_str2_2_15.txt"))
    for k in range(8, 16):
        a, b = read_fixture(os.path.join(DATA, f"str1_2_{k}_str2_2_{k}.txt"))
        assert np.array_equal(A[: len(a)], a) and np.array_equal(B[: len(b)], b), k
    blob = struct.pack("<4sII", b"GME2", len(A), len(B)) + pack2(A).tobytes() + pack2(B).tobytes()
    with open(os.path.join(HERE, "fixture_2_15.bin"), "wb") as f:
        f.write(blob)
    kat = {"source": "reference CPU programs LCS.cpp / ED.cpp / SW.cpp, unmodified, g++ -O2",
           "fixture": "fixture_2_15.bin (prefixes of length n of both sequences)",
           "fixture_sha256": hashlib.sha256(blob).hexdigest(),
           "fixture_text_sha256": hashlib.sha256(open(os.path.join(DATA, "str1_2_15_str2_2_15.txt"), "rb").read()).hexdigest(),
           "fixture_text": "sha256 of LCS/Data/str1_2_15_str2_2_15.txt as shipped (the text layout the data-file tools read and write)",
           "gpu_log_pin": {"n": 32768, "lcs": 21469, "source": "LCS/GPU_Hyperlane_Share.txt:102"},
           "cases": []}
    for k in range(8, 16):
        row = {"n": 2 ** k, "lcs": run_ref("LCS", k), "ed": run_ref("ED", k), "sw_corner": run_ref("SW", k)}
        print(row, flush=True)
        kat["cases"].append(row)
    with open(os.path.join(HERE, "kat.json"), "w") as f:
        json.dump(kat, f, indent=1)


if __name__ == "__main__":
    main()
