"""Times the reference's own CPU programs (LCS.cpp, ED.cpp, SW.cpp, unmodified, g++ -O2,
built by oracle/build_ref.sh into oracle/_ref/) on the reference's square fixture
(LCS/Data/str1_2_15_str2_2_15.txt, kept 2-bit packed in tests/golden/fixture_2_15.bin)
and on its square prefixes.

Measurement infrastructure only: it runs the checker's binaries, never the product.
The programs are single-threaded and take the fixture from ./Data/ of the directory
they run in; each prints its own timing of the DP alone in milliseconds ("execution
time: X ms."; SW.cpp prints the same figure labelled "second"), which is what is
reported, with GCUPS = n1 * n2 / X.

    python oracle/time_ref.py [--sizes 13 14 15] [--reps 1]

Prints one JSON line per program and size.  Needs the binaries (they run on the
machine that built them).
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import re
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
FIXTURE = os.path.join(REPO, "tests", "golden", "fixture_2_15.bin")


def fixture():
    blob = open(FIXTURE, "rb").read()
    magic, n1, n2 = struct.unpack("<4sII", blob[:12])
    assert magic == b"GME2"

    def unpack(buf, n):
        x = np.frombuffer(buf, np.uint8)
        return np.stack([x & 3, (x >> 2) & 3, (x >> 4) & 3, (x >> 6) & 3], 1).reshape(-1)[:n]

    return unpack(blob[12:12 + (n1 + 3) // 4], n1), unpack(blob[12 + (n1 + 3) // 4:], n2)


def data_text(a, b) -> str:
    """The reference's data-file layout (EditDistance/generator.cpp:50-66)."""
    return f"{len(a)} {len(b)}\n" + "".join(f"{x} " for x in a) + "\n" + "".join(f"{x} " for x in b) + "\n"


def cpu_name() -> str:
    try:
        for line in open("/proc/cpuinfo"):
            if line.startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--sizes", type=int, nargs="+", default=[13, 14, 15])
    p.add_argument("--reps", type=int, default=1)
    p.add_argument("--programs", nargs="+", default=["LCS", "ED", "SW"])
    args = p.parse_args()
    a, b = fixture()
    with tempfile.TemporaryDirectory() as tmp:
        os.mkdir(os.path.join(tmp, "Data"))
        for e in args.sizes:
            n = 1 << e
            with open(os.path.join(tmp, "Data", f"str1_2_{e}_str2_2_{e}.txt"), "w") as f:
                f.write(data_text(a[:n], b[:n]))
        for prog in args.programs:
            exe = os.path.join(HERE, "_ref", prog)
            if not os.path.exists(exe):
                print(json.dumps({"program": prog, "unavailable": "oracle/_ref not built (oracle/build_ref.sh)"}))
                continue
            for e in args.sizes:
                n = 1 << e
                best, last = None, None
                for _ in range(args.reps):
                    out = subprocess.run([exe, str(e), str(e)], cwd=tmp, capture_output=True, text=True,
                                         check=True).stdout
                    # milliseconds in all three (SW.cpp labels the same figure "second")
                    ms = float(re.search(r"execution time: ([0-9.eE+-]+) (?:ms|second)", out).group(1))
                    m = re.search(r"(?:last|lcs length): (-?\d+)", out)
                    last = int(m.group(1)) if m else None
                    best = ms if best is None else min(best, ms)
                print(json.dumps({"program": prog, "n": n, "ms": best, "gcups": n * n / best / 1e6,
                                  "last": last, "threads": 1, "cpu": cpu_name(),
                                  "build": "g++ -O2, unmodified source"}), flush=True)


if __name__ == "__main__":
    main()
