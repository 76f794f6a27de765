import json
import os
import struct
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def load_fixture():
    """The reference's square fixture LCS/Data/str1_2_15_str2_2_15.txt (2-bit packed)."""
    blob = open(os.path.join(GOLDEN, "fixture_2_15.bin"), "rb").read()
    magic, n1, n2 = struct.unpack("<4sII", blob[:12])
    assert magic == b"GME2"

    def unpack(buf, n):
        x = np.frombuffer(buf, np.uint8)
        return np.stack([x & 3, (x >> 2) & 3, (x >> 4) & 3, (x >> 6) & 3], 1).reshape(-1)[:n].astype(np.int32)

    a = unpack(blob[12:12 + (n1 + 3) // 4], n1)
    b = unpack(blob[12 + (n1 + 3) // 4:], n2)
    return a, b


def load_kat():
    return json.load(open(os.path.join(GOLDEN, "kat.json")))


def load_random_cases():
    return json.load(open(os.path.join(GOLDEN, "random_cases.json")))["cases"]


@pytest.fixture(scope="session")
def fixture_seqs():
    return load_fixture()


@pytest.fixture(scope="session")
def kat():
    return load_kat()


@pytest.fixture(scope="session")
def gme_ctx():
    import gpumemefficient_gb300 as g
    ctx = g.Context(0)
    yield ctx
    ctx.close()
