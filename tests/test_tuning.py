"""The autotuned batch table (CPU only): the committed header is the committed sweep's,
and a batch is planned with the entry of its own length range -- every sweep batch
selects the entry tuned on it, and the two benchmark streams select theirs."""
import json
import os

import numpy as np
import pytest

from conftest import REPO

BEST = json.load(open(os.path.join(REPO, "gpumemefficient_gb300", "tuned.json")))["best"]
KEYS = ("warps_per_block", "blocks_per_sm", "block_min_cells", "team_min_cells", "team_split", "rows_per_lane",
        "packed16")
DEFAULTS = {"team_split": 2, "rows_per_lane": 4, "packed16": 0}


def _pairs(la, lb):
    import gpumemefficient_gb300 as g
    p = np.zeros(len(la), g.PAIR_DTYPE)
    p["n1"] = la
    p["n2"] = lb
    return p


def _selected(la, lb):
    import __graft_entry__ as ge
    ge.build_library()
    import gpumemefficient_gb300 as g
    c = g.batch_tuned_config(_pairs(la, lb))
    return {k: c[k] for k in KEYS}


def _entry(name):
    return {k: BEST[name].get(k, DEFAULTS.get(k)) for k in KEYS}


def test_header_is_the_committed_sweep(tmp_path):
    from gpumemefficient_gb300 import tune
    out = tmp_path / "gme_tuned.h"
    tune.gen_header(BEST, path=str(out))
    assert out.read_text() == open(tune.TUNED_H).read()


@pytest.mark.parametrize("bucket", range(6))
def test_sweep_batches_select_their_entry(bucket):
    from gpumemefficient_gb300 import tune
    name, lo, hi = (tune.BUCKETS + tune.MIXES)[bucket]
    la, lb = tune.lengths_for(lo, hi, 1.5e10, np.random.default_rng(0x5EED + bucket))
    assert _selected(la, lb) == _entry(name)


def test_benchmark_streams_select_their_entries():
    from gpumemefficient_gb300 import synth
    _, sa, sb = synth.batch_pairs()
    la = np.array([len(x) for x in sa])
    lb = np.array([len(x) for x in sb])
    assert _selected(la, lb) == _entry("mixed_64_4096")
    _, pairs = synth.served_requests()
    assert _selected(pairs["n1"], pairs["n2"]) == _entry("mixed_32_16384")
