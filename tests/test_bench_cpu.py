"""bench.py's reference arm runs on the host alone: its one JSON line carries the
contract's keys for the default, batched and summed-area-table workloads (CPU only)."""
import json
import os
import subprocess
import sys

import pytest

from conftest import REPO

KEYS = {"impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
        "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"}


@pytest.mark.parametrize("workload", ["ed65536", "batched", "sat"])
def test_reference_arm_line(workload):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--workload",
                        workload, "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, timeout=600, env=env, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert KEYS <= set(d), KEYS - set(d)
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "GCUPS"
    assert d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"]


def test_sat_cpu_baseline_helper():
    """The SAT workload's cpu_baseline leg (host only): repeated samples, all threads."""
    import importlib.util
    import numpy as np
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(REPO, "bench.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    h = np.random.default_rng(2).integers(0, 10000, (300, 1027), dtype=np.int32)
    c = b.sat_cpu_baseline(h, 1024, 298, 1027, target_s=0.2)
    assert c["value"] > 0 and c["kind"] == "port" and c["cores"] >= 1 and " x " in c["sample"]
