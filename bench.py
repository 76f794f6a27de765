#!/usr/bin/env python3
"""Benchmark: GCUPS of the GB300 wavefront DP on one GPU (replicas across GPUs).

Default workload: edit distance, one pair of 65536 x 65536 (4.3e9 cells), second
sequence derived from the first by 10% seeded edits, plain path (one persistent
kernel per alignment), int32 scores, score-only with O(n) boundary memory.

Prints ONE JSON line (rank 0).  `value` is device-timed throughput with inputs
resident in HBM; `e2e` is the same metric through the C ABI with host buffers
(host->device copies and the device->host result read inside the timed region).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gme|reference]
                  [--workload ed65536|lcs8192|sw32768|lcs32768|batched|served|path|sat|baselines]

The batched workload is 16384 pairs, each length log-uniform in [64, 4096], kinds
LCS/ED/SW one third each, all in one planned launch replayed as a CUDA graph.  The
served workload submits a request stream to the server; sat is the reference's
summed-area table; baselines times the plain path beside the reference's
table-based strategies rebuilt on this GPU.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

# algorithmic integer operations per cell of the reference recurrences as written
# (LCS.cpp:59-63: compare, select, add, max; ED.cpp:63-65: 3 adds, 2 mins, compare,
# select; SW.cpp:45-47,63-65: 2 subtracts, compare+select, add, 3 maxes)
OPS_PER_CELL = {0: 4, 1: 7, 2: 8}
KIND_NAME = {0: "LCS", 1: "ED", 2: "SW"}
INT_LANES_PER_SM = 128
METRIC = "GCUPS on 1 GB300, batched/served vs plain per-pair (bit-exact); p50/p99 latency"
L2_FLUSH_BYTES = 256 << 20


def profiled_traffic(name: str):
    """DRAM bytes per launch of the dominant kernel, from the committed ncu summary
    (`dram_bytes_per_launch: N` in profiles/<name>.md), or None."""
    import re
    try:
        txt = open(os.path.join(REPO, "profiles", name + ".md")).read()
    except OSError:
        return None
    m = re.search(r"dram_bytes_per_launch:\s*(\d+)", txt)
    return int(m.group(1)) if m else None


def workload(name: str):
    from gpumemefficient_gb300 import synth
    if name == "ed65536":
        a, b = synth.ed_pair(65536)
        return 1, a, b, {"workload": "edit distance, one pair 65536x65536, 10% seeded edits, plain path",
                         "n1": 65536, "n2": 65536, "alphabet": 4, "edit_rate": 0.1,
                         "seed": synth.SEED_ED, "ed_boundary": "ED.cpp (REF_CPU)"}
    if name == "lcs8192":
        a, b = synth.lcs_pair(8192)
        return 0, a, b, {"workload": "LCS, one pair 8192x8192, plain path", "n1": 8192, "n2": 8192,
                         "alphabet": 4, "seed": synth.SEED_LCS}
    if name == "lcs32768":
        a, b = synth.lcs_pair(32768)
        return 0, a, b, {"workload": "LCS, one pair 32768x32768, plain path", "n1": 32768,
                         "n2": 32768, "alphabet": 4, "seed": synth.SEED_LCS}
    if name == "sw32768":
        a, b = synth.sw_pair(32768)
        return 2, a, b, {"workload": "Smith-Waterman, one pair 32768x32768, planted 2048 segment "
                                     "mutated 15%, max score and cell", "n1": 32768, "n2": 32768,
                         "alphabet": 20, "seed": synth.SEED_SW}
    raise SystemExit(f"unknown workload {name}")


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int, interval_ms: int = 50):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                       f"-lms", str(interval_ms), "-i", str(device)],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for r in csv.reader(fh):
                if len(r) >= 9:
                    rows.append([x.strip() for x in r])
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows if r[3].replace(".", "").isdigit()), default=None)}


def cpu_baseline(kind: int, a, b, target_s: float = 2.0, max_rows: int = None):
    """The oracle port on all host threads over a bounded sample: the full first
    sequence against a prefix of the second, grown until the run takes target_s."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    rows = 1024
    limit = max_rows or len(b)
    while True:
        t0 = time.perf_counter()
        O.align(kind, a, b[:rows], threads=threads, band_rows=64, chunk_cols=2048)
        dt = time.perf_counter() - t0
        if dt >= target_s or rows >= limit:
            break
        rows = min(limit, rows * 2 if dt < target_s / 4 else int(rows * target_s / dt) + 1)
    cells = len(a) * rows
    return {"value": cells / dt / 1e9, "unit": "GCUPS", "cores": threads, "kind": "port",
            "sample": f"{KIND_NAME[kind]} {len(a)} columns x {rows} rows ({cells:.3g} cells), "
                      f"oracle/oracle.c blocked wavefront on {threads} threads, {dt:.2f} s"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(args):
    """Reference arm: the reference's CPU recurrence (oracle port; the reference sources are
    not on this host) on all host threads, same metric and workload, bounded samples."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    if args.workload == "batched":
        return run_reference_batch(args, ws)
    if args.workload == "sat":
        return run_reference_sat(args, ws)
    kind, a, b, cfg = workload(args.workload)
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    rows = min(len(b), 4096 if len(a) >= 32768 else len(b))
    for _ in range(args.warmup):
        O.align(kind, a, b[:rows], threads=threads, band_rows=64, chunk_cols=2048)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.align(kind, a, b[:rows], threads=threads, band_rows=64, chunk_cols=2048)
        times.append(time.perf_counter() - t0)
    cells = len(a) * rows
    tot = sum(times)
    val = cells * len(times) / tot / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "GCUPS",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tot / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded)", "config": cfg,
            "cpu_baseline": {"value": val, "unit": "GCUPS", "cores": threads, "kind": "port",
                             "sample": f"{KIND_NAME[kind]} {len(a)} columns x {rows} rows per step "
                                       f"({cells:.3g} cells), oracle/oracle.c on {threads} threads"},
            "e2e": {"value": val, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference_sat(args, ws):
    """Reference arm, SAT workload: the recurrence on the CPU (oracle port: row prefix sums,
    then column sums, on all host threads) over a bounded band of rows per step."""
    from oracle import oracle as O
    n1 = args.sat_n
    ld = n1 + 3
    k = min(args.sat_n, 4096)
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(0x5A7)
    host = rng.integers(0, 10000, (k + 1, ld), dtype=np.int32)
    for _ in range(args.warmup):
        O.lib().orc_sat_mt(O._p32(host), n1, k, ld, threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.lib().orc_sat_mt(O._p32(host), n1, k, ld, threads)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    val = n1 * k * len(times) / tot / 1e9
    cfg = {"workload": f"summed-area table, {n1} x {n1} interior in the reference's layout, in place",
           "n1": n1, "n2": n1, "ld": ld, "seed": 0x5A7}
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "GCUPS",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32 (wrapping)",
            "data": "synthetic (seeded)", "config": cfg,
            "cpu_baseline": {"value": val, "unit": "GCUPS", "cores": threads, "kind": "port",
                             "sample": f"rows 1..{k} of the table per step ({n1 * k:.3g} cells), "
                                       f"oracle/oracle.c row prefixes then column sums on {threads} threads"},
            "e2e": {"value": val, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference_batch(args, ws):
    """Reference arm, batched workload: the CPU recurrence over a bounded sample of the pairs."""
    from gpumemefficient_gb300 import synth
    from oracle import oracle as O
    kinds, sa, sb = synth.batch_pairs(args.pairs)
    threads = os.cpu_count() or 1
    k = min(len(kinds), 1500)
    cells = float(sum(len(a) * len(b) for a, b in zip(sa[:k], sb[:k])))
    for _ in range(args.warmup):
        O.align_batch(kinds[:k], sa[:k], sb[:k], threads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.align_batch(kinds[:k], sa[:k], sb[:k], threads=threads)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    val = cells * len(times) / tot / 1e9
    cfg = {"workload": f"batched: {len(kinds)} pairs, lengths log-uniform [64, 4096], alphabet 4, "
                       "LCS/ED/SW 1/3 each", "pairs": len(kinds), "seed": synth.SEED_BATCH}
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "GCUPS",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded)", "config": cfg,
            "cpu_baseline": {"value": val, "unit": "GCUPS", "cores": threads, "kind": "port",
                             "sample": f"first {k} pairs per step ({cells:.3g} cells), oracle/oracle.c "
                                       f"pairs across {threads} threads"},
            "e2e": {"value": val, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gme(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    import __graft_entry__ as ge
    ge.build()
    import gpumemefficient_gb300 as g
    from oracle import oracle as O

    kind, a, b, cfg = workload(args.workload)
    n1, n2 = len(a), len(b)
    cells = n1 * n2
    ctx = g.Context(local)
    stream = torch.cuda.Stream(device=local)
    sc = g.scoring()
    with torch.cuda.stream(stream):
        d_a = torch.from_numpy(a).to(f"cuda:{local}")
        d_b = torch.from_numpy(b).to(f"cuda:{local}")
        d_out = torch.zeros(32, dtype=torch.uint8, device=f"cuda:{local}")
        flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{local}")
    sp = stream.cuda_stream

    def step():
        ctx.align_device(kind, d_a.data_ptr(), n1, d_b.data_ptr(), n2, d_out.data_ptr(), sc=sc,
                         stream=sp)

    # parity of this exact workload with the oracle (outside the timed region)
    step()
    stream.synchronize()
    res = g.Result.from_buffer_copy(bytes(d_out.cpu().numpy()))
    o = O.align(kind, a, b, threads=os.cpu_count() or 1, band_rows=64, chunk_cols=2048)
    parity = (res.status == 0 and res.score == o["score"] and
              (kind != 2 or (res.sw_max, res.sw_max_y, res.sw_max_x) == (o["sw_max"], o["sw_y"], o["sw_x"])))

    for _ in range(args.warmup):
        step()
    stream.synchronize()

    clocks = ClockSampler(local)
    time.sleep(0.15)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches0 = ctx.launches
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.zero_()            # L2 flush between timed steps (outside the events)
            starts[i].record(stream)
            step()
            ends[i].record(stream)
    torch.cuda.synchronize()
    launches = ctx.launches - launches0
    clk = clocks.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    from gpumemefficient_gb300.replicas import aggregate
    t_dev, job_cells = aggregate(sum(step_ms) / 1e3, cells * args.steps, device=f"cuda:{local}")
    value = job_cells / t_dev / 1e9

    # end to end through the C ABI with pinned host buffers
    ha = torch.from_numpy(a).pin_memory().numpy()
    hb = torch.from_numpy(b).pin_memory().numpy()
    e2e_steps = max(3, min(args.steps, 50))
    for _ in range(2):
        ctx.align(kind, ha, hb, sc=sc)
    if ws > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        r = ctx.align(kind, ha, hb, sc=sc)
    t_e2e, e2e_cells = aggregate(time.perf_counter() - t0, cells * e2e_steps, device=f"cuda:{local}")
    e2e = {"value": e2e_cells / t_e2e / 1e9, "unit": "GCUPS",
           "h2d_bytes_per_step": int(a.nbytes + b.nbytes), "d2h_bytes_per_step": 32,
           "steps": e2e_steps, "score_ok": r.score == o["score"]}

    # roofline: integer ALU (the recurrence is min/max/add/select on int32)
    props = torch.cuda.get_device_properties(local)
    sms = props.multi_processor_count
    mhz = clk.get("sm_mhz") or 1920.0
    peak_tops = sms * INT_LANES_PER_SM * mhz * 1e6 / 1e12
    mean_s = t_dev / args.steps
    achieved = cells * OPS_PER_CELL[kind] / mean_s / 1e12
    roof = {"bound": "int_alu", "achieved": achieved, "peak": peak_tops, "unit": "Tops/s",
            "frac": achieved / peak_tops,
            "traffic": profiled_traffic("plain_kernel_ed65536") if args.workload == "ed65536" else None,
            "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum of one launch, ncu capture in "
                            "profiles/plain_kernel_ed65536.md",
            "peak_basis": f"{sms} SMs x {INT_LANES_PER_SM} INT32 lanes x median SM clock "
                          f"{mhz:.0f} MHz under load ({'measured' if clk.get('sm_mhz') else 'assumed'}); "
                          "MEASURED_PEAKS.json has no integer figure",
            "ops_per_cell": OPS_PER_CELL[kind], "kernel": "plain_kernel (whole step timed)"}

    cpu = cpu_baseline(kind, a, b) if (rank == 0 and not args.no_cpu) else None
    cfg = dict(cfg)
    cfg.update({"l2": "flushed between timed steps (256 MiB write)", "plain_config": ctx.plain_config(n1, n2),
                "parity_vs_oracle": "ok" if parity else "MISMATCH", "score": int(res.score)})
    if kind == 2:
        cfg["sw_max"] = {"value": int(res.sw_max), "y": int(res.sw_max_y), "x": int(res.sw_max_x)}
    line = {"metric": METRIC, "value": value, "unit": "GCUPS", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * mean_s,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded)", "config": cfg, "clocks": clk, "e2e": e2e,
            "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu,
            "step_ms": {"min": min(step_ms), "median": statistics.median(step_ms), "max": max(step_ms)}}
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return line if rank == 0 else None


def run_gme_batch(args):
    """16384 uneven mixed pairs in one planned launch (CUDA-graph replay)."""
    import ctypes
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    import __graft_entry__ as ge
    ge.build()
    import gpumemefficient_gb300 as g
    from gpumemefficient_gb300 import synth
    from oracle import oracle as O

    kinds, sa, sb = synth.batch_pairs(args.pairs)
    symbols, pairs = g.pack_batch(kinds, sa, sb)
    n = len(pairs)
    cells_k = np.array([len(a) * len(b) for a, b in zip(sa, sb)], np.float64)
    cells = float(cells_k.sum())
    ops = float(sum(cells_k[np.asarray(kinds) == k].sum() * OPS_PER_CELL[k] for k in range(3)))
    ctx = g.Context(local)
    if args.batch_warps or args.int32:
        ctx.set_batch_config(warps_per_block=args.batch_warps, packed16=-1 if args.int32 else 0)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=local)
    sp = stream.cuda_stream
    with torch.cuda.stream(stream):
        d_sym = torch.from_numpy(symbols).to(dev)
        d_res = torch.zeros(n * g.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
        flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream.synchronize()
    plan = g.BatchPlan(ctx, pairs, len(symbols))
    split = ctx.batch_stats()

    # parity of every pair with the oracle (outside the timed region)
    plan.run(d_sym.data_ptr(), d_res.data_ptr(), stream=sp)
    stream.synchronize()
    res = np.frombuffer(d_res.cpu().numpy().tobytes(), g.RESULT_DTYPE)
    o = O.align_batch(kinds, sa, sb, threads=os.cpu_count() or 1)
    sw = np.asarray(kinds) == 2
    parity = bool((res["status"] == 0).all() and (res["score"] == o["score"]).all() and
                  (res["sw_max"][sw] == o["sw_max"][sw]).all() and (res["sw_max_y"][sw] == o["sw_y"][sw]).all()
                  and (res["sw_max_x"][sw] == o["sw_x"][sw]).all())

    for _ in range(args.warmup):
        plan.run(d_sym.data_ptr(), d_res.data_ptr(), stream=sp, use_graph=True)
    stream.synchronize()
    clocks = ClockSampler(local)
    time.sleep(0.15)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches0 = ctx.launches
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            plan.run(d_sym.data_ptr(), d_res.data_ptr(), stream=sp, use_graph=True)
            ends[i].record(stream)
    torch.cuda.synchronize()
    launches = ctx.launches - launches0
    clk = clocks.stop()
    step_ms = [s_.elapsed_time(e_) for s_, e_ in zip(starts, ends)]
    from gpumemefficient_gb300.replicas import aggregate
    t_dev, job_cells = aggregate(sum(step_ms) / 1e3, cells * args.steps, device=dev)
    value = job_cells / t_dev / 1e9
    mean_s = t_dev / args.steps

    # end to end through the C ABI: pinned host symbols in, results out, plan made per call
    hsym = torch.from_numpy(symbols).pin_memory().numpy()
    hres = np.zeros(n, g.RESULT_DTYPE)
    sc = g.scoring()
    L = g.lib()
    e2e_steps = max(3, min(args.steps, 10))
    for _ in range(2):
        L.gme_align_batch(ctx.handle, hsym.ctypes.data, len(hsym), pairs.ctypes.data, n, ctypes.byref(sc),
                          hres.ctypes.data)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        st_ = L.gme_align_batch(ctx.handle, hsym.ctypes.data, len(hsym), pairs.ctypes.data, n,
                                ctypes.byref(sc), hres.ctypes.data)
    t_e2e = time.perf_counter() - t0
    e2e = {"value": ws * cells * e2e_steps / t_e2e / 1e9, "unit": "GCUPS",
           "h2d_bytes_per_step": int(hsym.nbytes + pairs.nbytes), "d2h_bytes_per_step": int(hres.nbytes),
           "steps": e2e_steps, "scores_ok": bool(st_ == 0 and (hres["score"] == o["score"]).all())}

    # the plain per-pair path on a spread subset of the same pairs
    sub = np.arange(0, n, max(1, n // args.plain_sample))
    d_one = torch.zeros(32, dtype=torch.uint8, device=dev)
    offs = pairs[sub]
    for _ in range(2):
        for i in sub[:8]:
            ctx.align_device(int(kinds[i]), d_sym.data_ptr() + 4 * int(pairs[i]["a_off"]), int(pairs[i]["n1"]),
                             d_sym.data_ptr() + 4 * int(pairs[i]["b_off"]), int(pairs[i]["n2"]), d_one.data_ptr(), stream=sp)
    stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in sub:
        ctx.align_device(int(kinds[i]), d_sym.data_ptr() + 4 * int(pairs[i]["a_off"]), int(pairs[i]["n1"]),
                         d_sym.data_ptr() + 4 * int(pairs[i]["b_off"]), int(pairs[i]["n2"]), d_one.data_ptr(), stream=sp)
    e1.record(stream)
    stream.synchronize()
    plain_gcups = float(cells_k[sub].sum()) / (e0.elapsed_time(e1) / 1e3) / 1e9
    del offs

    # what batching buys where one pair alone already fills part of the GPU: 64 pairs
    # with lengths log-uniform in [2048, 4096], one planned launch against one plain
    # call per pair (both on resident inputs, CUDA events)
    lrng = np.random.default_rng(synth.SEED_BATCH + 7)
    lk = lrng.integers(0, 3, 64)
    la = np.exp(lrng.uniform(np.log(2048), np.log(4096), 64)).astype(int)
    lb = np.exp(lrng.uniform(np.log(2048), np.log(4096), 64)).astype(int)
    lsa = [lrng.integers(0, 4, int(x)).astype(np.int32) for x in la]
    lsb = [lrng.integers(0, 4, int(x)).astype(np.int32) for x in lb]
    lsym, lpairs = g.pack_batch(lk, lsa, lsb)
    lcells = float((la.astype(np.float64) * lb).sum())
    with torch.cuda.stream(stream):
        ld_sym = torch.from_numpy(lsym).to(dev)
        ld_res = torch.zeros(64 * g.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    lplan = g.BatchPlan(ctx, lpairs, len(lsym))
    for _ in range(3):
        lplan.run(ld_sym.data_ptr(), ld_res.data_ptr(), stream=sp, use_graph=True)
    e0.record(stream)
    for _ in range(10):
        lplan.run(ld_sym.data_ptr(), ld_res.data_ptr(), stream=sp, use_graph=True)
    e1.record(stream)
    stream.synchronize()
    large_batched = lcells * 10 / (e0.elapsed_time(e1) / 1e3) / 1e9
    lres = np.frombuffer(ld_res.cpu().numpy().tobytes(), g.RESULT_DTYPE)
    large_ok = bool((lres["score"] == O.align_batch(lk, lsa, lsb, threads=os.cpu_count() or 1)["score"]).all())
    lplan.close()

    def _plain_all():
        for i in range(64):
            ctx.align_device(int(lk[i]), ld_sym.data_ptr() + 4 * int(lpairs[i]["a_off"]), int(lpairs[i]["n1"]),
                             ld_sym.data_ptr() + 4 * int(lpairs[i]["b_off"]), int(lpairs[i]["n2"]),
                             d_one.data_ptr(), stream=sp)
    _plain_all()
    stream.synchronize()
    e0.record(stream)
    _plain_all()
    e1.record(stream)
    stream.synchronize()
    large_plain = lcells / (e0.elapsed_time(e1) / 1e3) / 1e9
    large = {"pairs": 64, "lengths": "log-uniform [2048, 4096], LCS/ED/SW mixed", "cells": lcells,
             "batched_gcups": large_batched, "plain_per_pair_gcups": large_plain,
             "batched_over_plain": large_batched / large_plain, "parity_vs_oracle": "ok" if large_ok else "MISMATCH"}

    props = torch.cuda.get_device_properties(local)
    sms = props.multi_processor_count
    mhz = clk.get("sm_mhz") or 1920.0
    peak_tops = sms * INT_LANES_PER_SM * mhz * 1e6 / 1e12
    achieved = ops / mean_s / 1e12
    roof = {"bound": "int_alu", "achieved": achieved, "peak": peak_tops, "unit": "Tops/s",
            "frac": achieved / peak_tops,
            "traffic": profiled_traffic("batch_kernel_batched16384") if n == 16384 else None,
            "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum of one launch, ncu capture in "
                            "profiles/batch_kernel_batched16384.md",
            "peak_basis": f"{sms} SMs x {INT_LANES_PER_SM} INT32 lanes x median SM clock {mhz:.0f} MHz under load",
            "ops_per_cell": "LCS 4, ED 7, SW 8 weighted by cells", "kernel": "batch_kernel (whole graph timed)"}
    cpu = None
    if rank == 0 and not args.no_cpu:
        k = min(n, 3000)
        t0 = time.perf_counter()
        O.align_batch(kinds[:k], sa[:k], sb[:k], threads=os.cpu_count() or 1)
        dt = time.perf_counter() - t0
        cpu = {"value": float(cells_k[:k].sum()) / dt / 1e9, "unit": "GCUPS", "cores": os.cpu_count(),
               "kind": "port", "sample": f"first {k} of the {n} pairs ({cells_k[:k].sum():.3g} cells), "
                                         f"oracle/oracle.c pairs across {os.cpu_count()} threads, {dt:.2f} s"}
    cfg = {"workload": f"batched: {n} pairs, lengths log-uniform [64, 4096], alphabet 4, LCS/ED/SW 1/3 each, "
                       "one planned launch replayed as a CUDA graph",
           "pairs": n, "cells": cells, "seed": synth.SEED_BATCH, "split": split,
           "l2": "flushed between timed steps (256 MiB write)", "parity_vs_oracle": "ok" if parity else "MISMATCH",
           "plain_per_pair_gcups": plain_gcups, "plain_sample_pairs": int(len(sub)),
           "batched_over_plain": value / ws / plain_gcups, "large_pairs": large}
    line = {"metric": METRIC, "value": value, "unit": "GCUPS", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * mean_s,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32" if args.int32 else "int16x2 (pairs whose scores fit 16 bits) / int32",
            "data": "synthetic (seeded)", "config": cfg, "clocks": clk, "e2e": e2e,
            "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu,
            "step_ms": {"min": min(step_ms), "median": statistics.median(step_ms), "max": max(step_ms)}}
    plan.close()
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return line if rank == 0 else None


def _percentiles(lat_ns):
    if len(lat_ns) == 0:
        return {"p50_ms": None, "p99_ms": None}
    return {"p50_ms": float(np.percentile(lat_ns, 50)) / 1e6, "p99_ms": float(np.percentile(lat_ns, 99)) / 1e6,
            "max_ms": float(np.max(lat_ns)) / 1e6}


def _collect_served(srv, want):
    """Drains the server and takes `want` results: (tickets, results, latencies) in completion order."""
    if not srv.drain(600):
        raise RuntimeError("served: drain timed out")
    ts, rs, ls = [], [], []
    got = 0
    while got < want:
        t, r, l = srv.poll_many(65536)
        if len(t) == 0:
            break
        ts.append(t); rs.append(r); ls.append(l)
        got += len(t)
    return np.concatenate(ts), np.concatenate(rs), np.concatenate(ls)


def run_gme_served(args):
    """Served path: the request stream submitted open loop; saturation GCUPS, then a
    Poisson arrival-rate sweep with p50/p99 latency; the same requests as one batch."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    import __graft_entry__ as ge
    ge.build()
    import gpumemefficient_gb300 as g
    from gpumemefficient_gb300 import synth
    from oracle import oracle as O

    symbols, pairs = synth.served_requests(args.requests)
    n = len(pairs)
    kinds = pairs["kind"]
    cells_k = pairs["n1"].astype(np.float64) * pairs["n2"]
    cells = float(cells_k.sum())
    ops = float(sum(cells_k[kinds == k].sum() * OPS_PER_CELL[k] for k in range(3)))
    sc = g.scoring()
    mode = g.SERVE_WAVES if args.serve_mode == "waves" else g.SERVE_RING
    srv = g.Server(local, sc=sc, waves=args.waves, wave_max_cells=args.wave_cells, mode=mode)

    # parity of every request with the oracle (outside the timed region)
    tick = srv.submit_many(symbols, pairs)
    assert len(tick) == n, "served: the queue took only part of one pass"
    t_, r_, _ = _collect_served(srv, n)
    order = np.argsort(t_)
    res = r_[order]
    assert (np.sort(t_) == np.sort(tick)).all()
    sa = [symbols[o:o + k] for o, k in zip(pairs["a_off"], pairs["n1"])]
    sb = [symbols[o:o + k] for o, k in zip(pairs["b_off"], pairs["n2"])]
    parity = None
    if not args.no_parity:
        o = O.align_batch(kinds, sa, sb, threads=os.cpu_count() or 1)
        sw = kinds == 2
        parity = bool((res["status"] == 0).all() and (res["score"] == o["score"]).all() and
                      (res["sw_max"][sw] == o["sw_max"][sw]).all() and
                      (res["sw_max_y"][sw] == o["sw_y"][sw]).all() and (res["sw_max_x"][sw] == o["sw_x"][sw]).all())

    def saturate(passes):
        """Every request of the stream, `passes` times, submitted back to back as fast
        as the host can (chunks of 1024), then drained: sustained throughput."""
        t0 = time.perf_counter()
        for _ in range(passes):
            for c in range(0, n, 1024):
                chunk = pairs[c:c + 1024]
                while len(chunk):
                    chunk = chunk[len(srv.submit_many(symbols, chunk)):]
                    if len(chunk):
                        time.sleep(0.001)  # the queue is full: let the dispatcher catch up
        _, _, lat = _collect_served(srv, n * passes)
        return time.perf_counter() - t0, lat

    saturate(args.warmup)
    st0 = srv.stats()
    clocks = ClockSampler(local)
    time.sleep(0.15)
    t_tot, lat_sat = saturate(args.steps)
    clk = clocks.stop()
    st1 = srv.stats()
    times = [t_tot / args.steps] * args.steps
    value = cells * args.steps / t_tot / 1e9

    # arrival-rate sweep: Poisson arrivals at a fraction of the saturation throughput
    rng = np.random.default_rng(synth.SEED_SERVE + 1)
    mean_cells = cells / n
    sweep = []
    for frac in args.rates:
        lam = frac * value * 1e9 / mean_cells          # requests per second
        m = int(min(n, max(200, lam * args.rate_seconds)))
        idx = rng.permutation(n)[:m]
        arr = np.cumsum(rng.exponential(1.0 / lam, m))
        sub_pairs = pairs[idx]
        call_t = np.zeros(m)
        t0 = time.perf_counter()
        i = 0
        while i < m:
            now = time.perf_counter() - t0
            j = int(np.searchsorted(arr, now, side="right"))
            if j > i:
                j = i + len(srv.submit_many(symbols, sub_pairs[i:j]))  # a full queue takes a prefix
                call_t[i:j] = time.perf_counter() - t0
                i = j
            else:
                wait = arr[i] - now
                if wait > 2e-4:
                    time.sleep(wait - 1e-4)
        tk, rr, ll = _collect_served(srv, m)
        t_end = time.perf_counter() - t0
        # open-loop latency: from the scheduled arrival, so a late submission counts
        first = int(tk.min())
        late = (call_t - arr)[(tk - first).astype(np.int64)]
        lat = ll + late * 1e9
        sweep.append({"offered_fraction": frac, "requests": m, "offered_gcups": frac * value,
                      "achieved_gcups": float(cells_k[idx].sum()) / t_end / 1e9,
                      **_percentiles(lat), "max_submit_lag_ms": float(late.max() * 1e3),
                      "ok": bool((rr["status"] == 0).all())})

    # the same requests as one planned batch (graph replay, inputs resident)
    ctx = g.Context(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=local)
    sp = stream.cuda_stream
    with torch.cuda.stream(stream):
        d_sym = torch.from_numpy(symbols).to(dev)
        d_res = torch.zeros(n * g.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    stream.synchronize()
    plan = g.BatchPlan(ctx, pairs, len(symbols))
    for _ in range(3):
        plan.run(d_sym.data_ptr(), d_res.data_ptr(), stream=sp, use_graph=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        plan.run(d_sym.data_ptr(), d_res.data_ptr(), stream=sp, use_graph=True)
    e1.record(stream)
    stream.synchronize()
    batched = cells * args.steps / (e0.elapsed_time(e1) / 1e3) / 1e9
    plan.close()
    ctx.close()

    props = torch.cuda.get_device_properties(local)
    sms = props.multi_processor_count
    mhz = clk.get("sm_mhz") or 1920.0
    peak_tops = sms * INT_LANES_PER_SM * mhz * 1e6 / 1e12
    achieved = ops * len(times) / t_tot / 1e12
    roof = {"bound": "int_alu", "achieved": achieved, "peak": peak_tops, "unit": "Tops/s",
            "frac": achieved / peak_tops, "traffic": None,
            "peak_basis": f"{sms} SMs x {INT_LANES_PER_SM} INT32 lanes x median SM clock {mhz:.0f} MHz under load",
            "ops_per_cell": "ED 7, SW 8 weighted by cells",
            "kernel": ("serve_kernel" if mode == g.SERVE_RING else "batch_kernel") + " (served, host clock)"}
    cpu = None
    if rank == 0 and not args.no_cpu:
        k = min(n, 400)
        t0 = time.perf_counter()
        O.align_batch(kinds[:k], sa[:k], sb[:k], threads=os.cpu_count() or 1)
        dt = time.perf_counter() - t0
        cpu = {"value": float(cells_k[:k].sum()) / dt / 1e9, "unit": "GCUPS", "cores": os.cpu_count(),
               "kind": "port", "sample": f"first {k} of the {n} requests ({cells_k[:k].sum():.3g} cells), "
                                         f"oracle/oracle.c pairs across {os.cpu_count()} threads, {dt:.2f} s"}
    h2d = int(symbols.nbytes + n * (pairs.itemsize + 64))
    d2h = int(n * (g.RESULT_DTYPE.itemsize + 4))
    how = ("one persistent kernel taking jobs from device-resident rings" if mode == g.SERVE_RING else
           "waves of the batched kernel on launch slots on separate streams")
    cfg = {"workload": f"served: {n} requests per step, half ED half SW, lengths log-uniform [32, 16384], "
                       f"alphabet 4, submitted open loop to the server (host queue, HBM-budget admission, {how}, "
                       "completion flags in pinned memory); value = sustained throughput with `steps` passes "
                       "of the stream submitted back to back",
           "serve_mode": args.serve_mode,
           "requests": n, "cells": cells, "seed": synth.SEED_SERVE, "hbm_budget_bytes": st1["hbm_budget_bytes"],
           "hbm_bytes_peak": st1["hbm_bytes_peak"], "waves_per_step": (st1["waves_launched"] - st0["waves_launched"]) / len(times),
           "l2": "inputs (172 MB of symbols per step) larger than L2", "parity_vs_oracle": {True: "ok", False: "MISMATCH", None: "skipped"}[parity],
           "waves": args.waves, "wave_max_cells": args.wave_cells,
           "saturation_latency": _percentiles(lat_sat), "rate_sweep": sweep,
           "batched_same_requests_gcups": batched, "served_over_batched": value / batched}
    line = {"metric": METRIC, "value": value, "unit": "GCUPS", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_tot / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded)", "config": cfg, "clocks": clk,
            "e2e": {"value": value, "unit": "GCUPS", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "note": "the served path is end to end: host symbols in, host results out"},
            "gpu_launches": int(st1["kernels_launched"] - st0["kernels_launched"]), "roofline": roof,
            "cpu_baseline": cpu}
    srv.close()
    return line


def run_gme_path(args):
    """Alignment path of the headline pair (Hirschberg on the GPU): the same GCUPS metric
    over the n1 x n2 cells of the problem (the traceback itself computes about twice
    that many), host sequences in, the edit script out."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    import __graft_entry__ as ge
    ge.build()
    import gpumemefficient_gb300 as g
    from oracle import oracle as O
    kind, a, b, cfg = workload("ed65536" if args.workload == "path" else args.workload)
    ctx = g.Context(local)
    score, ops = ctx.align_path(kind, a, b)
    want = O.align(kind, a, b, rule=O.ED_STANDARD, threads=os.cpu_count() or 1)["score"]
    cost = sum(1 for c in ops if c != "M") + sum(1 for i, j, c in _walk(ops) if c == "M" and a[i] != b[j])
    parity = score == want and cost == want
    for _ in range(args.warmup):
        ctx.align_path(kind, a, b)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ctx.align_path(kind, a, b)
        times.append(time.perf_counter() - t0)
    cells = len(a) * len(b)
    t = sum(times) / len(times)
    cfg = dict(cfg)
    cfg.update({"workload": cfg["workload"] + "; optimal alignment path (edit script), Hirschberg on the GPU",
                "ed_boundary": "standard", "parity_vs_oracle": "ok" if parity else "MISMATCH",
                "script_length": len(ops), "score": score})
    line = {"metric": METRIC, "value": cells / t / 1e9, "unit": "GCUPS", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded)", "config": cfg,
            "e2e": {"value": cells / t / 1e9, "unit": "GCUPS", "h2d_bytes_per_step": int(a.nbytes + b.nbytes),
                    "d2h_bytes_per_step": len(ops)},
            "gpu_launches": None, "roofline": None, "cpu_baseline": None}
    ctx.close()
    return line


def sat_cpu_baseline(host, n1: int, n2: int, ld: int, target_s: float = 2.0, max_reps: int = 200):
    """The SAT recurrence on all host threads (oracle port) over rows 1..k of the table,
    repeated until about `target_s` seconds (each repetition is the same work)."""
    from oracle import oracle as O
    k = min(n2, 8192)
    threads = os.cpu_count() or 1
    sample = np.ascontiguousarray(host[:k + 1]).copy()
    reps, dt = 0, 0.0
    while dt < target_s and reps < max_reps:
        t0 = time.perf_counter()
        O.lib().orc_sat_mt(O._p32(sample), n1, k, ld, threads)
        dt += time.perf_counter() - t0
        reps += 1
    return {"value": n1 * k * reps / dt / 1e9, "unit": "GCUPS", "cores": threads, "kind": "port",
            "sample": f"rows 1..{k} of the table ({n1 * k:.3g} cells) x {reps}, oracle/oracle.c row "
                      f"prefixes then column sums on {threads} threads, {dt:.2f} s"}


def run_gme_sat(args):
    """Summed-area table of the reference's SAT case `15 15` (a 32768 x 32768 interior
    in the reference's layout: n2 + 2 rows of n1 + 3 ints, values rand() % 10000 as its
    generator writes them), in place on the device: cell updates per second, HBM
    roofline at 8 bytes per cell (each cell read and written once)."""
    import json as _json
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    import __graft_entry__ as ge
    ge.build()
    import gpumemefficient_gb300 as g
    from oracle import oracle as O
    n1 = n2 = args.sat_n
    # the reference's layout (rows of n1 + 3 ints), or rows rounded up to 16 bytes, which
    # takes the tensor-map kernel
    ld = n1 + 3 if args.sat_layout == "reference" else (n1 + 3 + 3) // 4 * 4
    rng = np.random.default_rng(0x5A7)
    host = rng.integers(0, 10000, (n2 + 2, ld), dtype=np.int32)
    cells = n1 * n2
    ctx = g.Context(local)
    dev = torch.device("cuda", local)
    # one explicit stream for the copies, the kernel and the events (a null stream
    # handle would mean the library's own stream)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    d0 = torch.from_numpy(host).to(dev)
    d = torch.empty_like(d0)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    # parity: the whole table against the oracle (outside the timed region)
    d.copy_(d0)
    ctx.sat_device(d.data_ptr(), n1, n2, ld, status.data_ptr(), stream.cuda_stream)
    stream.synchronize()
    got = d.cpu().numpy()
    want = O.sat(host, n1, n2)
    parity = bool(int(status.item()) == 0 and np.array_equal(got, want))
    del got, want
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(args.warmup):
        d.copy_(d0)
        ctx.sat_device(d.data_ptr(), n1, n2, ld, status.data_ptr(), stream.cuda_stream)
    times = []
    l0 = ctx.launches
    clocks = ClockSampler(local)
    for _ in range(args.steps):
        d.copy_(d0)          # the input back (untimed); then L2 emptied of it
        flush.fill_(1)
        e0.record(stream)
        ctx.sat_device(d.data_ptr(), n1, n2, ld, status.data_ptr(), stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    clk = clocks.stop()
    launches = ctx.launches - l0
    ok_status = int(status.item()) == 0
    t = sum(times) / len(times)
    value = cells / t / 1e9
    # end to end through gme_sat: pinned host table in, rows 1..n2 back, every step
    pinned = torch.from_numpy(host).pin_memory()
    ctx.sat(pinned.numpy(), n1, n2)
    et = []
    for _ in range(max(1, min(args.steps, 5))):
        t0 = time.perf_counter()
        ctx.sat(pinned.numpy(), n1, n2)  # in place: each step recomputes on the last output (same work)
        et.append(time.perf_counter() - t0)
    e2e = cells / (sum(et) / len(et)) / 1e9
    try:
        peak = _json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))["hbm_gbs"]
        basis = "MEASURED_PEAKS.json hbm_gbs (copy, measured on this pool)"
    except (OSError, KeyError, ValueError):
        peak, basis = 6800.0, "fallback 6.8 TB/s"
    achieved = 8.0 * cells / t / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": profiled_traffic("sat_ws_kernel_16384" if ld % 4 else "sat_tma_kernel_16384"),
            "peak_basis": basis, "bytes_per_cell": 8,
            "kernel": ("sat_ws_kernel (cp.async)" if ld % 4 else "sat_tma_kernel (tensor maps)") + " (one launch)"}
    cpu = sat_cpu_baseline(host, n1, n2, ld) if rank == 0 and not args.no_cpu else None
    layout = "the reference's layout" if ld == n1 + 3 else "rows padded to 16 bytes"
    cfg = {"workload": f"summed-area table, {n1} x {n2} interior in {layout} "
                       f"({n2 + 2} rows of {ld} ints, values 0..9999 seeded), in place, one launch",
           "layout": args.sat_layout,
           "n1": n1, "n2": n2, "ld": ld, "seed": 0x5A7,
           "l2": "table (4.3 GB at 32768) larger than L2; input restored and L2 flushed (256 MiB write) before each step",
           "parity_vs_oracle": "ok" if parity and ok_status else "MISMATCH"}
    line = {"metric": METRIC, "value": value, "unit": "GCUPS", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32 (wrapping)", "data": "synthetic (seeded)", "config": cfg,
            "clocks": clk,
            "e2e": {"value": e2e, "unit": "GCUPS", "h2d_bytes_per_step": int((n2 + 1) * ld * 4),
                    "d2h_bytes_per_step": int(n2 * ld * 4), "note": "gme_sat from pinned host memory"},
            "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu,
            "step_ms": {"min": 1e3 * min(times), "median": 1e3 * statistics.median(times),
                        "max": 1e3 * max(times)}}
    ctx.close()
    return line


def run_gme_baselines(args):
    """The plain path beside the comparison baselines -- the reference's table-based
    strategies on this GPU (the whole DP table in HBM; one launch per anti-diagonal of
    128 x 64 tiles, LCS/GPU_TILE_SHARE.cu; or of cells, EditDistance/GPU.cu) -- on
    the same edit-distance pairs, every result checked against the oracle."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    import __graft_entry__ as ge
    ge.build()
    import gpumemefficient_gb300 as g
    from gpumemefficient_gb300 import synth
    from oracle import oracle as O
    ctx = g.Context(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    sc = g.scoring()
    out = torch.zeros(g.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rows = []
    l0 = ctx.launches
    clocks = ClockSampler(local)
    for n in args.baseline_sizes:
        a, b = synth.ed_pair(n)
        want = int(O.align(O.ED, a, b, threads=os.cpu_count() or 1)["score"])
        da = torch.from_numpy(a).to(dev)
        db = torch.from_numpy(b).to(dev)
        table = torch.empty((n + 1) * (n + 1), dtype=torch.int32, device=dev)
        runs = {
            "plain (this library)": lambda: ctx.align_device(1, da.data_ptr(), n, db.data_ptr(), n, out.data_ptr(), stream=sp),
            "tiles 128x64, a launch per tile anti-diagonal": lambda: ctx.baseline_align_device(
                g.BASELINE_TILES, 1, da.data_ptr(), n, db.data_ptr(), n, table.data_ptr(), out.data_ptr(),
                tile_x=64, tile_y=128, sc=sc, stream=sp),
            "cells, a launch per cell anti-diagonal": lambda: ctx.baseline_align_device(
                g.BASELINE_CELLS, 1, da.data_ptr(), n, db.data_ptr(), n, table.data_ptr(), out.data_ptr(), sc=sc,
                stream=sp),
        }
        for name, fn in runs.items():
            fn()
            stream.synchronize()
            got = int(np.frombuffer(out.cpu().numpy().tobytes(), g.RESULT_DTYPE)[0]["score"])
            reps = 5 if name.startswith("plain") else 2
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
            stream.synchronize()
            ms = e0.elapsed_time(e1) / reps
            rows.append({"n": n, "strategy": name, "ms": ms, "gcups": n * n / ms / 1e6,
                         "table_bytes": 0 if name.startswith("plain") else (n + 1) * (n + 1) * 4,
                         "parity_vs_oracle": "ok" if got == want else "MISMATCH"})
        del table
    clk = clocks.stop()
    plain = {r["n"]: r["gcups"] for r in rows if r["strategy"].startswith("plain")}
    for r in rows:
        r["plain_over_this"] = plain[r["n"]] / r["gcups"]
    line = {"metric": METRIC, "value": plain[max(plain)], "unit": "GCUPS", "n_gpus": 1, "steps": 5, "warmup": 1,
            "ms_per_step": min(r["ms"] for r in rows if r["n"] == max(plain) and r["strategy"].startswith("plain")),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded)",
            "config": {"workload": "edit distance, one n x n pair per call (10% seeded edits): the plain path beside "
                                   "the reference's table-based strategies rebuilt on this GPU",
                       "rows": rows},
            "clocks": clk, "gpu_launches": ctx.launches - l0, "roofline": None, "cpu_baseline": None}
    ctx.close()
    return line


def _walk(ops):
    i = j = 0
    for c in ops:
        yield i, j, c
        if c == "M":
            i += 1
            j += 1
        elif c == "D":
            i += 1
        else:
            j += 1


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gme", choices=["gme", "reference"])
    p.add_argument("--workload", default="ed65536")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--pairs", type=int, default=16384, help="batched workload: number of pairs")
    p.add_argument("--plain-sample", type=int, default=256,
                   help="batched workload: pairs timed one by one on the plain path")
    p.add_argument("--batch-warps", type=int, default=0, help="batched workload: warps per CTA")
    p.add_argument("--int32", action="store_true",
                   help="batched workload: every pair on the int32 engine (default: pairs that fit "
                        "16 bits on the packed s16x2 engine)")
    p.add_argument("--requests", type=int, default=8192, help="served workload: requests per step")
    p.add_argument("--waves", type=int, default=0, help="served workload: launch slots (0 = default)")
    p.add_argument("--rates", type=float, nargs="*", default=[0.1, 0.3, 0.5, 0.7, 0.9, 1.0, 1.2],
                   help="served workload: offered load as fractions of the saturation throughput")
    p.add_argument("--serve-mode", default="ring", choices=["ring", "waves"],
                   help="served workload: persistent kernel on device job rings, or waves of launches")
    p.add_argument("--rate-seconds", type=float, default=2.0, help="served workload: seconds per rate point")
    p.add_argument("--wave-cells", type=int, default=0, help="served workload: cells per launch at most (0 = default)")
    p.add_argument("--no-parity", action="store_true", help="skip the oracle parity check (tuning runs)")
    p.add_argument("--baseline-sizes", type=int, nargs="+", default=[8192, 16384],
                   help="baselines workload: square ED sizes")
    p.add_argument("--sat-layout", choices=["reference", "aligned"], default="reference",
                   help="sat workload: rows of n1 + 3 ints (the reference's), or rounded up to 16 bytes")
    p.add_argument("--sat-n", type=int, default=32768,
                   help="sat workload: interior side (the reference's `15 15` case is 32768)")
    p.add_argument("--solo", action="store_true",
                   help="default workload only (no batched/served summaries beside it)")
    args = p.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "batched":
        line = run_gme_batch(args)
    elif args.workload == "served":
        line = run_gme_served(args)
    elif args.workload == "path":
        line = run_gme_path(args)
    elif args.workload == "sat":
        line = run_gme_sat(args)
    elif args.workload == "baselines":
        line = run_gme_baselines(args)
    else:
        line = run_gme(args)
        ws = dist_env()[0]
        if line is not None and args.workload == "ed65536" and ws == 1 and not args.solo:
            line["also"] = also_batched_served(args)
    if line is not None:
        print(json.dumps(line), flush=True)


def also_batched_served(args):
    """Short runs of the batched and served workloads, summarised beside the headline
    line (the metric compares batched/served with the plain per-pair path), and of the
    summed-area table (the reference's SAT case)."""
    import copy
    out = {}
    # the other single-pair workloads on the plain path: LCS 8192^2 and SW 32768^2
    for name in ("lcs8192", "sw32768"):
        a = copy.copy(args)
        a.workload, a.steps, a.warmup, a.no_cpu = name, 20, 3, True
        try:
            p = run_gme(a)
            c = p["config"]
            out[name] = {"workload": c["workload"], "value": p["value"], "unit": "GCUPS",
                         "ms_per_step": p["ms_per_step"], "e2e": p["e2e"]["value"],
                         "roofline": {k: p["roofline"][k] for k in
                                      ("bound", "achieved", "peak", "unit", "frac", "ops_per_cell")},
                         "plain_config": c["plain_config"], "parity_vs_oracle": c["parity_vs_oracle"],
                         "score": c["score"], "gpu_launches": p["gpu_launches"], "clocks": p["clocks"]}
        except Exception as e:  # the headline line stands on its own
            out[name] = {"error": repr(e)[:300]}
    a = copy.copy(args)
    a.steps, a.warmup, a.no_cpu, a.pairs, a.batch_warps, a.int32 = 10, 3, True, 16384, 0, False
    b = run_gme_batch(a)
    c = b["config"]
    out["batched"] = {"workload": c["workload"], "value": b["value"], "unit": "GCUPS",
                      "ms_per_step": b["ms_per_step"], "e2e": b["e2e"]["value"],
                      "plain_per_pair_gcups": c["plain_per_pair_gcups"],
                      "batched_over_plain": c["batched_over_plain"], "large_pairs": c["large_pairs"],
                      "split": c["split"],
                      "parity_vs_oracle": c["parity_vs_oracle"], "roofline_frac": b["roofline"]["frac"],
                      "gpu_launches": b["gpu_launches"], "clocks": b["clocks"]}
    a = copy.copy(args)
    a.steps, a.warmup, a.no_cpu, a.requests, a.waves, a.wave_cells = 5, 3, True, 8192, 0, 0
    a.rates, a.rate_seconds, a.no_parity, a.serve_mode = [0.1, 0.5, 0.8, 1.0], 1.5, False, "ring"
    s = run_gme_served(a)
    c = s["config"]
    out["served"] = {"workload": c["workload"], "value": s["value"], "unit": "GCUPS",
                     "batched_same_requests_gcups": c["batched_same_requests_gcups"],
                     "served_over_batched": c["served_over_batched"], "rate_sweep": c["rate_sweep"],
                     "parity_vs_oracle": c["parity_vs_oracle"], "hbm_bytes_peak": c["hbm_bytes_peak"],
                     "hbm_budget_bytes": c["hbm_budget_bytes"], "gpu_launches": s["gpu_launches"],
                     "clocks": s["clocks"]}
    # last: it sets its own stream as the current one; the reference's layout (cp.async
    # kernel), then rows padded to 16 bytes (tensor-map kernel)
    for key, layout in (("sat", "reference"), ("sat_aligned", "aligned")):
        a = copy.copy(args)
        a.steps, a.warmup, a.no_cpu, a.sat_n, a.sat_layout = 10, 3, True, 32768, layout
        try:
            t = run_gme_sat(a)
            c = t["config"]
            out[key] = {"workload": c["workload"], "value": t["value"], "unit": "GCUPS",
                        "ms_per_step": t["ms_per_step"], "e2e": t["e2e"]["value"],
                        "roofline": {k: t["roofline"][k] for k in ("bound", "achieved", "peak", "unit", "frac", "kernel")},
                        "parity_vs_oracle": c["parity_vs_oracle"], "gpu_launches": t["gpu_launches"],
                        "clocks": t["clocks"]}
        except Exception as e:  # the headline line stands on its own
            out[key] = {"error": repr(e)[:300]}
    return out


if __name__ == "__main__":
    main()
