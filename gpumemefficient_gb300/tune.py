"""Autotuner of the batched kernel.

Sweeps, per length bucket, the launch shape and the job-class cut-offs of the
batched work-queue kernel:

* warps per CTA (the CTA's tile: warps_per_block x 32 lanes x 4 rows of a band group),
* CTAs per SM,
* block_min_cells (pairs at least this large run one per CTA, the rest one per warp),
* team_min_cells (pairs at least this large run on a team of CTAs),
* the tile height: rows per lane (4: 128-row bands, or 2: 64-row bands),
* the engine: packed 16-bit cells where values fit (at 4 rows per lane), or int32 only,

on seeded synthetic batches whose lengths are log-uniform within the bucket (LCS,
ED and SW one third each), timing CUDA-graph replays of one planned launch with CUDA
events.  Every configuration is checked bit-exact against the first one's results
(which the batched tests pin to the oracle).

    python -m gpumemefficient_gb300.tune [--out-json F] [--out-md F] [--quick]

writes the whole sweep (`--out-md`, a table) and the winners per bucket
(`--out-json`).  `gen_header()` (or `--header`, or `header_from_json()` on a
committed result) turns the winners into `csrc/gme_tuned.h`, the table the
library's batch plan consults when the caller has not set a batch configuration
(gme_set_batch_config): the entry whose length range is nearest the batch's.
"""
from __future__ import annotations

import argparse
import itertools
import json
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TUNED_JSON = os.path.join(HERE, "tuned.json")
TUNED_H = os.path.join(HERE, "csrc", "gme_tuned.h")

# (name, shortest, longest length); the buckets tile the lengths the batch kernel takes
BUCKETS = [
    ("short", 32, 512),
    ("mid", 512, 2048),
    ("long", 2048, 8192),
    ("wide", 8192, 16384),
]
# the two benchmark distributions, tuned and reported beside the buckets
MIXES = [
    ("mixed_64_4096", 64, 4096),
    ("mixed_32_16384", 32, 16384),
]

GRID = {
    "warps_per_block": [4, 8],
    "blocks_per_sm": [0, 2],
    "block_min_cells": [1 << 20, 1 << 21, 1 << 22, 1 << 23],
    "team_min_cells": [1 << 24, 1 << 25, 1 << 26, -1],
    "team_split": [2, 3, 4],
    "rows_per_lane": [4, 2],
    "packed16": [0, -1],   # 0: packed where values fit, -1: int32 for every pair
}
QUICK_GRID = {
    "warps_per_block": [4, 8],
    "blocks_per_sm": [0],
    "block_min_cells": [1 << 21, 1 << 22],
    "team_min_cells": [1 << 25, -1],
    "team_split": [2],
    "rows_per_lane": [4, 2],
    "packed16": [0, -1],
}


def redundant(cfg, grid) -> bool:
    """Configurations that repeat another: without teams the split changes nothing; at
    2 rows per lane there is no packed engine."""
    if cfg.get("team_min_cells") == -1 and cfg.get("team_split", 2) != grid.get("team_split", [2])[0]:
        return True
    if cfg.get("rows_per_lane", 4) == 2 and cfg.get("warps_per_block") == 4:
        return True  # 2 rows per lane exists only with 8 warps per CTA
    return cfg.get("rows_per_lane", 4) == 2 and cfg.get("packed16", 0) != -1


def lengths_for(lo: int, hi: int, cells: float, rng):
    """Lengths of a and b, log-uniform in [lo, hi], for about `cells` cells."""
    mean = ((hi - lo) / np.log(hi / lo)) ** 2
    n = int(min(40000, max(64, cells / mean)))
    la = np.exp(rng.uniform(np.log(lo), np.log(hi), n)).astype(np.int64)
    lb = np.exp(rng.uniform(np.log(lo), np.log(hi), n)).astype(np.int64)
    return la, lb


def length_range(la, lb):
    """The statistic the batch plan matches table entries by (batch_tuning_for): the
    2nd and 98th percentile of sqrt(n1 * n2) + 1 over the batch's pairs."""
    v = np.sort(np.sqrt(la.astype(np.float64) * lb) + 1.0)
    n = len(v)
    return float(v[int(0.02 * (n - 1))]), float(v[int(0.98 * (n - 1))])


def bucket_range(lo: int, hi: int, cells: float, seed: int):
    return length_range(*lengths_for(lo, hi, cells, np.random.default_rng(seed)))


def batch_for(lo: int, hi: int, cells: float, seed: int):
    """Seeded pairs with lengths log-uniform in [lo, hi] until about `cells` cells."""
    from . import pack_batch
    rng = np.random.default_rng(seed)
    la, lb = lengths_for(lo, hi, cells, rng)
    n = len(la)
    kinds = np.repeat(np.arange(3, dtype=np.int32), (n + 2) // 3)[:n]
    rng.shuffle(kinds)
    sa = [rng.integers(0, 4, int(k), dtype=np.int64).astype(np.int32) for k in la]
    sb = [rng.integers(0, 4, int(k), dtype=np.int64).astype(np.int32) for k in lb]
    symbols, pairs = pack_batch(kinds, sa, sb)
    return symbols, pairs, float((la * lb).sum())


def measure(ctx, d_sym, d_res, pairs, nsym, cfg, reps, stream):
    """GCUPS of one configuration (graph replays timed with CUDA events) and its results."""
    import torch
    from . import BatchPlan, RESULT_DTYPE
    ctx.set_batch_config(**cfg)
    plan = BatchPlan(ctx, pairs, nsym)
    split = ctx.batch_stats()
    sp = stream.cuda_stream
    try:
        for _ in range(2):
            plan.run(d_sym.data_ptr(), d_res.data_ptr(), stream=sp, use_graph=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            plan.run(d_sym.data_ptr(), d_res.data_ptr(), stream=sp, use_graph=True)
        e1.record(stream)
        stream.synchronize()
        ms = e0.elapsed_time(e1) / reps
    finally:
        plan.close()
        ctx.set_batch_config()
    res = np.frombuffer(d_res.cpu().numpy().tobytes(), RESULT_DTYPE).copy()
    return ms, split, res


def sweep(grid=None, cells: float = 1.5e10, reps: int = 5, device: int = 0, log=print):
    import torch
    from . import Context, RESULT_DTYPE
    grid = grid or GRID
    keys = list(grid)
    ctx = Context(device)
    dev = torch.device("cuda", device)
    stream = torch.cuda.Stream(device=device)
    rows = []
    for bi, (name, lo, hi) in enumerate(BUCKETS + MIXES):
        symbols, pairs, total = batch_for(lo, hi, cells, 0x5EED + bi)
        p_lo, p_hi = bucket_range(lo, hi, cells, 0x5EED + bi)
        d_sym = torch.from_numpy(symbols).to(dev)
        d_res = torch.zeros(len(pairs) * RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
        ref = None
        for vals in itertools.product(*(grid[k] for k in keys)):
            cfg = dict(zip(keys, vals))
            if redundant(cfg, grid):
                continue
            ms, split, res = measure(ctx, d_sym, d_res, pairs, len(symbols), cfg, reps, stream)
            ok = bool((res["status"] == 0).all())
            if ref is None:
                ref = res
            same = bool((res["score"] == ref["score"]).all() and (res["sw_max"] == ref["sw_max"]).all())
            row = {"bucket": name, "lo": lo, "hi": hi, "p_lo": p_lo, "p_hi": p_hi, "pairs": len(pairs),
                   "cells": total, **cfg,
                   "ms": ms, "gcups": total / ms / 1e6, "split": split, "ok": ok and same}
            rows.append(row)
            log(json.dumps(row))
        del d_sym, d_res
    ctx.close()
    return rows


def winners(rows):
    best = {}
    for r in rows:
        if not r["ok"]:
            continue
        b = best.get(r["bucket"])
        if b is None or r["gcups"] > b["gcups"]:
            best[r["bucket"]] = r
    return best


def write_md(rows, best, path, cmd):
    keys = ["warps_per_block", "blocks_per_sm", "block_min_cells", "team_min_cells"]
    lines = ["# Batched-kernel autotune sweep", "",
             f"Command (GB300): `{cmd}`", "",
             "GCUPS of one planned launch (CUDA-graph replay, CUDA events, mean of the replays) "
             "per length bucket; lengths log-uniform in [lo, hi], LCS/ED/SW one third each. "
             "`team_min_cells` -1 = no teams; groups/member: a team job of G band groups runs on "
             "clamp(G / that, 2, 8) CTAs. Every row's results equal the first row's. The match range "
             "is the statistic the plan picks a table entry by: the 2nd..98th percentile of "
             "sqrt(n1*n2)+1 over the bucket's pairs.", ""]
    for name in [b[0] for b in BUCKETS + MIXES]:
        rs = [r for r in rows if r["bucket"] == name]
        if not rs:
            continue
        w = best.get(name)
        rng_txt = f", match range [{rs[0]['p_lo']:.0f}, {rs[0]['p_hi']:.0f}]" if "p_lo" in rs[0] else ""
        lines.append(f"## {name}: lengths [{rs[0]['lo']}, {rs[0]['hi']}], {rs[0]['pairs']} pairs, "
                     f"{rs[0]['cells']:.3g} cells{rng_txt}")
        lines.append("")
        lines.append("| warps/CTA | CTAs/SM | block_min | team_min | groups/member | rows/lane | packed16 | ms | GCUPS | split (team/block/warp/plain) | |")
        lines.append("|---:|---:|---:|---:|---:|---:|---|---:|---:|---|---|")
        for r in sorted(rs, key=lambda r: -r["gcups"]):
            s = r["split"]
            mark = "best" if r == w else ("" if r["ok"] else "MISMATCH")
            lines.append(f"| {r['warps_per_block']} | {r['blocks_per_sm'] or 'max'} | 2^{int(np.log2(r['block_min_cells']))} | "
                         f"{('2^%d' % int(np.log2(r['team_min_cells']))) if r['team_min_cells'] > 0 else 'none'} | "
                         f"{r.get('team_split', 2)} | {r.get('rows_per_lane', 4)} | {'off' if r.get('packed16', 0) < 0 else 'on'} | "
                         f"{r['ms']:.3f} | {r['gcups']:.1f} | {s.get('team_jobs', 0)}/{s['block_jobs']}/{s['warp_jobs']}/{s['long_jobs']} | {mark} |")
        lines.append("")
    with open(path, "w") as f:
        f.write("\n".join(lines))


def gen_header(best, path=TUNED_H, cells: float = 1.5e10):
    """The winners per bucket (and per mix) as the table the batch plan reads; each
    entry's range is its own sweep batch's statistic (length_range)."""
    keys = [b for b in BUCKETS + MIXES if b[0] in best]
    out = ["// gme_tuned.h -- batched-kernel settings per length range, written by",
           "// gpumemefficient_gb300/tune.py from a sweep on GB300 (the sweep table is kept",
           "// beside the profiles).  A batch is planned with the entry whose range [lo, hi]",
           "// is nearest (in log scale) to the batch's own -- both the 2nd..98th percentile",
           "// of sqrt(n1*n2) + 1 over the pairs, for an entry those of the batch it was",
           "// tuned on -- unless the caller set its own.",
           "#pragma once", "", "namespace gme {", "",
           "struct TunedBucket {", "  float lo, hi;", "  int warps_per_block, blocks_per_sm;",
           "  long long block_min_cells, team_min_cells;", "  int team_split;",
           "  int rows_per_lane;  // 4 or 2", "  int packed16;       // 1: packed 16-bit cells where values fit",
           "};", "",
           f"constexpr int TUNED_BUCKETS = {len(keys)};",
           "constexpr TunedBucket TUNED[TUNED_BUCKETS > 0 ? TUNED_BUCKETS : 1] = {"]
    for bi, (name, lo, hi) in enumerate(BUCKETS + MIXES):
        if name not in best:
            continue
        r = best[name]
        p_lo, p_hi = (r["p_lo"], r["p_hi"]) if "p_lo" in r else bucket_range(lo, hi, cells, 0x5EED + bi)
        out.append(f"    {{{p_lo:.1f}f, {p_hi:.1f}f, {r['warps_per_block']}, {r['blocks_per_sm']}, {r['block_min_cells']}ll, "
                   f"{r['team_min_cells']}ll, {r.get('team_split', 2)}, {r.get('rows_per_lane', 4)}, "
                   f"{0 if r.get('packed16', 0) < 0 else 1}}},  // {name}: {r['gcups']:.0f} GCUPS")
    if not keys:
        out.append("    {1.0f, 1.0f, 4, 0, 1ll << 22, 1ll << 25, 2, 4, 1},")
    out += ["};", "", "}  // namespace gme", ""]
    with open(path, "w") as f:
        f.write("\n".join(out))


def header_from_json(path=TUNED_JSON):
    """Regenerates csrc/gme_tuned.h from a committed sweep result."""
    gen_header(json.load(open(path))["best"])


# ---- the plain path: one pair per call --------------------------------------------
PLAIN_SIZES = [2048, 4096, 8192, 16384, 32768, 65536]
PLAIN_SHAPES = [(4, 4), (4, 8), (2, 4), (2, 8)]
TUNED_PLAIN_H = os.path.join(HERE, "csrc", "gme_tuned_plain.h")


def sweep_plain(sizes=None, shapes=None, reps: int = 5, device: int = 0, log=print):
    """Per square size n (edit distance, n x n, seeded): rows per lane x warps per band,
    with the grid at one CTA per band up to the SM count (0) and, for more bands than
    SMs, the SM count; times one call by CUDA events.  Results must equal the first
    shape's."""
    import torch
    from . import Context
    sizes = sizes or PLAIN_SIZES
    shapes = shapes or PLAIN_SHAPES
    ctx = Context(device)
    dev = torch.device("cuda", device)
    st = torch.cuda.Stream(device=device)
    out = torch.zeros(32, dtype=torch.uint8, device=dev)
    rows = []
    for n in sizes:
        rng = np.random.default_rng(0xF00D + n)
        a = torch.from_numpy(rng.integers(0, 4, n).astype(np.int32)).to(dev)
        b = torch.from_numpy(rng.integers(0, 4, n).astype(np.int32)).to(dev)
        ref = None
        for R, NW in shapes:
            ctx.set_plain_config(R, NW, 0)
            for _ in range(2):
                ctx.align_device(1, a.data_ptr(), n, b.data_ptr(), n, out.data_ptr(), stream=st.cuda_stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            for _ in range(reps):
                ctx.align_device(1, a.data_ptr(), n, b.data_ptr(), n, out.data_ptr(), stream=st.cuda_stream)
            e1.record(st)
            st.synchronize()
            ms = e0.elapsed_time(e1) / reps
            score = bytes(out.cpu().numpy())[:4]
            if ref is None:
                ref = score
            row = {"n": n, "rows_per_lane": R, "warps_per_band": NW, "grid": ctx.plain_config(n, n)["grid"],
                   "ms": ms, "gcups": n * n / ms / 1e6, "ok": score == ref}
            rows.append(row)
            log(json.dumps(row))
    ctx.set_plain_config()
    ctx.close()
    return rows


def gen_plain_header(rows, path=TUNED_PLAIN_H):
    """Best shape per size as the table plain_auto_config reads (nearest size wins)."""
    best = {}
    for r in rows:
        if r["ok"] and (r["n"] not in best or r["gcups"] > best[r["n"]]["gcups"]):
            best[r["n"]] = r
    out = ["// gme_tuned_plain.h -- plain-path shape per table height, written by",
           "// gpumemefficient_gb300/tune.py (sweep_plain) from a sweep on GB300: edit distance",
           "// on square pairs.  plain_auto_config takes the entry whose n is nearest (in log",
           "// scale) to the pair's row count n2.",
           "#pragma once", "", "namespace gme {", "",
           "struct TunedPlain {", "  int n, rows_per_lane, warps_per_band;", "};", "",
           f"constexpr int TUNED_PLAIN = {len(best)};",
           "constexpr TunedPlain TUNED_PLAIN_TABLE[TUNED_PLAIN > 0 ? TUNED_PLAIN : 1] = {"]
    for n in sorted(best):
        r = best[n]
        out.append(f"    {{{n}, {r['rows_per_lane']}, {r['warps_per_band']}}},  // {r['gcups']:.0f} GCUPS")
    if not best:
        out.append("    {0, 4, 4},")
    out += ["};", "", "}  // namespace gme", ""]
    with open(path, "w") as f:
        f.write("\n".join(out))
    return best


def write_plain_md(rows, best, path, cmd):
    lines = ["# Plain-path autotune sweep (edit distance, n x n)", "", f"Command (GB300): `{cmd}`", "",
             "One call per shape, CUDA-event time, mean of the repetitions; grid = one CTA per band "
             "up to the SM count.  Every shape's score equals the first shape's.", "",
             "| n | rows/lane | warps/band | grid | ms | GCUPS | |", "|---:|---:|---:|---:|---:|---:|---|"]
    for r in rows:
        mark = "best" if best.get(r["n"]) == r else ("" if r["ok"] else "MISMATCH")
        lines.append(f"| {r['n']} | {r['rows_per_lane']} | {r['warps_per_band']} | {r['grid']} | "
                     f"{r['ms']:.3f} | {r['gcups']:.1f} | {mark} |")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--out-json", default=TUNED_JSON)
    p.add_argument("--out-md", default=None)
    p.add_argument("--quick", action="store_true")
    p.add_argument("--cells", type=float, default=1.5e10)
    p.add_argument("--reps", type=int, default=5)
    p.add_argument("--header", action="store_true", help="also regenerate csrc/gme_tuned.h")
    p.add_argument("--plain", action="store_true",
                   help="sweep the plain path instead (writes csrc/gme_tuned_plain.h with --header)")
    a = p.parse_args()
    t0 = time.time()
    if a.plain:
        rows = sweep_plain()
        best = gen_plain_header(rows) if a.header else {}
        if a.out_md:
            if not best:
                best = {}
                for r in rows:
                    if r["ok"] and (r["n"] not in best or r["gcups"] > best[r["n"]]["gcups"]):
                        best[r["n"]] = r
            write_plain_md(rows, best, a.out_md, "python -m gpumemefficient_gb300.tune --plain --header "
                           f"--out-md {a.out_md}")
        with open(a.out_json, "w") as f:
            json.dump({"plain_rows": rows, "seconds": time.time() - t0}, f, indent=1)
        return
    rows = sweep(QUICK_GRID if a.quick else GRID, a.cells, a.reps)
    best = winners(rows)
    with open(a.out_json, "w") as f:
        json.dump({"best": best, "rows": rows, "seconds": time.time() - t0}, f, indent=1)
    if a.out_md:
        write_md(rows, best, a.out_md, "python -m gpumemefficient_gb300.tune" + (" --quick" if a.quick else "")
                 + f" --out-md {a.out_md}")
    if a.header:
        gen_header(best)
    print(json.dumps({k: {"gcups": v["gcups"], **{kk: v.get(kk) for kk in GRID}} for k, v in best.items()}))


if __name__ == "__main__":
    main()
