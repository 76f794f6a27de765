"""GB300 wavefront alignment DP (LCS / edit distance / Smith-Waterman).

Python host side of ``libgme.so`` (the C ABI in ``include/gme.h``).  It mirrors
the reference's host functions -- ``LCS``, ``ED`` and ``SW`` taking two integer
sequences and returning the bottom-right cell (LCS/GPU_Hyperlane_Share.h:5,
EditDistance/GPU_Hyperlane_Share.h:5, SmithWaterman/GPU_Hyperlane_Share.h:5) --
and adds the richer calls of the C ABI (last row/column, SW maximum and its
cell, device-pointer entry points, batched and served forms).

There is no CPU fallback: importing this package without the built library
raises, and every call runs on the GPU.
"""
from __future__ import annotations

import ctypes
import os
import threading
from dataclasses import dataclass
from typing import Optional

import numpy as np

LCS_KIND, ED_KIND, SW_KIND = 0, 1, 2
ED_REF_CPU, ED_STANDARD = 0, 1
KINDS = {"lcs": LCS_KIND, "ed": ED_KIND, "sw": SW_KIND}

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgme.so")

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of memory",
          4: "device wait timed out", 5: "sizes could overflow int32 scores",
          6: "request exceeds the HBM budget", 7: "not ready", 8: "server closed"}


class GmeError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}" + (f": {msg}" if msg else ""))


class Scoring(ctypes.Structure):
    _fields_ = [("match", ctypes.c_int32), ("mismatch", ctypes.c_int32),
                ("gap", ctypes.c_int32), ("ed_boundary", ctypes.c_int32)]


class Result(ctypes.Structure):
    _fields_ = [("score", ctypes.c_int32), ("sw_max", ctypes.c_int32),
                ("sw_max_y", ctypes.c_int64), ("sw_max_x", ctypes.c_int64),
                ("status", ctypes.c_int32), ("kind", ctypes.c_int32)]


class Pair(ctypes.Structure):
    _fields_ = [("a_off", ctypes.c_int64), ("b_off", ctypes.c_int64), ("n1", ctypes.c_int32),
                ("n2", ctypes.c_int32), ("kind", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class BatchConfig(ctypes.Structure):
    _fields_ = [("warps_per_block", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32),
                ("block_min_cells", ctypes.c_int64), ("long_min_cells", ctypes.c_int64),
                ("team_min_cells", ctypes.c_int64), ("packed16", ctypes.c_int32),
                ("team_split", ctypes.c_int32), ("rows_per_lane", ctypes.c_int32)]


PAIR_DTYPE = np.dtype([("a_off", "<i8"), ("b_off", "<i8"), ("n1", "<i4"), ("n2", "<i4"),
                       ("kind", "<i4"), ("reserved", "<i4")])
RESULT_DTYPE = np.dtype([("score", "<i4"), ("sw_max", "<i4"), ("sw_max_y", "<i8"),
                         ("sw_max_x", "<i8"), ("status", "<i4"), ("kind", "<i4")])


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_int64), ("wave_max_cells", ctypes.c_int64),
                ("waves", ctypes.c_int32), ("queue_max", ctypes.c_int32),
                ("warps_per_block", ctypes.c_int32), ("mode", ctypes.c_int32)]


SERVE_RING, SERVE_WAVES = 0, 1
BASELINE_TILES, BASELINE_CELLS = 0, 1


class ServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in (
        "submitted", "completed", "queued", "running", "waves_launched", "kernels_launched",
        "cells_completed", "hbm_bytes_held", "hbm_bytes_peak", "hbm_budget_bytes", "h2d_bytes",
        "d2h_bytes")]


class PlainConfig(ctypes.Structure):
    _fields_ = [("rows_per_lane", ctypes.c_int32), ("warps_per_band", ctypes.c_int32),
                ("grid", ctypes.c_int32), ("reserved", ctypes.c_int32)]


_i32p = ctypes.POINTER(ctypes.c_int32)
_vp = ctypes.c_void_p
_lib = None
_lib_lock = threading.Lock()


def _declare(L):
    c = ctypes
    L.gme_create.argtypes = [c.c_int, c.POINTER(c.c_void_p)]
    L.gme_destroy.argtypes = [_vp]
    L.gme_last_error.argtypes = [_vp]
    L.gme_last_error.restype = c.c_char_p
    L.gme_status_string.restype = c.c_char_p
    L.gme_default_scoring.restype = Scoring
    L.gme_set_wait_timeout_ns.argtypes = [_vp, c.c_uint64]
    L.gme_set_plain_config.argtypes = [_vp, c.POINTER(PlainConfig)]
    L.gme_get_plain_config.argtypes = [_vp, c.c_int64, c.c_int64, c.POINTER(PlainConfig)]
    L.gme_align.argtypes = [_vp, c.c_int, _vp, c.c_int64, _vp, c.c_int64, c.POINTER(Scoring),
                            c.POINTER(Result), _vp, _vp]
    L.gme_align_device.argtypes = [_vp, c.c_int, _vp, c.c_int64, _vp, c.c_int64,
                                   c.POINTER(Scoring), _vp, _vp, _vp, _vp]
    L.gme_set_batch_config.argtypes = [_vp, c.POINTER(BatchConfig)]
    L.gme_align_batch.argtypes = [_vp, _vp, c.c_int64, _vp, c.c_int64, c.POINTER(Scoring), _vp]
    L.gme_align_batch_device.argtypes = [_vp, _vp, c.c_int64, _vp, c.c_int64, c.POINTER(Scoring),
                                         _vp, _vp]
    L.gme_align_batch_device_rows.argtypes = [_vp, _vp, c.c_int64, _vp, c.c_int64, c.POINTER(Scoring), _vp,
                                              _vp, _vp, _vp, _vp, _vp]
    L.gme_batch_stats.argtypes = [_vp, c.POINTER(c.c_int64), c.POINTER(c.c_int64),
                                  c.POINTER(c.c_int64), c.POINTER(c.c_int64)]
    L.gme_batch_plan_create.argtypes = [_vp, _vp, c.c_int64, c.c_int64, c.POINTER(c.c_void_p)]
    L.gme_batch_plan_run.argtypes = [_vp, _vp, c.POINTER(Scoring), _vp, _vp, c.c_int]
    L.gme_batch_plan_destroy.argtypes = [_vp]
    L.gme_server_create.argtypes = [c.c_int, c.POINTER(ServerConfig), c.POINTER(Scoring),
                                    c.POINTER(c.c_void_p)]
    L.gme_server_destroy.argtypes = [_vp]
    L.gme_submit.argtypes = [_vp, c.c_int, _vp, c.c_int64, _vp, c.c_int64, c.POINTER(c.c_uint64)]
    L.gme_submit_many.argtypes = [_vp, _vp, _vp, c.c_int64, _vp, c.POINTER(c.c_int64)]
    L.gme_poll.argtypes = [_vp, c.c_uint64, c.POINTER(Result), c.POINTER(c.c_int64)]
    L.gme_poll_many.argtypes = [_vp, _vp, _vp, _vp, c.c_int64, c.POINTER(c.c_int64)]
    L.gme_server_drain.argtypes = [_vp, c.c_uint64]
    L.gme_server_get_stats.argtypes = [_vp, c.POINTER(ServerStats)]
    L.gme_server_last_error.argtypes = [_vp]
    L.gme_server_last_error.restype = c.c_char_p
    L.gme_batch_tuned_config.argtypes = [_vp, c.c_int64, c.POINTER(BatchConfig)]
    L.gme_sat_device.argtypes = [_vp, _vp, c.c_int64, c.c_int64, c.c_int64, _vp, _vp]
    L.gme_sat.argtypes = [_vp, _vp, c.c_int64, c.c_int64, c.c_int64]
    L.gme_align_path.argtypes = [_vp, c.c_int, _vp, c.c_int64, _vp, c.c_int64, c.POINTER(Scoring), _vp,
                                 c.c_int64, c.POINTER(c.c_int64), c.POINTER(c.c_int32)]
    L.gme_debug_wait_timeout.argtypes = [_vp, c.c_uint64, c.POINTER(c.c_int32)]
    L.gme_baseline_align_device.argtypes = [_vp, c.c_int32, c.c_int32, _vp, c.c_int64, _vp, c.c_int64, _vp, _vp,
                                            c.c_int32, c.c_int32, _vp, _vp]
    L.gme_launch_count.argtypes = [_vp]
    L.gme_launch_count.restype = c.c_int64
    for name in ("gme_ref_lcs", "gme_ref_ed", "gme_ref_sw"):
        f = getattr(L, name)
        f.argtypes = [c.c_int32, c.c_int32, _vp, _vp]
        f.restype = c.c_int32
    return L


def lib():
    """The loaded libgme.so (raises if it has not been built)."""
    global _lib
    with _lib_lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(f"libgme.so not built ({LIB_PATH}); run __graft_entry__.build()")
            _lib = _declare(ctypes.CDLL(LIB_PATH))
    return _lib


def _check(status: int, ctx=None):
    if status != 0:
        msg = lib().gme_last_error(ctx).decode() if ctx else ""
        raise GmeError(status, msg)


def scoring(match: int = 3, mismatch: int = -3, gap: int = -2,
            ed_boundary: int = ED_REF_CPU) -> Scoring:
    """Scoring constants; the defaults are SmithWaterman/SW.cpp:45-47,63-65 and ED.cpp's border."""
    return Scoring(match, mismatch, gap, ed_boundary)


@dataclass
class AlignResult:
    score: int
    sw_max: int = 0
    sw_max_y: int = 0
    sw_max_x: int = 0
    last_row: Optional[np.ndarray] = None
    last_col: Optional[np.ndarray] = None


class Context:
    """A device, its stream and a reusable workspace (one host thread at a time)."""

    def __init__(self, device: int = 0):
        h = ctypes.c_void_p()
        _check(lib().gme_create(device, ctypes.byref(h)))
        self.handle = h
        self.device = device

    def close(self):
        if getattr(self, "handle", None):
            lib().gme_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def launches(self) -> int:
        return int(lib().gme_launch_count(self.handle))

    def set_timeout_ns(self, ns: int):
        _check(lib().gme_set_wait_timeout_ns(self.handle, ns), self.handle)

    def set_plain_config(self, rows_per_lane: int = 0, warps_per_band: int = 0, grid: int = 0):
        cfg = PlainConfig(rows_per_lane, warps_per_band, grid, 0)
        _check(lib().gme_set_plain_config(self.handle, ctypes.byref(cfg)), self.handle)

    def plain_config(self, n1: int, n2: int) -> dict:
        cfg = PlainConfig()
        _check(lib().gme_get_plain_config(self.handle, n1, n2, ctypes.byref(cfg)), self.handle)
        return {"rows_per_lane": cfg.rows_per_lane, "warps_per_band": cfg.warps_per_band,
                "grid": cfg.grid}

    def align(self, kind, a, b, sc: Optional[Scoring] = None, last_row: bool = False,
              last_col: bool = False) -> AlignResult:
        """One alignment from host arrays (the reference host functions' contract)."""
        kind = KINDS.get(kind, kind) if isinstance(kind, str) else kind
        a = np.ascontiguousarray(a, dtype=np.int32)
        b = np.ascontiguousarray(b, dtype=np.int32)
        sc = sc or scoring()
        res = Result()
        lr = np.empty(len(a) + 1, np.int32) if last_row else None
        lc = np.empty(len(b) + 1, np.int32) if last_col else None
        st = lib().gme_align(self.handle, kind, a.ctypes.data, len(a), b.ctypes.data, len(b),
                             ctypes.byref(sc), ctypes.byref(res),
                             lr.ctypes.data if lr is not None else None,
                             lc.ctypes.data if lc is not None else None)
        _check(st, self.handle)
        return AlignResult(res.score, res.sw_max, res.sw_max_y, res.sw_max_x, lr, lc)

    def align_device(self, kind, d_a: int, n1: int, d_b: int, n2: int, d_out: int,
                     sc: Optional[Scoring] = None, d_last_row: int = 0, d_last_col: int = 0,
                     stream: int = 0):
        """Asynchronous alignment on device pointers; d_out points to a device gme_result."""
        sc = sc or scoring()
        _check(lib().gme_align_device(self.handle, kind, d_a, n1, d_b, n2, ctypes.byref(sc),
                                      d_out, d_last_row or None, d_last_col or None,
                                      stream or None), self.handle)

    def set_batch_config(self, warps_per_block: int = 0, blocks_per_sm: int = 0,
                         block_min_cells: int = 0, long_min_cells: int = 0, team_min_cells: int = 0,
                         packed16: int = 0, team_split: int = 0, rows_per_lane: int = 0):
        cfg = BatchConfig(warps_per_block, blocks_per_sm, block_min_cells, long_min_cells, team_min_cells,
                          int(packed16), team_split, rows_per_lane)
        _check(lib().gme_set_batch_config(self.handle, ctypes.byref(cfg)), self.handle)

    def batch_stats(self) -> dict:
        b, w, l, t = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _check(lib().gme_batch_stats(self.handle, ctypes.byref(b), ctypes.byref(w), ctypes.byref(l),
                                     ctypes.byref(t)))
        return {"block_jobs": b.value, "warp_jobs": w.value, "long_jobs": l.value, "team_jobs": t.value}

    def align_batch(self, kinds, seqs_a, seqs_b, sc: Optional[Scoring] = None) -> np.ndarray:
        """Many alignments in one launch; returns a structured array of results."""
        symbols, pairs = pack_batch(kinds, seqs_a, seqs_b)
        res = np.zeros(len(pairs), RESULT_DTYPE)
        sc = sc or scoring()
        _check(lib().gme_align_batch(self.handle, symbols.ctypes.data, len(symbols),
                                     pairs.ctypes.data, len(pairs), ctypes.byref(sc),
                                     res.ctypes.data), self.handle)
        return res

    def align_batch_device_rows(self, d_symbols: int, nsym: int, pairs: np.ndarray, d_results: int,
                                d_last_rows: int = 0, row_offsets=None, d_last_cols: int = 0,
                                col_offsets=None, sc: Optional[Scoring] = None, stream: int = 0):
        """Device batch with each pair's last row/column written at the given element offsets."""
        pairs = np.ascontiguousarray(pairs, PAIR_DTYPE)
        ro = np.ascontiguousarray(row_offsets, np.int64) if row_offsets is not None else None
        co = np.ascontiguousarray(col_offsets, np.int64) if col_offsets is not None else None
        sc = sc or scoring()
        _check(lib().gme_align_batch_device_rows(
            self.handle, d_symbols, nsym, pairs.ctypes.data, len(pairs), ctypes.byref(sc), d_results,
            d_last_rows or None, ro.ctypes.data if ro is not None else None, d_last_cols or None,
            co.ctypes.data if co is not None else None, stream or None), self.handle)

    def align_batch_device(self, d_symbols: int, nsym: int, pairs: np.ndarray, d_results: int,
                           sc: Optional[Scoring] = None, stream: int = 0):
        """Device symbols/results, host pair list (a PAIR_DTYPE array); asynchronous."""
        pairs = np.ascontiguousarray(pairs, PAIR_DTYPE)
        sc = sc or scoring()
        _check(lib().gme_align_batch_device(self.handle, d_symbols, nsym, pairs.ctypes.data,
                                            len(pairs), ctypes.byref(sc), d_results,
                                            stream or None), self.handle)

    def align_path(self, kind, a, b):
        """(score, edit script) of an optimal global alignment: 'M' a[i]~b[j], 'D' a[i]~gap,
        'I' gap~b[j].  LCS, or ED with the standard border."""
        kind = KINDS.get(kind, kind) if isinstance(kind, str) else kind
        a = np.ascontiguousarray(a, dtype=np.int32)
        b = np.ascontiguousarray(b, dtype=np.int32)
        cap = len(a) + len(b)
        buf = ctypes.create_string_buffer(max(cap, 1))
        n = ctypes.c_int64()
        sc_ = ctypes.c_int32()
        scoring_ = scoring(ed_boundary=ED_STANDARD)
        _check(lib().gme_align_path(self.handle, kind, a.ctypes.data, len(a), b.ctypes.data, len(b),
                                    ctypes.byref(scoring_), buf, cap, ctypes.byref(n), ctypes.byref(sc_)),
               self.handle)
        return sc_.value, buf.raw[:n.value].decode()

    def sat(self, table, n1: int, n2: int) -> np.ndarray:
        """Summed-area table (``gme_sat``) of a host int32 table of rows 0..n2 (row length
        >= n1 + 1; the reference's layout has n1 + 3): rows 1..n2 x columns 1..n1 are
        rewritten in place; returns the table."""
        t = table if isinstance(table, np.ndarray) and table.dtype == np.int32 and \
            table.flags.c_contiguous else np.ascontiguousarray(table, dtype=np.int32)
        assert t.ndim == 2 and t.shape[0] >= n2 + 1 and t.shape[1] >= n1 + 1
        _check(lib().gme_sat(self.handle, t.ctypes.data, n1, n2, t.shape[1]), self.handle)
        return t

    def sat_device(self, d_table: int, n1: int, n2: int, ld: int, d_status: int = 0, stream: int = 0):
        """``gme_sat_device``: in place on a device table, asynchronous on ``stream``."""
        _check(lib().gme_sat_device(self.handle, d_table, n1, n2, ld, d_status or None, stream or None),
               self.handle)

    def baseline_align_device(self, strategy: int, kind: int, d_a: int, n1: int, d_b: int, n2: int, d_table: int,
                              d_out: int, tile_x: int = 64, tile_y: int = 128, sc: Optional[Scoring] = None,
                              stream: int = 0):
        """A comparison baseline (not the product path): the whole table in d_table,
        BASELINE_TILES (one launch per anti-diagonal of tiles) or BASELINE_CELLS (one
        launch per anti-diagonal of cells); the result (gme_result) at d_out."""
        sc = sc or scoring()
        _check(lib().gme_baseline_align_device(self.handle, strategy, kind, d_a, n1, d_b, n2, ctypes.byref(sc),
                                               d_table, tile_x, tile_y, d_out, stream), self.handle)

    def debug_wait_timeout(self, timeout_ns: int) -> int:
        """Runs a bounded device wait on a flag nothing sets; returns the kernel's status."""
        ks = ctypes.c_int32(-1)
        _check(lib().gme_debug_wait_timeout(self.handle, timeout_ns, ctypes.byref(ks)), self.handle)
        return int(ks.value)


class BatchPlan:
    """A planned batch (fixed pair list) that can be run many times, optionally as a CUDA graph."""

    def __init__(self, ctx: "Context", pairs: np.ndarray, nsym: int):
        self.ctx = ctx
        self.pairs = np.ascontiguousarray(pairs, PAIR_DTYPE)
        h = ctypes.c_void_p()
        _check(lib().gme_batch_plan_create(ctx.handle, self.pairs.ctypes.data, len(self.pairs), nsym,
                                           ctypes.byref(h)), ctx.handle)
        self.handle = h

    def run(self, d_symbols: int, d_results: int, sc: Optional[Scoring] = None, stream: int = 0,
            use_graph: bool = False):
        sc = sc or scoring()
        _check(lib().gme_batch_plan_run(self.handle, d_symbols, ctypes.byref(sc), d_results,
                                        stream or None, int(use_graph)), self.ctx.handle)

    def close(self):
        if getattr(self, "handle", None):
            lib().gme_batch_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """The served path: submit alignments one at a time, collect each as it finishes.

    A native dispatcher thread admits queued requests against the HBM budget.  In ring
    mode (the default) a persistent kernel takes them from device-resident job rings as
    they are published; in waves mode they run as launches of the batched kernel on
    several streams.  Results and completion flags come back through pinned host memory
    (``include/gme.h``, served path).
    """

    NOT_READY = 7

    def __init__(self, device: int = 0, sc: Optional[Scoring] = None, hbm_budget_bytes: int = 0,
                 wave_max_cells: int = 0, waves: int = 0, queue_max: int = 0,
                 warps_per_block: int = 0, mode: int = SERVE_RING):
        cfg = ServerConfig(hbm_budget_bytes, wave_max_cells, waves, queue_max, warps_per_block, mode)
        self.sc = sc or scoring()
        h = ctypes.c_void_p()
        _check(lib().gme_server_create(device, ctypes.byref(cfg), ctypes.byref(self.sc),
                                       ctypes.byref(h)))
        self.handle = h

    def _err(self, st):
        if st != 0:
            raise GmeError(st, lib().gme_server_last_error(self.handle).decode())

    def submit(self, kind, a, b) -> int:
        """Queues one alignment; returns its ticket (a and b are copied)."""
        kind = KINDS.get(kind, kind) if isinstance(kind, str) else kind
        a = np.ascontiguousarray(a, dtype=np.int32)
        b = np.ascontiguousarray(b, dtype=np.int32)
        t = ctypes.c_uint64()
        self._err(lib().gme_submit(self.handle, int(kind), a.ctypes.data, len(a), b.ctypes.data,
                                   len(b), ctypes.byref(t)))
        return t.value

    def submit_many(self, symbols: np.ndarray, pairs: np.ndarray) -> np.ndarray:
        """Queues alignments (PAIR_DTYPE over one int32 symbol buffer); returns the tickets
        of those queued: all of them, or a prefix when the queue is full (the caller
        submits the rest later)."""
        symbols = np.ascontiguousarray(symbols, np.int32)
        pairs = np.ascontiguousarray(pairs, PAIR_DTYPE)
        tickets = np.zeros(len(pairs), np.uint64)
        k = ctypes.c_int64()
        st = lib().gme_submit_many(self.handle, symbols.ctypes.data, pairs.ctypes.data, len(pairs),
                                   tickets.ctypes.data, ctypes.byref(k))
        if st != self.NOT_READY:
            self._err(st)
        return tickets[:k.value]

    def poll(self, ticket: int):
        """(result dict, latency_ns) once done, else None."""
        r = Result()
        lat = ctypes.c_int64()
        st = lib().gme_poll(self.handle, ticket, ctypes.byref(r), ctypes.byref(lat))
        if st == self.NOT_READY:
            return None
        self._err(st)
        return ({"score": r.score, "sw_max": r.sw_max, "sw_max_y": r.sw_max_y,
                 "sw_max_x": r.sw_max_x, "status": r.status, "kind": r.kind}, lat.value)

    def poll_many(self, max_n: int = 65536):
        """(tickets, RESULT_DTYPE results, latencies in ns) of requests finished since the last call."""
        tickets = np.zeros(max_n, np.uint64)
        res = np.zeros(max_n, RESULT_DTYPE)
        lat = np.zeros(max_n, np.int64)
        n = ctypes.c_int64()
        self._err(lib().gme_poll_many(self.handle, tickets.ctypes.data, res.ctypes.data,
                                      lat.ctypes.data, max_n, ctypes.byref(n)))
        k = n.value
        return tickets[:k], res[:k], lat[:k]

    def drain(self, timeout_s: float = 600.0) -> bool:
        st = lib().gme_server_drain(self.handle, int(timeout_s * 1e9))
        if st == self.NOT_READY:
            return False
        self._err(st)
        return True

    def stats(self) -> dict:
        s = ServerStats()
        self._err(lib().gme_server_get_stats(self.handle, ctypes.byref(s)))
        return {n: getattr(s, n) for n, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "handle", None):
            lib().gme_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def batch_tuned_config(pairs: np.ndarray) -> dict:
    """The autotuned settings a batch of these pairs (PAIR_DTYPE; only n1, n2 matter) is
    planned with when no configuration is set (``gme_batch_tuned_config``; no GPU needed)."""
    pairs = np.ascontiguousarray(pairs, PAIR_DTYPE)
    cfg = BatchConfig()
    _check(lib().gme_batch_tuned_config(pairs.ctypes.data, len(pairs), ctypes.byref(cfg)))
    return {n: getattr(cfg, n) for n, _ in BatchConfig._fields_}


def pack_batch(kinds, seqs_a, seqs_b):
    """One int32 symbol buffer plus a PAIR_DTYPE pair list for the batched entry points."""
    parts, pairs = [], np.zeros(len(kinds), PAIR_DTYPE)
    off = 0
    for i, (k, a, b) in enumerate(zip(kinds, seqs_a, seqs_b)):
        a = np.asarray(a, np.int32)
        b = np.asarray(b, np.int32)
        pairs[i] = (off, off + len(a), len(a), len(b), int(k), 0)
        parts += [a, b]
        off += len(a) + len(b)
    symbols = np.ascontiguousarray(np.concatenate(parts) if parts else np.zeros(1, np.int32), np.int32)
    return symbols, pairs


_default_ctx: Optional[Context] = None
_default_lock = threading.Lock()


def default_context() -> Context:
    global _default_ctx
    with _default_lock:
        if _default_ctx is None:
            _default_ctx = Context(0)
    return _default_ctx


def align(kind, a, b, **kw) -> AlignResult:
    sc_keys = {k: kw.pop(k) for k in ("match", "mismatch", "gap", "ed_boundary") if k in kw}
    return default_context().align(kind, a, b, sc=scoring(**sc_keys) if sc_keys else None, **kw)


# --- the reference's host functions (same names, argument meaning and result) ----------

def _ref_call(kind, n1, n2, arr1, arr2):
    a = np.ascontiguousarray(arr1, dtype=np.int32)[:n1]
    b = np.ascontiguousarray(arr2, dtype=np.int32)[:n2]
    if len(a) != n1 or len(b) != n2:
        raise GmeError(1, "arrays shorter than n1/n2")
    sc = scoring(ed_boundary=ED_STANDARD)  # the GPU reference's GPU_setInit border
    return default_context().align(kind, a, b, sc=sc).score


def LCS(n1, n2, arr1, arr2, paddX=3, paddY=1, table=None, tX=None, tY=None) -> int:
    """LCS/GPU_Hyperlane_Share.h:5 -- length of the longest common subsequence."""
    return _ref_call(LCS_KIND, n1, n2, arr1, arr2)


def ED(n1, n2, arr1, arr2, paddX=3, paddY=1, table=None, tX=None, tY=None) -> int:
    """EditDistance/GPU_Hyperlane_Share.h:5 -- edit distance (GPU_setInit border)."""
    return _ref_call(ED_KIND, n1, n2, arr1, arr2)


def SW(n1, n2, arr1, arr2, paddX=3, paddY=1, table=None, tX=None, tY=None) -> int:
    """SmithWaterman/GPU_Hyperlane_Share.h:5 -- bottom-right cell of the SW table."""
    return _ref_call(SW_KIND, n1, n2, arr1, arr2)
