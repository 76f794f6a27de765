"""CPU oracle for the alignment recurrences -- TEST INFRASTRUCTURE ONLY.

This module is the checker the CUDA path is compared against.  Only tests/,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline legs may import it;
the product package never does.

It wraps ``oracle.c`` (a C restatement of LCS/LCS.cpp:45-82,
EditDistance/ED.cpp:45-80 and SmithWaterman/SW.cpp:45-83 with rolling rows and
64-bit indices) through ctypes, and carries a second, independent pure-Python
restatement (``table_py``) used only to cross-check the C code on tiny inputs.

Convention: columns x = 0..n1 run over ``a`` (the reference's arr1), rows
y = 0..n2 run over ``b`` (arr2); cell (y, x) compares a[x-1] with b[y-1].
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

LCS, ED, SW = 0, 1, 2
ED_REF_CPU, ED_STANDARD = 0, 1
SW_MATCH, SW_MISMATCH, SW_GAP = 3, -3, -2  # SmithWaterman/SW.cpp:45-47, :63-65

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "oracle.c")
_OUT = os.path.join(_HERE, "_build", "liboracle.so")
_lock = threading.Lock()
_lib = None

_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)


def build(force: bool = False) -> str:
    """Compile oracle.c into oracle/_build/liboracle.so (gcc, portable flags)."""
    if force or not os.path.exists(_OUT) or os.path.getmtime(_OUT) < os.path.getmtime(_SRC):
        os.makedirs(os.path.dirname(_OUT), exist_ok=True)
        tmp = _OUT + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-shared", "-fPIC", "-pthread",
                               _SRC, "-o", tmp])
        os.replace(tmp, _OUT)
    return _OUT


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = ctypes.CDLL(build())
            L.orc_align.restype = ctypes.c_int32
            L.orc_align.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, ctypes.c_int64, _i32p,
                                    ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                    _i32p, _i32p, _i32p, _i64p, _i64p]
            L.orc_align_mt.restype = ctypes.c_int32
            L.orc_align_mt.argtypes = L.orc_align.argtypes + [ctypes.c_int, ctypes.c_int64,
                                                              ctypes.c_int64]
            L.orc_table.restype = None
            L.orc_table.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, ctypes.c_int64, _i32p,
                                    ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                    _i32p]
            L.orc_align_batch_mt.restype = None
            L.orc_align_batch_mt.argtypes = [_i32p, _i32p, _i64p, _i64p, _i64p, _i64p,
                                             ctypes.c_int64, ctypes.c_int, ctypes.c_int32,
                                             ctypes.c_int32, ctypes.c_int32, _i32p, _i32p, _i64p,
                                             _i64p, ctypes.c_int]
            L.orc_sat.restype = None
            L.orc_sat.argtypes = [_i32p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64]
            L.orc_sat_mt.restype = None
            L.orc_sat_mt.argtypes = [_i32p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int]
            _lib = L
    return _lib


def _p32(x):
    return x.ctypes.data_as(_i32p) if x is not None else None


def _p64(x):
    return x.ctypes.data_as(_i64p) if x is not None else None


def align(kind: int, a, b, rule: int = ED_REF_CPU, match: int = SW_MATCH,
          mismatch: int = SW_MISMATCH, gap: int = SW_GAP, threads: int = 1,
          band_rows: int = 256, chunk_cols: int = 1024) -> dict:
    """Score, last row, last column (and SW max/cell) of one alignment."""
    a = np.ascontiguousarray(a, dtype=np.int32)
    b = np.ascontiguousarray(b, dtype=np.int32)
    n1, n2 = len(a), len(b)
    last_row = np.empty(n1 + 1, np.int32)
    last_col = np.empty(n2 + 1, np.int32)
    m = np.zeros(1, np.int32)
    y = np.zeros(1, np.int64)
    x = np.zeros(1, np.int64)
    L = lib()
    if threads > 1:
        score = L.orc_align_mt(kind, rule, _p32(a), n1, _p32(b), n2, match, mismatch, gap,
                               _p32(last_row), _p32(last_col), _p32(m), _p64(y), _p64(x),
                               threads, band_rows, chunk_cols)
    else:
        score = L.orc_align(kind, rule, _p32(a), n1, _p32(b), n2, match, mismatch, gap,
                            _p32(last_row), _p32(last_col), _p32(m), _p64(y), _p64(x))
    return {"score": int(score), "last_row": last_row, "last_col": last_col,
            "sw_max": int(m[0]), "sw_y": int(y[0]), "sw_x": int(x[0])}


def table(kind: int, a, b, rule: int = ED_REF_CPU, match: int = SW_MATCH,
          mismatch: int = SW_MISMATCH, gap: int = SW_GAP) -> np.ndarray:
    """Full (n2+1) x (n1+1) DP table (tiny inputs only)."""
    a = np.ascontiguousarray(a, dtype=np.int32)
    b = np.ascontiguousarray(b, dtype=np.int32)
    t = np.empty((len(b) + 1, len(a) + 1), np.int32)
    lib().orc_table(kind, rule, _p32(a), len(a), _p32(b), len(b), match, mismatch, gap, _p32(t))
    return t


def align_batch(kinds, seqs_a, seqs_b, rule: int = ED_REF_CPU, match: int = SW_MATCH,
                mismatch: int = SW_MISMATCH, gap: int = SW_GAP, threads: int = 0) -> dict:
    """Many independent alignments across host threads (pairs claimed dynamically)."""
    n = len(kinds)
    parts, a_off, a_len, b_off, b_len = [], [], [], [], []
    off = 0
    for sa, sb in zip(seqs_a, seqs_b):
        sa = np.asarray(sa, np.int32)
        sb = np.asarray(sb, np.int32)
        a_off.append(off); a_len.append(len(sa)); parts.append(sa); off += len(sa)
        b_off.append(off); b_len.append(len(sb)); parts.append(sb); off += len(sb)
    seq = np.concatenate(parts) if parts else np.zeros(1, np.int32)
    kinds = np.ascontiguousarray(kinds, np.int32)
    a_off, a_len, b_off, b_len = (np.asarray(v, np.int64) for v in (a_off, a_len, b_off, b_len))
    score = np.zeros(n, np.int32)
    m = np.zeros(n, np.int32)
    y = np.zeros(n, np.int64)
    x = np.zeros(n, np.int64)
    threads = threads or os.cpu_count() or 1
    lib().orc_align_batch_mt(_p32(kinds), _p32(seq), _p64(a_off), _p64(a_len), _p64(b_off),
                             _p64(b_len), n, rule, match, mismatch, gap, _p32(score), _p32(m),
                             _p64(y), _p64(x), threads)
    return {"score": score, "sw_max": m, "sw_y": y, "sw_x": x}


def table_py(kind: int, a, b, rule: int = ED_REF_CPU, match: int = SW_MATCH,
             mismatch: int = SW_MISMATCH, gap: int = SW_GAP):
    """Independent pure-Python restatement (loops), for cross-checking tiny cases.

    Follows the reference CPU loops literally: LCS/LCS.cpp:47-64,
    EditDistance/ED.cpp:48-66, SmithWaterman/SW.cpp:51-66.
    """
    n1, n2 = len(a), len(b)
    w = n1 + 1
    t = [[0] * w for _ in range(n2 + 1)]
    if kind == ED:
        for x in range(w):
            t[0][x] = x if rule == ED_STANDARD else x - 1
        for y in range(n2 + 1):
            t[y][0] = y
    for y in range(1, n2 + 1):
        for x in range(1, w):
            eq = a[x - 1] == b[y - 1]
            up, left, diag = t[y - 1][x], t[y][x - 1], t[y - 1][x - 1]
            if kind == LCS:
                v = diag + 1 if eq else max(left, up)
            elif kind == ED:
                v = min(up + 1, min(left + 1, diag + 1))
                if eq:
                    v = diag
            else:
                v = max(left + gap, max(up + gap, max(diag + (match if eq else mismatch), 0)))
            t[y][x] = v
    return t


def sat(table, n1: int, n2: int):
    """Summed-area table of the reference's layout (rows 0..n2 of any row length
    >= n1 + 1), returned as a new int32 array: rows 1..n2 x columns 1..n1 follow the
    SAT recurrence (SAT/GPU_Hyperlane_Share.cu:169,196,231) in wrapping 32-bit
    arithmetic; everything else is copied."""
    t = np.ascontiguousarray(table, dtype=np.int32).copy()
    assert t.ndim == 2 and t.shape[0] >= n2 + 1 and t.shape[1] >= n1 + 1
    lib().orc_sat(_p32(t), n1, n2, t.shape[1])
    return t


def sat_mt(table, n1: int, n2: int, threads: int = 0):
    """``sat`` on all host threads (row prefixes, then column accumulation; the CPU
    baselines' form), bit-identical to ``sat``."""
    t = np.ascontiguousarray(table, dtype=np.int32).copy()
    assert t.ndim == 2 and t.shape[0] >= n2 + 1 and t.shape[1] >= n1 + 1
    lib().orc_sat_mt(_p32(t), n1, n2, t.shape[1], threads or os.cpu_count() or 1)
    return t


def sat_py(table, n1: int, n2: int):
    """Independent restatement for cross-checks: the closed form of the recurrence,
    t[y][x] = A[y][0] + A[0][x] - A[0][0] + sum_{1<=i<=y, 1<=j<=x} A[i][j] (mod 2^32),
    with numpy cumulative sums."""
    a = np.asarray(table, dtype=np.int64)
    out = np.array(table, dtype=np.int32, copy=True)
    if n1 == 0 or n2 == 0:
        return out
    inner = a[1:n2 + 1, 1:n1 + 1].cumsum(0).cumsum(1)
    v = inner + a[1:n2 + 1, 0:1] + a[0:1, 1:n1 + 1] - a[0, 0]
    out[1:n2 + 1, 1:n1 + 1] = (v & 0xffffffff).astype(np.uint32).view(np.int32)
    return out
