"""Seeded synthetic inputs with the benchmark shapes (no public dataset is involved).

The reference draws its inputs with rand()%4 and an unseeded srand(time(NULL))
(EditDistance/generator.cpp:35-40), so its runs are not reproducible; these
generators keep the same alphabets and lengths and fix the seeds.
"""
from __future__ import annotations

import numpy as np

SEED_LCS = 0x9E3779B9
SEED_ED = 0x9E3779BA
SEED_SW = 0x9E3779BB
SEED_BATCH = 0x9E3779BC
SEED_SERVE = 0x9E3779BD


def uniform(n: int, alphabet: int, rng) -> np.ndarray:
    return rng.integers(0, alphabet, n, dtype=np.int64).astype(np.int32)


def lcs_pair(n: int = 8192, seed: int = SEED_LCS):
    """Two i.i.d. uniform sequences over {0,1,2,3}."""
    rng = np.random.default_rng(seed)
    return uniform(n, 4, rng), uniform(n, 4, rng)


def mutate(a: np.ndarray, rate: float, alphabet: int, rng, kinds=("sub", "ins", "del")) -> np.ndarray:
    """Random edits at `rate` per position, equal mix of the given kinds."""
    out = []
    which = rng.integers(0, len(kinds), len(a))
    hit = rng.random(len(a)) < rate
    for i, s in enumerate(a.tolist()):
        if not hit[i]:
            out.append(s)
            continue
        k = kinds[which[i]]
        if k == "sub":
            out.append((s + int(rng.integers(1, alphabet))) % alphabet)
        elif k == "ins":
            out.append(int(rng.integers(0, alphabet)))
            out.append(s)
        # "del": drop s
    return np.asarray(out, np.int32)


def ed_pair(n: int = 65536, rate: float = 0.10, seed: int = SEED_ED):
    """a uniform over 4 symbols; b = a with seeded edits (sub/ins/del equally), cut or padded to n."""
    rng = np.random.default_rng(seed)
    a = uniform(n, 4, rng)
    b = mutate(a, rate, 4, rng)
    if len(b) >= n:
        b = b[:n]
    else:
        b = np.concatenate([b, uniform(n - len(b), 4, rng)])
    return a, b.astype(np.int32)


def sw_pair(n: int = 32768, alphabet: int = 20, seg: int = 2048, rate: float = 0.15,
            seed: int = SEED_SW):
    """Uniform 20-symbol sequences with one shared segment planted at random offsets,
    mutated (substitutions) at `rate` in the second copy."""
    rng = np.random.default_rng(seed)
    a = uniform(n, alphabet, rng)
    b = uniform(n, alphabet, rng)
    s = uniform(seg, alphabet, rng)
    oa = int(rng.integers(0, n - seg))
    ob = int(rng.integers(0, n - seg))
    a[oa:oa + seg] = s
    b[ob:ob + seg] = mutate(s, rate, alphabet, rng, kinds=("sub",))
    return a, b


def batch_pairs(npairs: int = 16384, lo: int = 64, hi: int = 4096, alphabet: int = 4,
                seed: int = SEED_BATCH):
    """Pairs with each length log-uniform in [lo, hi], kinds LCS/ED/SW one third each."""
    rng = np.random.default_rng(seed)
    la = np.exp(rng.uniform(np.log(lo), np.log(hi), npairs)).astype(np.int64)
    lb = np.exp(rng.uniform(np.log(lo), np.log(hi), npairs)).astype(np.int64)
    kinds = np.repeat(np.arange(3, dtype=np.int32), (npairs + 2) // 3)[:npairs]
    rng.shuffle(kinds)
    seqs_a = [uniform(int(n), alphabet, rng) for n in la]
    seqs_b = [uniform(int(n), alphabet, rng) for n in lb]
    return kinds, seqs_a, seqs_b


def served_requests(n: int = 8192, lo: int = 32, hi: int = 16384, alphabet: int = 4,
                    seed: int = SEED_SERVE):
    """Request stream of the served workload: half edit distance, half Smith-Waterman,
    each length log-uniform in [lo, hi], symbols uniform.  Returns (symbols, pairs)
    with pairs a PAIR_DTYPE array over the one symbol buffer (request order = arrival order)."""
    from . import PAIR_DTYPE
    rng = np.random.default_rng(seed)
    la = np.exp(rng.uniform(np.log(lo), np.log(hi), n)).astype(np.int64)
    lb = np.exp(rng.uniform(np.log(lo), np.log(hi), n)).astype(np.int64)
    kinds = np.repeat(np.array([1, 2], np.int32), (n + 1) // 2)[:n]
    rng.shuffle(kinds)
    lens = np.stack([la, lb], 1).reshape(-1)
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]])
    symbols = rng.integers(0, alphabet, int(lens.sum()), dtype=np.int64).astype(np.int32)
    pairs = np.zeros(n, PAIR_DTYPE)
    pairs["a_off"] = offs[0::2]
    pairs["b_off"] = offs[1::2]
    pairs["n1"] = la
    pairs["n2"] = lb
    pairs["kind"] = kinds
    return symbols, pairs
