"""Seeded synthetic texts with the shapes of the benchmark configurations.

No public dataset backs these workloads; each generator is deterministic for
its seed (numpy PCG64) and documents the distribution it draws from.

  uniform_dna         n i.i.d. uniform symbols over {0,1,2,3}
  dna_with_repeats    uniform base over {0,1,2,3}; segments of log-uniform
                      length [lmin, lmax] copied from uniformly chosen earlier
                      offsets until `coverage` of the positions are covered,
                      each copied symbol substituted by a different uniform
                      symbol with probability `sub`
  segmented_filtered  lognormal segment lengths (median 2000, sigma 1.5), each
                      ending in separator 4, bodies uniform over {0..3}, 2% of
                      positions in runs of symbol 5 of uniform length
                      1000..50000 (separators kept); returns the text, the
                      segment ends and the positions whose symbol is < 4
  batched_texts       many texts with log-uniform lengths, each a
                      dna_with_repeats text; returns the concatenation and
                      the offsets
"""
from __future__ import annotations

import math

import numpy as np


def uniform_dna(n: int, seed: int = 1) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.integers(0, 4, n, dtype=np.uint8)


def _plant(rng, text, coverage, lmin, lmax, sub):
    n = len(text)
    if n < 2 * lmin:
        return text
    covered = np.zeros(n, dtype=bool)
    done = 0
    target = int(coverage * n)
    lo, hi = math.log(lmin), math.log(lmax)
    guard = 0
    while done < target and guard < 10_000_000:
        guard += 1
        L = int(math.exp(rng.uniform(lo, hi)))
        L = max(lmin, min(L, n // 2))
        dst = int(rng.integers(L, n - L + 1))
        src = int(rng.integers(0, dst - L + 1))
        seg = text[src:src + L].copy()
        flip = rng.random(L) < sub
        k = int(flip.sum())
        if k:
            seg[flip] = (seg[flip] + rng.integers(1, 4, k, dtype=np.uint8)) % 4
        text[dst:dst + L] = seg
        done += L - int(covered[dst:dst + L].sum())
        covered[dst:dst + L] = True
    return text


def dna_with_repeats(n: int, seed: int = 2, coverage: float = 0.30, lmin: int = 100,
                     lmax: int = 10_000, sub: float = 0.01) -> np.ndarray:
    rng = np.random.default_rng(seed)
    text = rng.integers(0, 4, n, dtype=np.uint8)
    return _plant(rng, text, coverage, lmin, lmax, sub)


def segmented_filtered(n: int, seed: int = 3, median: float = 2000.0, sigma: float = 1.5,
                       run_frac: float = 0.02, run_min: int = 1000, run_max: int = 50_000):
    rng = np.random.default_rng(seed)
    text = rng.integers(0, 4, n, dtype=np.uint8)
    lens = []
    total = 0
    mu = math.log(median)
    while total < n:
        L = max(2, int(rng.lognormal(mu, sigma)))
        L = min(L, n - total)
        if n - total - L == 1:  # never leave a one-symbol tail
            L += 1
        lens.append(L)
        total += L
    ends = np.cumsum(np.asarray(lens, dtype=np.uint64))
    sep = (ends - 1).astype(np.int64)
    target = int(run_frac * n)
    done = 0
    while done < target and n > run_max:
        L = int(rng.integers(run_min, run_max + 1))
        s = int(rng.integers(0, n - L))
        text[s:s + L] = 5
        done += L
    text[sep] = 4
    positions = np.nonzero(text < 4)[0].astype(np.uint64)
    return text, ends, positions


def batched_texts(count: int = 8192, seed: int = 5, min_log2: int = 10, max_log2: int = 20,
                  coverage: float = 0.10, lmin: int = 50, lmax: int = 5000, sub: float = 0.01):
    rng = np.random.default_rng(seed)
    lo, hi = min_log2 * math.log(2), max_log2 * math.log(2)
    lens = np.array([int(math.exp(rng.uniform(lo, hi))) for _ in range(count)], dtype=np.int64)
    offs = np.zeros(count + 1, dtype=np.uint64)
    offs[1:] = np.cumsum(lens)
    cat = rng.integers(0, 4, int(offs[-1]), dtype=np.uint8)
    for i in range(count):
        a, b = int(offs[i]), int(offs[i + 1])
        _plant(rng, cat[a:b], coverage, lmin, min(lmax, max(lmin, (b - a) // 2)), sub)
    return cat, offs
