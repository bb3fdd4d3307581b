"""Seeded synthetic workloads shaped like the benchmark configurations
(no dataset exists for this path; these stand in for it)."""
import math

import numpy as np


def smooth7(lo, hi):
    """Numbers 2^a 3^b 5^c 7^d in [lo, hi] (601 of them in [16, 65536])."""
    out = []
    p2 = 1
    while p2 <= hi:
        p3 = p2
        while p3 <= hi:
            p5 = p3
            while p5 <= hi:
                p7 = p5
                while p7 <= hi:
                    if p7 >= lo:
                        out.append(p7)
                    p7 *= 7
                p5 *= 5
            p3 *= 3
        p2 *= 2
    return np.array(sorted(out), dtype=np.int64)


def primes(lo, hi):
    """Primes in [lo, hi] (6536 of them in [16, 65536], the largest 65521)."""
    sieve = np.ones(hi + 1, dtype=bool)
    sieve[:2] = False
    for p in range(2, int(math.isqrt(hi)) + 1):
        if sieve[p]:
            sieve[p * p::p] = False
    idx = np.nonzero(sieve)[0]
    return idx[idx >= lo].astype(np.int64)


def _nearest(sorted_vals, x):
    i = np.searchsorted(sorted_vals, x)
    i = np.clip(i, 1, len(sorted_vals) - 1)
    lo, hi = sorted_vals[i - 1], sorted_vals[i]
    return np.where(np.abs(x - lo) <= np.abs(hi - x), lo, hi)


def ragged_lengths(count, seed=4, lo=16, hi=65536, frac_smooth=0.7):
    """Lengths log-uniform in [lo, hi], ~70% snapped to the nearest 7-smooth
    number and ~30% to the nearest prime; modes Forward or Inverse with
    p = 1/2 (returned as the C ABI codes -1 / 2)."""
    rng = np.random.default_rng(seed)
    x = np.exp(rng.uniform(math.log(lo), math.log(hi), count))
    sm = smooth7(lo, hi)
    pr = primes(lo, hi)
    use_smooth = rng.random(count) < frac_smooth
    lengths = np.where(use_smooth, _nearest(sm.astype(np.float64), x), _nearest(pr.astype(np.float64), x))
    lengths = lengths.astype(np.int64)
    modes = np.where(rng.random(count) < 0.5, -1, 2).astype(np.int32)
    return lengths, modes
