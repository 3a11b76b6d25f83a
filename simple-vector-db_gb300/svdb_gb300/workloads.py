"""Seeded synthetic workloads with the shapes and value distributions the
similarity path is measured on.  The reference measures on no public
dataset; these generators stand in for its inputs.

numpy's PCG64 gives the same doubles on every platform.  Large arrays are
filled in fixed 1 Mi-element chunks, chunk c drawing from child c of the
seed's SeedSequence, so the bytes do not depend on how many threads fill
them.
"""
from __future__ import annotations

import concurrent.futures as cf
import os

import numpy as np

_CHUNK = 1 << 20


def _fill(out: np.ndarray, seed, kind: str, threads: int | None = None, **kw) -> np.ndarray:
    flat = out.reshape(-1)
    n = flat.size
    nchunks = (n + _CHUNK - 1) // _CHUNK
    seqs = np.random.SeedSequence(seed).spawn(nchunks)

    def work(c):
        g = np.random.Generator(np.random.PCG64(seqs[c]))
        lo, hi = c * _CHUNK, min(n, (c + 1) * _CHUNK)
        if kind == "normal":
            g.standard_normal(hi - lo, out=flat[lo:hi])
        else:
            flat[lo:hi] = g.uniform(kw["low"], kw["high"], hi - lo)

    threads = threads or min(32, os.cpu_count() or 1)
    if nchunks <= 1 or threads == 1:
        for c in range(nchunks):
            work(c)
    else:
        with cf.ThreadPoolExecutor(threads) as ex:
            list(ex.map(work, range(nchunks)))
    return out


def uniform(n: int, d: int, seed, low: float = -1.0, high: float = 1.0) -> np.ndarray:
    """i.i.d. uniform[low, high) float64 rows."""
    return _fill(np.empty((n, d), np.float64), seed, "uniform", low=low, high=high)


def normal(n: int, d: int, seed, normalise: bool = False) -> np.ndarray:
    """i.i.d. N(0, 1) float64 rows, optionally L2-normalised."""
    x = _fill(np.empty((n, d), np.float64), seed, "normal")
    if normalise:
        x /= np.linalg.norm(x, axis=1, keepdims=True)
    return x


class Mixture:
    """Gaussian mixture: `ncentres` centres ~ N(0, 1) in D dimensions, equal
    weights, isotropic spread `sigma`.  Points of one centre are near-ties
    for each other's queries."""

    def __init__(self, d: int, seed: int, ncentres: int = 1024, sigma: float = 0.05):
        self.d, self.seed, self.sigma = d, seed, sigma
        self.centres = _fill(np.empty((ncentres, d), np.float64), [seed, 0], "normal")

    def sample(self, n: int, stream: int) -> np.ndarray:
        """n points; `stream` separates the store (0) from query batches (1, 2, ...)."""
        g = np.random.Generator(np.random.PCG64(np.random.SeedSequence([self.seed, 1, stream])))
        which = g.integers(0, self.centres.shape[0], n)
        x = _fill(np.empty((n, self.d), np.float64), [self.seed, 2, stream], "normal")
        x *= self.sigma
        for lo in range(0, n, 1 << 16):  # bounded temporaries
            hi = min(n, lo + (1 << 16))
            x[lo:hi] += self.centres[which[lo:hi]]
        return x


def config1():
    """Plain reference path: N=10,000 x 128 U[-1,1] (seed 0), KD dimension 3,
    1,000 queries U[-1,1] (seed 1)."""
    X = np.random.default_rng(0).uniform(-1.0, 1.0, (10_000, 128))
    Q = np.random.default_rng(1).uniform(-1.0, 1.0, (1_000, 128))
    return X, Q, 3


def config2(n: int = 1_000_000, d: int = 128, nq: int = 10_000):
    """FP64 single-query scan at scale: N(0,1) rows, L2-normalised (seed 2)."""
    return normal(n, d, 2, normalise=True), normal(nq, d, [2, 1], normalise=True)


def config3(n: int = 1_000_000, d: int = 768, seed: int = 3):
    """Mixed-precision batched search store: 1,024-centre mixture, sigma 0.05."""
    m = Mixture(d, seed)
    return m, m.sample(n, 0)


# Uneven batched multi-collection workload: (dimension, rows) per collection and
# the share of the ragged query batch that goes to it.
CONFIG4_COLLECTIONS = ((64, 2_000_000), (128, 1_000_000), (384, 500_000), (768, 200_000), (1536, 50_000))
CONFIG4_SHARES = (0.40, 0.25, 0.15, 0.12, 0.08)


def config4(total_queries: int = 8192, scale: float = 1.0):
    """Five collections of uniform[-1,1] float64 rows (seed 4), a ragged batch
    of `total_queries` split 40/25/15/12/8 % across them, k per query uniform
    in [1, 100].  `scale` shrinks the collections (tests)."""
    rng = np.random.default_rng(4)
    out = []
    counts = [int(round(total_queries * f)) for f in CONFIG4_SHARES]
    counts[0] += total_queries - sum(counts)
    for c, ((d, n), nq) in enumerate(zip(CONFIG4_COLLECTIONS, counts)):
        n = max(1, int(n * scale))
        X = uniform(n, d, [4, c])
        Q = uniform(nq, d, [4, 100 + c])
        ks = rng.integers(1, 101, nq)
        out.append((X, Q, ks))
    return out
