"""Seeded inputs behind tests/golden/golden_reference.npz.

numpy's default_rng (PCG64) gives the same doubles on every platform, so the
fixtures store only the reference's outputs plus a checksum of each input;
tests regenerate the inputs here and check the checksum first.
"""
from __future__ import annotations

import hashlib

import numpy as np


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def compare_inputs():
    """Config-1 shapes: N=10,000 x 128 U[-1,1] (seed 0); 1,000 queries x 10
    random stored ids (seed 1 stream) -> pairs."""
    X = np.random.default_rng(0).uniform(-1.0, 1.0, (10_000, 128))
    r = np.random.default_rng(1)
    a = r.integers(0, 10_000, 10_000)
    b = r.integers(0, 10_000, 10_000)
    return X, np.stack([a, b], 1).astype(np.int64)


def addvec_pairs():
    """Adversarial /compare pairs: the test/add_vectors.sh value distribution
    (integer part 1..9, 0-6 random decimal digits, all positive -> cosines
    near 1), odd dimensions 1..1536, zero vectors, large magnitudes."""
    r = np.random.default_rng(7)
    A, B = [], []

    def addvec(d):
        ip = r.integers(1, 10, d).astype(np.float64)
        nd = r.integers(0, 7, d)
        frac = np.array([r.integers(0, 10**k) / 10**k if k else 0.0 for k in nd])
        return ip + frac

    for d in (1, 2, 3, 5, 17, 64, 127, 128, 129, 384, 768, 1536):
        A.append(addvec(d))
        B.append(addvec(d))
        A.append(r.uniform(-1, 1, d))
        B.append(r.uniform(-1, 1, d))
        A.append(r.normal(0, 1e3, d))
        B.append(r.normal(0, 1e-3, d))
    A.append(np.zeros(128))
    B.append(r.uniform(-1, 1, 128))
    A.append(np.zeros(16))
    B.append(np.zeros(16))
    x = r.uniform(-1, 1, 128)
    A.append(x)
    B.append(x.copy())
    return A, B


def kd_inputs():
    """Config 1 /nearest: N=10,000 x 128 U[-1,1] seed 0, kd_dim 3; 1,000
    queries U[-1,1] seed 1."""
    X = np.random.default_rng(0).uniform(-1.0, 1.0, (10_000, 128))
    Q = np.random.default_rng(1).uniform(-1.0, 1.0, (1_000, 128))
    return X, Q, 3


def mutation_trace():
    """3,000 operations on a D=16 store: 60% insert, 20% update, 20% delete,
    indices sometimes out of range (ignored by the reference), a few exact
    duplicates to exercise the KD tie rule."""
    D = 16
    r = np.random.default_rng(11)
    ops = []
    size = 0
    pool = []
    for _ in range(3_000):
        u = r.random()
        if u < 0.6 or size == 0:
            if pool and r.random() < 0.05:
                v = pool[int(r.integers(0, len(pool)))].copy()
            else:
                v = r.uniform(-1, 1, D)
            pool.append(v)
            ops.append((0, 0, v))
            size += 1
        elif u < 0.8:
            idx = int(r.integers(0, size + 3))
            ops.append((1, idx, r.uniform(-1, 1, D)))
        else:
            idx = int(r.integers(0, size + 3))
            ops.append((2, idx, None))
            if idx < size:
                size -= 1
    return ops, D


def uuid_pool():
    """uuid strings for the uuid trace: 36-character uuid-like strings, a
    family sharing a 30-character prefix, short ones, duplicates by reuse,
    and the empty uuid."""
    r = np.random.default_rng(21)
    hexd = np.array(list("0123456789abcdef"))

    def u36():
        h = "".join(r.choice(hexd, 32))
        return f"{h[:8]}-{h[8:12]}-{h[12:16]}-{h[16:20]}-{h[20:]}".encode()

    pool = [u36() for _ in range(120)]
    stem = u36()[:30]
    pool += [stem + f"{i:06d}".encode() for i in range(40)]
    pool += [bytes(r.choice(list(b"abcxyz"), int(r.integers(1, 6))).tolist()) for _ in range(40)]
    pool += [b""]
    return pool


def uuid_trace():
    """2,000 operations on a D=8 store: 55 % insert with a uuid drawn from the
    pool (so uuids repeat), 20 % update with a new uuid (sometimes empty), 20 %
    delete, indices sometimes out of range; then every pool uuid and a few
    absent ones are looked up."""
    D = 8
    r = np.random.default_rng(22)
    pool = uuid_pool()
    ops = []
    size = 0
    for _ in range(2_000):
        u = r.random()
        if u < 0.55 or size == 0:
            ops.append((0, 0, r.uniform(-1, 1, D), pool[int(r.integers(0, len(pool)))]))
            size += 1
        elif u < 0.75:
            idx = int(r.integers(0, size + 3))
            ops.append((1, idx, r.uniform(-1, 1, D), pool[int(r.integers(0, len(pool)))]))
        else:
            idx = int(r.integers(0, size + 3))
            ops.append((2, idx, None, b""))
            if idx < size:
                size -= 1
    keys = pool + [b"absent", pool[0][:35], pool[120][:31] + b"x"]
    return ops, D, keys
