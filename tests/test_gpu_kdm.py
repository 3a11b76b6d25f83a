"""GPU parity of the opt-in median-split KD tree (svdb_nearest_batch_median).

Bar: for every query, the position of the row nearest over the first kd
coordinates -- the reference's unfused FP64 squared distance
(src/kdtree.c:134-137) -- with ties to the lowest position, equal to a brute
force over the store's current rows, on the config-1 shapes (10,000 x 128,
kd 3, 1,000 queries), exact duplicates, kd dimensions 1..16, tiny and empty
stores, after inserts, updates and deletes (the tree is rebuilt on the
device), and at 300,000 rows.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S(svdb):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return svdb


def brute_nearest(P, Q, kdim):
    """Lowest position with the least sum_i (p_i - q_i)^2 over i < kdim,
    summed left to right, every operation rounded (no fused multiply-add)."""
    out = np.empty(Q.shape[0], np.int64)
    for j, q in enumerate(Q):
        d = np.zeros(P.shape[0])
        for a in range(kdim):
            t = P[:, a] - q[a]
            d = d + t * t
        out[j] = int(np.argmin(d)) if P.shape[0] else -1
    return out


def test_median_tree_config1_shapes(S):
    X = np.random.default_rng(0).uniform(-1.0, 1.0, (10_000, 128))
    Q = np.random.default_rng(1).uniform(-1.0, 1.0, (1_000, 128))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    got = db.nearest_batch_median(Q)
    assert np.array_equal(got, brute_nearest(X, Q, 3))
    db.close()


def test_median_tree_duplicates_and_ties(S):
    rng = np.random.default_rng(2)
    base = rng.integers(-3, 4, (500, 4)).astype(np.float64)  # a coarse grid: many equal coordinates
    X = np.vstack([base, base[::-1], base[:50]])  # exact duplicates at higher positions
    Q = np.vstack([base[:100], rng.integers(-3, 4, (100, 4)) + 0.5])  # hits and exact equidistant ties
    for kdim in (1, 2, 3, 4):
        db = S.VectorDatabase(0, kdim)
        db.insert_batch(X)
        assert np.array_equal(db.nearest_batch_median(Q), brute_nearest(X, Q, kdim)), kdim
        db.close()


@pytest.mark.parametrize("n", [0, 1, 2, 3, 7, 64, 1000])
def test_median_tree_small_stores(S, n):
    rng = np.random.default_rng(n)
    Q = rng.normal(size=(20, 16))
    db = S.VectorDatabase(0, 5)
    if n:
        X = rng.normal(size=(n, 16))
        db.insert_batch(X)
        want = brute_nearest(X, Q, 5)
    else:
        db.insert(rng.normal(size=16))
        db.delete(0)
        want = np.full(20, -1)
    assert np.array_equal(db.nearest_batch_median(Q), want)
    db.close()


def test_median_tree_kd_dimensions(S):
    rng = np.random.default_rng(3)
    X = rng.normal(size=(20_000, 16))
    Q = rng.normal(size=(300, 16))
    for kdim in (1, 2, 5, 16):
        db = S.VectorDatabase(0, kdim)
        db.insert_batch(X)
        assert np.array_equal(db.nearest_batch_median(Q), brute_nearest(X, Q, kdim)), kdim
        db.close()


def test_median_tree_follows_mutations(S):
    """The tree is rebuilt after the rows change and holds no stale nodes:
    results are the brute force over the current rows (where the reference's
    insertion-order tree would still hold deleted and overwritten points)."""
    rng = np.random.default_rng(4)
    X = rng.uniform(-1, 1, (5_000, 8))
    Q = rng.uniform(-1, 1, (400, 8))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    rows = list(X)
    assert np.array_equal(db.nearest_batch_median(Q), brute_nearest(np.stack(rows), Q, 3))
    for _ in range(300):
        u = rng.random()
        if u < 0.4:
            v = rng.uniform(-1, 1, 8)
            db.insert(v)
            rows.append(v)
        elif u < 0.7:
            i = int(rng.integers(0, len(rows)))
            v = Q[int(rng.integers(0, len(Q)))] + 1e-6  # pull rows next to queries
            db.update(i, v)
            rows[i] = v
        else:
            i = int(rng.integers(0, len(rows)))
            db.delete(i)
            del rows[i]
    assert np.array_equal(db.nearest_batch_median(Q), brute_nearest(np.stack(rows), Q, 3))
    db.close()


def test_median_tree_skips_rows_of_another_dimension(S):
    rng = np.random.default_rng(5)
    X = rng.normal(size=(100, 6))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X[:50])
    db.insert(np.zeros(4))  # another dimension: a placeholder position, not in the tree
    db.insert_batch(X[50:])
    Q = np.vstack([np.zeros(6), X[70] + 1e-9])
    got = db.nearest_batch_median(Q)
    full = brute_nearest(X, Q, 3)
    assert list(got) == [p + (p >= 50) for p in full]  # positions shift past the placeholder
    db.close()


def test_median_tree_at_scale(S):
    rng = np.random.default_rng(6)
    X = rng.normal(size=(300_000, 8))
    Q = rng.normal(size=(200, 8))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    assert np.array_equal(db.nearest_batch_median(Q), brute_nearest(X, Q, 3))
    db.close()
