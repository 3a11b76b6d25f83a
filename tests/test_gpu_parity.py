"""GPU parity: every hot-path call through the C ABI against the oracle and
the golden fixtures made by running the reference itself.

Bars: /compare float results bit-identical to the reference's; /nearest ids
identical (ties and mutation history included); top-k ids identical to the
FP64 oracle with ties to the lowest index, and FP64 values bit-identical to
the oracle's canonical-order restatement (which itself agrees with the
sequential FP64 formulas to 1e-12 relative, test_oracle_golden.py).
"""
import numpy as np
import pytest

from golden_inputs import addvec_pairs, compare_inputs, kd_inputs, mutation_trace, sha

pytestmark = pytest.mark.gpu

REL_TOL_FP64 = 1e-12  # reported distances vs the sequential FP64 formulas


@pytest.fixture(scope="module")
def S(svdb):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return svdb


def _db(S, X, kd=3):
    db = S.VectorDatabase(0, kd)
    db.insert_batch(X)
    return db


# --------------------------------------------------------------------------- /compare
def test_compare_batch_bit_exact_config1(S, golden):
    X, pairs = compare_inputs()
    db = _db(S, X)
    for m in range(3):
        out, st = db.compare_batch(m, pairs[:, 0], pairs[:, 1], expected_dim=128)
        assert (st == S.CMP_OK).all()
        assert out.tobytes() == golden["compare_vals"][:, m].tobytes()
    db.close()


def test_dropin_metrics_adversarial(S, golden):
    A, B = addvec_pairs()
    adv = golden["adv_vals"]
    fns = (S.cosine_similarity, S.euclidean_distance, S.dot_product)
    for i in range(len(A)):
        for m in range(3):
            got = fns[m](A[i], B[i])
            assert got.tobytes() == adv[i, m].tobytes() or (np.isnan(got) and np.isnan(adv[i, m])), (i, m)
    for m in range(3):
        assert fns[m](np.ones(4), np.ones(5)) == np.float32(-1.0)


def test_dropin_calls_from_many_threads(S, golden, oracle):
    """The unmodified server's call pattern (src/compare_handler.c:153-159,
    403): one thread per connection, each calling cosine_similarity /
    euclidean_distance / dot_product on the store's own rows (the Vectors
    vector_db_read returns, so the rows are found where they are in HBM),
    on free-standing vectors, and kdtree_nearest, one call at a time and all
    at once.  Concurrent calls are combined into shared launches; every result
    is the reference's, bit for bit."""
    import ctypes as C
    import threading
    X, pairs = compare_inputs()
    db = _db(S, X)
    db.sync()
    fns = (S.lib.cosine_similarity, S.lib.euclidean_distance, S.lib.dot_product)
    rows = [S.lib.vector_db_read(db.ptr, i).contents for i in range(X.shape[0])]
    r = np.random.default_rng(31)
    free_a = r.uniform(-1, 1, (64, 128))
    free_b = r.uniform(-1, 1, (64, 128))
    fa = [S.make_vector(v, owned=False) for v in free_a]
    fb = [S.make_vector(v, owned=False) for v in free_b]
    Q = r.uniform(-1, 1, (400, 128))
    want_near = np.array([db.kdtree_nearest(q) for q in Q[:8]])  # single calls first
    O_kd = oracle.kd(3)
    for i in range(X.shape[0]):
        O_kd.insert(X[i], i)
    want_q = np.array([O_kd.nearest(q) for q in Q])
    assert np.array_equal(want_near, want_q[:8])
    nthreads, per = 16, 120
    got = np.zeros((nthreads, per), np.float32)
    want = np.zeros((nthreads, per), np.float32)
    near = np.full((nthreads, 25), -2, np.int64)
    errs = []

    def work(t_):
        try:
            g = np.random.default_rng(100 + t_)
            for j in range(per):
                m = int(g.integers(0, 3))
                if g.random() < 0.75:  # two stored rows
                    p = pairs[int(g.integers(0, len(pairs)))]
                    got[t_, j] = fns[m](rows[p[0]], rows[p[1]])
                    want[t_, j] = golden["compare_vals"][np.flatnonzero((pairs == p).all(1))[0], m]
                else:  # vectors of no store
                    k = int(g.integers(0, 64))
                    got[t_, j] = fns[m](fa[k], fb[k])
                    want[t_, j] = oracle.ref_metric(m, free_a[k], free_b[k])
                if j % 5 == 0:
                    qi = (t_ * 25 + j // 5) % len(Q)
                    near[t_, j // 5] = S.lib.kdtree_nearest(db.kdtree, Q[qi].ctypes.data_as(S._dp))
        except Exception as e:  # pragma: no cover - reported below
            errs.append(e)

    ths = [threading.Thread(target=work, args=(t_,)) for t_ in range(nthreads)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    assert not errs, errs
    assert got.tobytes() == want.tobytes()
    for t_ in range(nthreads):
        for j in range(0, per, 5):
            assert near[t_, j // 5] == want_q[(t_ * 25 + j // 5) % len(Q)]
    # a stored row changed through the store API is seen by the next call
    new = r.uniform(-1, 1, 128)
    db.update(3, new)
    v3 = S.lib.vector_db_read(db.ptr, 3).contents
    assert np.float32(S.lib.cosine_similarity(v3, rows[7])) == oracle.ref_metric(0, new, X[7])
    db.close()


def test_compare_rows_of_mixed_dimension(S, oracle):
    db = S.VectorDatabase(0, 3)
    r = np.random.default_rng(21)
    a, b, c = r.uniform(-1, 1, 64), r.uniform(-1, 1, 64), r.uniform(-1, 1, 9)
    db.insert(a)
    db.insert(c)  # another dimension: kept in positions, compared by the vector kernel
    db.insert(b)
    db.insert(c * 2)
    for m in range(3):
        out, st = db.compare_batch(m, [0, 1, 0], [2, 3, 1])
        assert list(st) == [0, 0, S.CMP_DIFF_DIM]
        assert out[0].tobytes() == oracle.ref_metric(m, a, b).tobytes()
        assert out[1].tobytes() == oracle.ref_metric(m, c, c * 2).tobytes()
    db.close()


# --------------------------------------------------------------------------- /nearest
def test_kd_nearest_config1_golden(S, golden):
    X, Q, kd = kd_inputs()
    db = _db(S, X, kd)
    got = db.nearest_batch(Q)
    assert np.array_equal(got, golden["kd_nearest"])
    # the drop-in single-query call, as src/compare_handler.c:403 makes it
    for i in range(0, Q.shape[0], 97):
        assert db.kdtree_nearest(Q[i]) == golden["kd_nearest"][i]
    db.close()


def test_kd_nearest_after_mutation_golden(S, golden):
    ops, D = mutation_trace()
    _, Q, kd = kd_inputs()
    db = S.VectorDatabase(0, kd)
    for op, idx, v in ops:
        if op == 0:
            db.insert(v)
        elif op == 1:
            db.update(idx, v)
        else:
            db.delete(idx)
    assert db.size == int(golden["mut_size"])
    rows = np.stack([db.read(i) for i in range(db.size)])
    assert sha(rows) == bytes(golden["mut_rows_sha"]).decode()
    assert np.array_equal(db.nearest_batch(Q[:200, :D]), golden["mut_nearest"])
    db.close()


def test_kd_standalone_tree_and_ties(S, oracle):
    t = S.KDTree(3)
    assert t.nearest(np.zeros(3)) == -1  # empty tree: (size_t)-1
    p = np.array([0.25, -0.5, 0.75])
    for i in range(6):
        t.insert(p, 100 + i)
    assert t.nearest(p) == 100
    # a deep degenerate tree (sorted insertion): the stack spills past 64 levels
    o = oracle.kd(2)
    pts = np.stack([np.linspace(0, 1, 300), np.linspace(1, 0, 300)], 1)
    t2 = S.KDTree(2)
    for i, x in enumerate(pts):
        t2.insert(x, i)
        o.insert(x, i)
    qs = np.random.default_rng(2).uniform(-0.2, 1.2, (50, 2))
    assert [t2.nearest(q) for q in qs] == [o.nearest(q) for q in qs]
    t.close()
    t2.close()


def test_kd_random_trees_various_dims(S, oracle):
    r = np.random.default_rng(8)
    for kd, n in ((1, 500), (2, 3000), (3, 20000), (5, 5000), (16, 4000)):
        X = r.uniform(-1, 1, (n, 16))
        X[n // 2] = X[n // 3]  # duplicate point
        db = _db(S, X, kd)
        o = oracle.kd(kd)
        for i, x in enumerate(X):
            o.insert(x, i)
        Q = np.concatenate([r.uniform(-1, 1, (300, 16)), X[:50]])
        assert np.array_equal(db.nearest_batch(Q), [o.nearest(q) for q in Q]), kd
        db.close()


# --------------------------------------------------------------------------- top-k
def _check_topk(ids, vals, wid, wval, metric, oracle, X, Q):
    assert np.array_equal(ids, wid)
    assert np.array_equal(vals, wval)
    # distances agree with the sequential FP64 formulas to 1e-12 relative
    for qi in range(0, Q.shape[0], max(1, Q.shape[0] // 4)):
        for j in range(ids.shape[1]):
            if ids[qi, j] < 0:
                continue
            s = oracle.fp64(metric, Q[qi], X[ids[qi, j]], seq=True)
            assert abs(vals[qi, j] - s) <= REL_TOL_FP64 * max(1.0, abs(s))


@pytest.mark.parametrize("d", [1, 3, 128, 200, 768])
@pytest.mark.parametrize("metric", [0, 1, 2])
def test_topk_fp64_matches_oracle(S, oracle, d, metric):
    r = np.random.default_rng(1000 + d)
    n = 6000 if d <= 200 else 3000
    X = r.normal(size=(n, d))
    X[17] = X[4000 % n]  # exact duplicate: tie to the lower index
    Q = np.concatenate([r.normal(size=(9, d)), X[[4000 % n, 5]]])
    db = _db(S, X)
    for k in (1, 10, 100):
        ids, vals = db.search(Q, k, metric, S.PREC_FP64)
        wid, wval = oracle.topk(metric, X, Q, k)
        _check_topk(ids, vals, wid, wval, metric, oracle, X, Q)
    db.close()


@pytest.mark.parametrize("nq", [1, 2, 5, 64, 300])
def test_topk_fp64_query_batches(S, oracle, nq):
    r = np.random.default_rng(nq)
    X = r.uniform(-1, 1, (20000, 64))
    Q = r.uniform(-1, 1, (nq, 64))
    db = _db(S, X)
    for metric in range(3):
        ids, vals = db.search(Q, 10, metric, S.PREC_FP64)
        wid, wval = oracle.topk(metric, X, Q, 10)
        _check_topk(ids, vals, wid, wval, metric, oracle, X, Q)
    db.close()


def test_topk_fp64_k_larger_than_store_and_empty(S, oracle):
    r = np.random.default_rng(3)
    X = r.normal(size=(7, 32))
    db = _db(S, X)
    ids, vals = db.search(X[:2], 12, 0, S.PREC_FP64)
    wid, wval = oracle.topk(0, X, X[:2], 12)
    assert np.array_equal(ids, wid) and (ids[:, 7:] == -1).all()
    assert np.array_equal(vals[:, :7], wval[:, :7]) and np.isnan(vals[:, 7:]).all()
    for i in range(7):
        db.delete(0)
    ids, vals = db.search(X[:2], 3, 1, S.PREC_FP64)
    assert (ids == -1).all() and np.isnan(vals).all()
    db.close()


def test_topk_fp64_after_deletes_and_updates(S, oracle):
    """Logical ids follow the reference's shifting positions
    (src/vector_database.c:185-195); updated rows are searched with their new
    values (src/vector_database.c:169-177)."""
    r = np.random.default_rng(12)
    X = r.normal(size=(5000, 48))
    db = _db(S, X)
    host = list(X)
    for step in range(300):
        i = int(r.integers(0, len(host)))
        if step % 3 == 0:
            v = r.normal(size=48)
            db.update(i, v)
            host[i] = v
        else:
            db.delete(i)
            host.pop(i)
    H = np.stack(host)
    Q = r.normal(size=(20, 48))
    for metric in range(3):
        ids, vals = db.search(Q, 10, metric, S.PREC_FP64)
        wid, wval = oracle.topk(metric, H, Q, 10)
        _check_topk(ids, vals, wid, wval, metric, oracle, H, Q)
    db.close()


def test_topk_error_bounds_hold(S, oracle):
    r = np.random.default_rng(44)
    X = r.normal(size=(4000, 96)) * 10
    Q = r.normal(size=(8, 96))
    db = _db(S, X)
    for metric in range(3):
        ids, vals, err = db.search(Q, 10, metric, S.PREC_FP64, with_err=True)
        for qi in range(Q.shape[0]):
            for j in range(10):
                s = oracle.fp64(metric, Q[qi], X[ids[qi, j]], seq=True)
                assert abs(vals[qi, j] - s) <= err[qi, j] + abs(s) * 2**-52
    db.close()


def test_topk_rejects_bad_arguments(S):
    db = _db(S, np.ones((4, 8)))
    with pytest.raises(S.SvdbError):
        db.search(np.ones(8), 0)
    with pytest.raises(S.SvdbError):
        db.search(np.ones(9), 1)
    with pytest.raises(S.SvdbError):
        db.search(np.ones(8), 1, metric=7)
    db.close()


def test_search_host_buffers_pinned_and_pageable(svdb, oracle):
    """Host-buffer searches give the same answers whether the queries and the
    result arrays are page-locked (DMA straight to and from them) or pageable
    (staged through the library's buffer)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    rng = np.random.default_rng(12)
    X = rng.normal(size=(5000, 96))
    Q = rng.normal(size=(70, 96))
    db = svdb.VectorDatabase(0, 3)
    db.insert_batch(X)
    Qp = torch.from_numpy(Q).pin_memory().numpy()
    for prec in (svdb.PREC_FP64, svdb.PREC_BF16):
        wid, wval = oracle.topk(1, X, Q, 10)
        a_ids, a_vals = db.search(Q, 10, 1, prec)
        ids_h = torch.empty((70, 10), dtype=torch.int64).pin_memory().numpy()
        dists_h = torch.empty((70, 10), dtype=torch.float64).pin_memory().numpy()
        for _ in range(2):  # reuse of the same page-locked buffers
            db.search(Qp, 10, 1, prec, out=(ids_h, dists_h))
            assert np.array_equal(ids_h, wid) and np.array_equal(dists_h, wval)
        assert np.array_equal(a_ids, wid) and np.array_equal(a_vals, wval)
        ids_m, dists_m = np.empty((70, 10), np.int64), np.empty((70, 10))  # pinned queries, pageable results
        db.search(Qp, 10, 1, prec, out=(ids_m, dists_m))
        assert np.array_equal(ids_m, wid) and np.array_equal(dists_m, wval)
    db.close()
