"""Pin the CPU oracle to the reference: the restatement in oracle/svdb_oracle.c
must reproduce the reference's own outputs (tests/golden, generated by
running the compiled reference) bit for bit, and -- where the reference
sources are present -- the compiled reference itself on fresh inputs."""
import numpy as np
import pytest

from golden_inputs import addvec_pairs, compare_inputs, kd_inputs, mutation_trace, sha


def test_compare_metrics_match_golden(oracle, golden):
    X, pairs = compare_inputs()
    assert sha(X) == str(golden["compare_x_sha"])
    assert sha(pairs) == str(golden["compare_pairs_sha"])
    vals = golden["compare_vals"]
    for i in range(0, pairs.shape[0], 7):
        a, b = pairs[i]
        for m in range(3):
            assert oracle.ref_metric(m, X[a], X[b]).tobytes() == vals[i, m].tobytes(), (i, m)


def test_adversarial_metrics_match_golden(oracle, golden):
    A, B = addvec_pairs()
    assert sha(np.concatenate([np.concatenate(A), np.concatenate(B)])) == str(golden["adv_sha"])
    adv = golden["adv_vals"]
    for i in range(len(A)):
        for m in range(3):
            got = oracle.ref_metric(m, A[i], B[i])
            assert got.tobytes() == adv[i, m].tobytes() or (np.isnan(got) and np.isnan(adv[i, m])), (i, m)


def test_dimension_mismatch_returns_minus_one(oracle):
    a, b = np.ones(4), np.ones(5)
    for m in range(3):
        assert oracle.ref_metric(m, a, b) == np.float32(-1.0)


def test_kd_nearest_matches_golden(oracle, golden):
    X, Q, kd = kd_inputs()
    assert sha(X) == str(golden["kd_x_sha"]) and sha(Q) == str(golden["kd_q_sha"])
    st = oracle.store(X.shape[1], kd)
    for i in range(X.shape[0]):
        st.insert(X[i])
    got = np.array([st.nearest(q) for q in Q])
    assert np.array_equal(got, golden["kd_nearest"])


def test_mutation_replay_matches_golden(oracle, golden):
    ops, D = mutation_trace()
    _, Q, kd = kd_inputs()
    st = oracle.store(D, kd)
    for op, idx, v in ops:
        if op == 0:
            st.insert(v)
        elif op == 1:
            st.update(idx, v)
        else:
            st.delete(idx)
    assert st.size == int(golden["mut_size"])
    assert sha(st.rows()) == bytes(golden["mut_rows_sha"]).decode()
    got = np.array([st.nearest(q) for q in Q[:200, :D]])
    assert np.array_equal(got, golden["mut_nearest"])


def test_kd_empty_and_duplicates(oracle):
    t = oracle.kd(3)
    assert t.nearest(np.zeros(3)) == -1
    p = np.array([0.5, 0.5, 0.5])
    for i in range(5):
        t.insert(p, 10 + i)  # duplicates descend right: the first inserted wins
    assert t.nearest(p) == 10


def test_fp64_canonical_vs_sequential(oracle):
    r = np.random.default_rng(3)
    for d in (1, 3, 8, 127, 768, 1536):
        a, b = r.normal(size=d), r.normal(size=d)
        for m in range(3):
            c, s = oracle.fp64(m, a, b), oracle.fp64(m, a, b, seq=True)
            assert abs(c - s) <= 1e-12 * max(1.0, abs(s)), (d, m, c, s)


def test_topk_oracle_order_and_ties(oracle):
    r = np.random.default_rng(4)
    X = r.normal(size=(500, 16))
    X[100] = X[7]  # exact duplicate: tie broken by the lower id
    q = X[7] + 1e-3
    for m in range(3):
        ids, vals = oracle.topk(m, X, q[None], 10)
        full = np.array([oracle.fp64(m, q, x) for x in X])
        key = full if m == 1 else -full
        order = np.lexsort((np.arange(len(X)), key))[:10]
        assert np.array_equal(ids[0], order)
        assert list(ids[0]).index(7) < list(ids[0]).index(100)


def test_oracle_matches_compiled_reference(oracle, refstore):
    """Fresh random inputs through both the restatement and the compiled
    reference (skipped where the reference sources are absent)."""
    import oracle as O
    r = np.random.default_rng(99)
    for t in range(300):
        d = int(r.integers(1, 200))
        a, b = r.uniform(-3, 3, d), r.uniform(-3, 3, d)
        for m in range(3):
            assert oracle.ref_metric(m, a, b).tobytes() == refstore.metric(m, a, b).tobytes()
    rs = O.RefStore(refstore, 3)
    os_ = oracle.store(32, 3)
    X = r.uniform(-1, 1, (3000, 32))
    for x in X:
        rs.insert(x)
        os_.insert(x)
    for _ in range(300):
        i = int(r.integers(0, rs.size + 2))
        if r.random() < 0.5:
            v = r.uniform(-1, 1, 32)
            rs.update(i, v)
            os_.update(i, v)
        else:
            rs.delete(i)
            os_.delete(i)
    Q = r.uniform(-1, 1, (300, 32))
    assert [rs.nearest(q) for q in Q] == [os_.nearest(q) for q in Q]
    rs.free()


def _replay_uuid_trace(ops):
    """The positional store's uuids after the trace (reference semantics:
    insert appends, update replaces the row's uuid, delete shifts; indices
    past the end are ignored), as an n x 37 record table."""
    import oracle as O
    recs = []
    for op, idx, _, u in ops:
        if op == 0:
            recs.append(O.uuid_record(u))
        elif op == 1 and idx < len(recs):
            recs[idx] = O.uuid_record(u)
        elif op == 2 and idx < len(recs):
            del recs[idx]
    return np.stack(recs) if recs else np.zeros((0, 37), np.uint8)


def test_uuid_restatement_matches_golden(golden):
    """vector_db_read_by_uuid (src/vector_database.c:145-158) after a trace of
    inserts with repeated, prefix-sharing, short and empty uuids, updates that
    change uuids and deletes: the numpy restatement finds the same rows the
    compiled reference found."""
    import oracle as O
    from golden_inputs import uuid_trace
    ops, _, keys = uuid_trace()
    table = _replay_uuid_trace(ops)
    assert table.shape[0] == int(golden["uuid_size"])
    found = np.array([O.uuid_first(table, k) for k in keys])
    assert np.array_equal(found, golden["uuid_found"])
    assert (found >= 0).sum() > 150 and (found < 0).sum() >= 3


def test_uuid_restatement_matches_compiled_reference(refstore):
    import oracle as O
    r = np.random.default_rng(3)
    st = O.RefStore(refstore, 3)
    recs = []
    pool = [b"", b"a", b"ab", b"x" * 36, b"x" * 35 + b"y"] + [f"{i:036d}".encode() for i in range(20)]
    for _ in range(400):
        u = pool[int(r.integers(0, len(pool)))]
        if r.random() < 0.7 or not recs:
            st.insert(r.uniform(-1, 1, 4), u)
            recs.append(O.uuid_record(u))
        else:
            i = int(r.integers(0, len(recs)))
            if r.random() < 0.5:
                st.update(i, r.uniform(-1, 1, 4), u)
                recs[i] = O.uuid_record(u)
            else:
                st.delete(i)
                del recs[i]
    table = np.stack(recs)
    for k in pool + [b"x" * 37, b"zz"]:
        assert st.find_uuid(k) == O.uuid_first(table, k), k
    st.free()
