"""GPU parity of the ragged multi-collection plan (svdb_ragged_*).

One plan binds an uneven batch over several stores of different dimensions,
each query with its own k.  Bar: for every query, the first k entries are
the ids and FP64 values of the oracle's exact top-k (ids identical, ties to
the lowest index; values bit-identical to the oracle's canonical order) and
the entries past its k are -1 / NaN -- whichever execution choice the
autotuner keeps, with or without the CUDA graph, and again after the stores
change between runs (the graph is captured anew).
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


def _mixture(rng, n, d, centres, sigma=0.05):
    C = rng.normal(size=(centres, d))
    return C, C[rng.integers(0, centres, n)] + sigma * rng.normal(size=(n, d))


def _collections(rng):
    out = []
    for d, n, nq in ((64, 20000, 300), (200, 6000, 130), (768, 3000, 60)):
        C, X = _mixture(rng, n, d, 24)
        Q = C[rng.integers(0, 24, nq)] + 0.05 * rng.normal(size=(nq, d))
        ks = rng.integers(1, 101, nq)
        ks[:3] = (1, 16, 33)  # every k class is present
        out.append((X, Q, ks))
    return out


def _bind(S, cols, dbs):
    import torch
    parts, bufs = [], []
    for (X, Q, ks), db in zip(cols, dbs):
        stride = int(ks.max()) + 3  # wider than any k: the tail must read -1 / NaN
        q = torch.from_numpy(Q).cuda()
        ids = torch.full((Q.shape[0], stride), 7, dtype=torch.int64, device="cuda")
        dd = torch.zeros((Q.shape[0], stride), dtype=torch.float64, device="cuda")
        parts.append((db, q.data_ptr(), Q.shape[0], Q.shape[1], ks, ids.data_ptr(), dd.data_ptr(), stride))
        bufs.append((q, ids, dd))
    return parts, bufs


def _check(oracle, metric, cols, bufs):
    for (X, Q, ks), (_, ids, dd) in zip(cols, bufs):
        ids, dd = ids.cpu().numpy(), dd.cpu().numpy()
        kmax = int(ks.max())
        wid, wval = oracle.topk(metric, X, Q, kmax)
        for i, k in enumerate(ks):
            assert np.array_equal(ids[i, :k], wid[i, :k]), (X.shape, i, k)
            assert np.array_equal(dd[i, :k], wval[i, :k]), (X.shape, i, k)
            assert (ids[i, k:] == -1).all() and np.isnan(dd[i, k:]).all(), (X.shape, i, k)


@pytest.mark.parametrize("metric,precision", [(0, 1), (1, 1), (2, 0)])
def test_ragged_plan_matches_oracle(S, oracle, metric, precision):
    rng = np.random.default_rng(300 + 3 * metric + precision)
    cols = _collections(rng)
    dbs = []
    for X, _, _ in cols:
        db = S.VectorDatabase(0, 3)
        db.insert_batch(X)
        dbs.append(db)
    parts, bufs = _bind(S, cols, dbs)
    plan = S.RaggedPlan(parts, metric, precision, S.RAGGED_AUTOTUNE)
    info = plan.info()
    assert info["graph"] == 1 and info["captures"] >= 1
    assert sum(t > 0 for t in info["tuned_ms"]) == 4  # mixed k classes, 3 stores: every layout was timed
    # cosine: each store's screen was also tried the other way (BF16 <-> FP8)
    assert sum(t > 0 for t in info["swap_ms"]) == (3 if metric == 0 else 0)
    # tensor-core precisions: the fused screen was timed for both groupings
    assert sum(t > 0 for t in info["fused_ms"]) == (2 if precision != S.PREC_FP64 else 0)
    for b in bufs:  # the plan's results are rewritten by the runs below
        b[1].fill_(7)
    plan.run()
    plan.wait()
    _check(oracle, metric, cols, bufs)
    plan.close()
    for db in dbs:
        db.close()


def test_ragged_plan_each_choice_and_no_graph(S, oracle):
    """Every (grouping, concurrency) choice the autotuner can keep, and the
    direct (no graph) form, give the same exact answers."""
    rng = np.random.default_rng(77)
    cols = _collections(rng)
    dbs = []
    for X, _, _ in cols:
        db = S.VectorDatabase(0, 3)
        db.insert_batch(X)
        dbs.append(db)
    parts, bufs = _bind(S, cols, dbs)
    plan = S.RaggedPlan(parts, 0, S.PREC_BF16, S.RAGGED_NO_GRAPH)
    assert plan.info()["graph"] == 0 and plan.info()["captures"] == 0
    plan.run()
    plan.wait()
    _check(oracle, 0, cols, bufs)
    plan.close()
    plan = S.RaggedPlan(parts, 0, S.PREC_BF16, 0)  # default choice, graph
    plan.run()
    plan.run()
    plan.wait()
    _check(oracle, 0, cols, bufs)
    plan.close()
    for db in dbs:
        db.close()


@pytest.mark.parametrize("metric", [0, 1, 2])
@pytest.mark.parametrize("flags", ["fused_by_class", "fused_per_part", "fused_no_graph", "fused_seeded"])
def test_ragged_fused_screen_matches_oracle(S, oracle, metric, flags):
    """The BF16 searches of every store screened by one fused launch (the
    schedule splits the launch's CTAs among the searches), with a
    fourth part on the first store so one store serves two searches of a
    class: exact answers for every query with its own k."""
    import torch
    rng = np.random.default_rng(900 + metric)
    cols = _collections(rng)
    X0 = cols[0][0]
    Qx = X0[rng.integers(0, X0.shape[0], 70)] + 0.01 * rng.normal(size=(70, X0.shape[1]))
    kx = rng.integers(1, 129, 70)
    kx[:3] = (128, 17, 2)
    dbs = []
    for X, _, _ in cols:
        db = S.VectorDatabase(0, 3)
        db.insert_batch(X)
        dbs.append(db)
    cols4 = cols + [(X0, Qx, kx)]
    parts, bufs = _bind(S, cols4, dbs + [dbs[0]])
    f = {"fused_by_class": S.RAGGED_FUSED | S.RAGGED_BY_K_CLASS, "fused_per_part": S.RAGGED_FUSED,
         "fused_no_graph": S.RAGGED_FUSED | S.RAGGED_BY_K_CLASS | S.RAGGED_NO_GRAPH,
         "fused_seeded": S.RAGGED_FUSED | S.RAGGED_BY_K_CLASS | S.RAGGED_SEED}[flags]
    plan = S.RaggedPlan(parts, metric, S.PREC_BF16, f)
    for b in bufs:
        b[1].fill_(7)
    plan.run()
    plan.run()
    plan.wait()
    info = plan.info()
    assert info["fused"] == 1 and info["seeded"] == (flags == "fused_seeded")
    # one launch holds up to 16 searches of any k: 12 searches (4 parts x 3
    # k classes) or 4 (one per part)
    assert info["fused_launches"] == 1
    st = plan.search_stats()  # per search: part, k, queries, fused, funnel of the last run
    assert st.shape == (info["searches"], 12) and (st[:, 3] == 1).all()
    assert (st[:, 2] > 0).all() and (st[:, 4] > 0).all() and (st[:, 8] == 0).all()
    assert sorted(set(st[:, 0].tolist())) == [0, 1, 2, 3]
    _check(oracle, metric, cols4, bufs)
    torch.cuda.synchronize()
    plan.close()
    for db in dbs:
        db.close()


def test_ragged_fused_screen_after_store_changes(S, oracle):
    """A fused plan is rebuilt for the stores' new shapes (more rows, fewer
    live rows) before the graph is captured again."""
    rng = np.random.default_rng(6)
    cols = _collections(rng)
    dbs = []
    for X, _, _ in cols:
        db = S.VectorDatabase(0, 3)
        db.insert_batch(X)
        dbs.append(db)
    parts, bufs = _bind(S, cols, dbs)
    plan = S.RaggedPlan(parts, 0, S.PREC_BF16, S.RAGGED_FUSED | S.RAGGED_BY_K_CLASS)
    plan.run()
    plan.wait()
    _check(oracle, 0, cols, bufs)
    X0, Q0, k0 = cols[0]
    extra = X0[:3000] + 1e-3 * rng.normal(size=(3000, X0.shape[1]))
    dbs[0].insert_batch(extra)
    cols[0] = (np.vstack([X0, extra]), Q0, k0)
    X1, Q1, k1 = cols[1]
    for i in (3, 40):
        dbs[1].delete(i)
    cols[1] = (np.delete(X1, [3, 41], axis=0), Q1, k1)
    plan.run()
    plan.wait()
    assert plan.info()["fused"] == 1
    _check(oracle, 0, cols, bufs)
    plan.close()
    for db in dbs:
        db.close()


def test_ragged_plan_recaptures_after_store_changes(S, oracle):
    """Mutations between runs are applied at the next run; a change the graph
    bakes in (more rows, fewer live rows) makes that run capture again."""
    rng = np.random.default_rng(5)
    cols = _collections(rng)
    dbs = []
    for X, _, _ in cols:
        db = S.VectorDatabase(0, 3)
        db.insert_batch(X)
        dbs.append(db)
    parts, bufs = _bind(S, cols, dbs)
    plan = S.RaggedPlan(parts, 1, S.PREC_BF16, 0)
    plan.run()
    plan.wait()
    _check(oracle, 1, cols, bufs)
    c0 = plan.info()["captures"]
    # grow the first store, delete from the second, overwrite in the third
    X0, Q0, k0 = cols[0]
    extra = X0[:500] + 1e-3 * rng.normal(size=(500, X0.shape[1]))
    dbs[0].insert_batch(extra)
    cols[0] = (np.vstack([X0, extra]), Q0, k0)
    X1, Q1, k1 = cols[1]
    for i in (0, 17, 4000):
        dbs[1].delete(i)
    cols[1] = (np.delete(X1, [0, 18, 4002], axis=0), Q1, k1)  # positions shift after each delete
    X2, Q2, k2 = cols[2]
    X2 = X2.copy()
    X2[5] = Q2[0]
    dbs[2].update(5, Q2[0])
    cols[2] = (X2, Q2, k2)
    plan.run()
    plan.wait()
    assert plan.info()["captures"] > c0
    _check(oracle, 1, cols, bufs)
    plan.close()
    for db in dbs:
        db.close()


def test_ragged_plan_rejects_bad_parts(S):
    import torch
    rng = np.random.default_rng(1)
    db = S.VectorDatabase(0, 3)
    db.insert_batch(rng.normal(size=(100, 16)))
    q = torch.zeros((4, 16), dtype=torch.float64, device="cuda")
    ids = torch.zeros((4, 8), dtype=torch.int64, device="cuda")
    dd = torch.zeros((4, 8), dtype=torch.float64, device="cuda")
    for ks, dim, stride in (([1, 2, 129, 4], 16, 200), ([1, 2, 9, 4], 16, 8), ([1, 0, 3, 4], 16, 8),
                            ([1, 2, 3, 4], 15, 8)):
        with pytest.raises(S.SvdbError):
            S.RaggedPlan([(db, q.data_ptr(), 4, dim, ks, ids.data_ptr(), dd.data_ptr(), stride)], 0, 1, 0)
    db.close()
