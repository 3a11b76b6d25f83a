"""Parity at the sizes the workloads are measured on, against the oracle.

The other GPU tests check the kernels on stores of up to ~300,000 rows.  The
schedule of the tensor-core screen depends on the batch and store shape (how
query tiles are split over the SMs, which CTAs take the tail rows of other
query tiles), so these tests run the measured shapes themselves and compare a
sample of queries with the oracle's FP64 brute force (ids equal with ties to
the lowest position, FP64 values bit-identical):

* 1M x 768 Gaussian mixture (1,024 centres, sigma 0.05, seed 3): Q = 1, 64,
  1024 and 4096 from the same mixture, top-10 cosine and Euclidean, BF16 and
  FP8 screens.  Sampled queries: three in every 128-query tile of the batch
  (its first, a random one and its last), so every tile of the schedule,
  including those whose tail rows go to helper CTAs, is checked.
* 1M x 128 L2-normalised N(0,1) rows (seed 2): single queries, top-1 and
  top-10, cosine / Euclidean / dot, through the plain FP64 scan.
* The ragged batch over five collections (D, N) = (64, 2M), (128, 1M),
  (384, 500k), (768, 200k), (1536, 50k), 8,192 queries with k per query in
  [1, 100] (seed 4): one autotuned ragged plan; a sample of every part
  against the oracle with each query's own k.

Each search's certification statistics are printed at the end of the run;
no bound may fail.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

K = 10


@pytest.fixture(scope="module")
def S(svdb):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return svdb


@pytest.fixture(scope="module")
def W():
    from svdb_gb300 import workloads
    return workloads


def _tile_sample(nq, rng):
    """Three queries per 128-query tile: its first, a random one, its last."""
    out = set()
    for t0 in range(0, nq, 128):
        t1 = min(nq, t0 + 128)
        out.update((t0, int(rng.integers(t0, t1)), t1 - 1))
    return np.array(sorted(out))


@pytest.fixture(scope="module")
def mixture_1m(S, W):
    mix, X = W.config3(1_000_000, 768, 3)
    Q = mix.sample(4096, 1)
    db = S.VectorDatabase(1_000_000, 3)
    db.reserve(1_000_000, 768)
    db.insert_batch(X)
    db.sync()
    db.set_fp8_screen(1)  # FP8 cases run the E4M3 screen at every batch size
    yield X, Q, db
    db.close()


@pytest.fixture(scope="module")
def mixture_oracle(mixture_1m, oracle):
    """The oracle's top-10 of every sampled query, per metric."""
    X, Q, _ = mixture_1m
    rng = np.random.default_rng(33)
    sample = np.union1d(_tile_sample(4096, rng), [0, 31, 63])
    want = {m: oracle.topk(m, X, Q[sample], K) for m in (0, 1)}
    return sample, want


@pytest.mark.parametrize("nq", [1, 64, 1024, 4096])
@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("prec", ["bf16", "fp8"])
def test_mixture_1m_x_768_against_oracle(S, mixture_1m, mixture_oracle, parity_report, nq, metric, prec):
    X, Q, db = mixture_1m
    sample, want = mixture_oracle
    p = S.PREC_BF16 if prec == "bf16" else S.PREC_FP8
    st = S.SearchStats()
    ids, vals = db.search(Q[:nq], K, metric, p, stats=st)
    rows = np.flatnonzero(sample < nq)
    got_i, got_v = ids[sample[rows]], vals[sample[rows]]
    w_i, w_v = want[metric][0][rows], want[metric][1][rows]
    assert np.array_equal(got_i, w_i), np.flatnonzero((got_i != w_i).any(1))
    assert np.array_equal(got_v, w_v)
    assert st.bound_failures == 0
    parity_report.append(f"1Mx768 mixture Q={nq} {('cosine', 'euclidean')[metric]} {prec}: {rows.size} sampled "
                         f"queries exact; per query {st.candidates / nq:.0f} candidates, {st.survivors / nq:.0f} "
                         f"survivors, {st.reranked / nq:.1f} re-ranked; widened {st.widened}, bound failures "
                         f"{st.bound_failures}")


@pytest.fixture(scope="module")
def scan_1m(S, W):
    X, Q = W.config2(1_000_000, 128, 10_000)
    db = S.VectorDatabase(1_000_000, 3)
    db.insert_batch(X)
    db.sync()
    yield X, Q, db
    db.close()


@pytest.mark.parametrize("metric", [0, 1, 2])
def test_scan_1m_x_128_single_queries_against_oracle(S, scan_1m, oracle, parity_report, metric):
    X, Q, db = scan_1m
    pick = np.random.default_rng(22 + metric).choice(Q.shape[0], 16, replace=False)
    w10 = oracle.topk(metric, X, Q[pick], 10)
    for k in (1, 10):
        for j, qi in enumerate(pick):  # one query per call, as the workload issues them
            ids, vals = db.search(Q[qi:qi + 1], k, metric, S.PREC_FP64)
            assert np.array_equal(ids[0], w10[0][j, :k]), (qi, k)
            assert np.array_equal(vals[0], w10[1][j, :k]), (qi, k)
    parity_report.append(f"1Mx128 scan {('cosine', 'euclidean', 'dot')[metric]}: 16 single queries x top-1/top-10 "
                         f"exact (FP64 scan)")


def test_ragged_five_collections_full_size_against_oracle(S, W, oracle, parity_report):
    import torch
    cols = W.config4(8192)
    dbs, bufs, parts = [], [], []
    for X, Q, ks in cols:
        db = S.VectorDatabase(X.shape[0], 3)
        db.insert_batch(X)
        db.sync()
        stride = int(ks.max())
        qd = torch.from_numpy(Q).cuda()
        ids = torch.full((Q.shape[0], stride), -7, dtype=torch.int64, device="cuda")
        dd = torch.full((Q.shape[0], stride), 7.0, dtype=torch.float64, device="cuda")
        dbs.append(db)
        bufs.append((qd, ids, dd))
        parts.append((db, qd.data_ptr(), Q.shape[0], Q.shape[1], ks, ids.data_ptr(), dd.data_ptr(), stride))
    torch.cuda.synchronize()
    plan = S.RaggedPlan(parts, S.COSINE, S.PREC_BF16, S.RAGGED_AUTOTUNE)
    for b in bufs:  # the autotuner's runs wrote the outputs: clear them
        b[1].fill_(-7)
        b[2].fill_(7.0)
    plan.run()
    plan.wait()
    info = plan.info()
    rng = np.random.default_rng(44)
    checked = 0
    for c, ((X, Q, ks), (_, ids, dd)) in enumerate(zip(cols, bufs)):
        nq = Q.shape[0]
        pick = np.union1d(rng.choice(nq, 12, replace=False), [0, nq - 1])
        pick = np.union1d(pick, np.flatnonzero(ks == ks.max())[:2])  # the part's largest k
        gi, gd = ids.cpu().numpy(), dd.cpu().numpy()
        for qi in pick:
            k = int(ks[qi])
            wi, wv = oracle.topk(S.COSINE, X, Q[qi:qi + 1], k)
            assert np.array_equal(gi[qi, :k], wi[0]), (c, qi, k)
            assert np.array_equal(gd[qi, :k], wv[0]), (c, qi, k)
            assert (gi[qi, k:] == -1).all() and np.isnan(gd[qi, k:]).all(), (c, qi, k)
            checked += 1
    plan.close()
    for db in dbs:
        db.close()
    parity_report.append(f"ragged 5 collections, 8192 queries (grouping {info['grouping']}, concurrent "
                         f"{info['concurrent']}, searches {info['searches']}): {checked} sampled queries exact "
                         f"with their own k")
