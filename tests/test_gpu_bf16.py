"""GPU parity of the BF16 tensor-core screen + certified FP64 re-rank.

Bar: ids identical to the FP64 oracle (ties to the lowest index) and FP64
values bit-identical to the oracle's canonical order, on data built to have
near-ties (Gaussian mixtures with sigma 0.05), exact duplicates, partial
tiles, query batches that cross the 128-query tile, deletes and updates.
Queries the screen cannot certify must still come back exact (through the
FP64 scan) and be counted in stats.widened; the screen's error bound must
never fail against the exact value (stats.bound_failures == 0).
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


def _search_both(S, db, Q, k, metric):
    st = S.SearchStats()
    ids, vals = db.search(Q, k, metric, S.PREC_BF16, stats=st)
    return ids, vals, st


@pytest.mark.parametrize("metric", [0, 1, 2])
@pytest.mark.parametrize("d", [64, 128, 200, 768])
def test_bf16_mixture_near_ties(S, oracle, metric, d):
    rng = np.random.default_rng(50 + d + metric)
    n = 30000 if d <= 200 else 12000
    C, X = _mixture(rng, n, d, 32)
    Q = C[rng.integers(0, 32, 40)] + 0.05 * rng.normal(size=(40, d))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    for k in (1, 10):
        ids, vals, st = _search_both(S, db, Q, k, metric)
        wid, wval = oracle.topk(metric, X, Q, k)
        assert np.array_equal(ids, wid), (k, st.widened)
        assert np.array_equal(vals, wval)
        assert st.bound_failures == 0
        assert st.widened < Q.shape[0]  # the screen answered at least part of the batch
    db.close()


@pytest.mark.parametrize("nq", [1, 127, 128, 129, 300])
def test_bf16_query_tiles_and_partial_row_tiles(S, oracle, nq):
    rng = np.random.default_rng(nq)
    X = rng.uniform(-1, 1, (10_000 + 37, 96))  # not a multiple of the 256-row tile
    Q = rng.uniform(-1, 1, (nq, 96))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    for metric in range(3):
        ids, vals, st = _search_both(S, db, Q, 10, metric)
        wid, wval = oracle.topk(metric, X, Q, 10)
        assert np.array_equal(ids, wid) and np.array_equal(vals, wval), metric
        assert st.bound_failures == 0 and st.widened == 0
    db.close()


def test_bf16_duplicates_tie_to_lowest_index(S, oracle):
    rng = np.random.default_rng(9)
    X = rng.normal(size=(5000, 32))
    for i in range(0, 60, 3):
        X[4000 + i] = X[i]  # exact duplicates at higher indices
    Q = X[:60:3] + 1e-9
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    for metric in range(3):
        for k in (2, 16, 32):
            ids, vals, st = _search_both(S, db, Q, k, metric)
            wid, wval = oracle.topk(metric, X, Q, k)
            assert np.array_equal(ids, wid) and np.array_equal(vals, wval), (metric, k)
    db.close()


def test_bf16_after_deletes_and_updates(S, oracle):
    rng = np.random.default_rng(31)
    C, X = _mixture(rng, 20000, 64, 16)
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    host = list(X)
    for step in range(400):
        i = int(rng.integers(0, len(host)))
        if step % 4 == 0:
            v = C[rng.integers(0, 16)] + 0.05 * rng.normal(size=64)
            db.update(i, v)
            host[i] = v
        else:
            db.delete(i)
            host.pop(i)
    H = np.stack(host)
    Q = C[rng.integers(0, 16, 25)] + 0.05 * rng.normal(size=(25, 64))
    for metric in range(3):
        ids, vals, st = _search_both(S, db, Q, 10, metric)
        wid, wval = oracle.topk(metric, H, Q, 10)
        assert np.array_equal(ids, wid) and np.array_equal(vals, wval), metric
    db.close()


def test_bf16_large_k_and_degenerate_queries_fall_back(S, oracle):
    rng = np.random.default_rng(17)
    X = rng.normal(size=(3000, 48))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    Q = rng.normal(size=(4, 48))
    Q[1] = 0.0  # zero query: cosine undefined for every row -> exact scan
    Q[2, 5] = np.nan
    for metric in range(3):
        for k in (10, 100, 128):
            ids, vals, st = _search_both(S, db, Q, k, metric)
            wid, wval = oracle.topk(metric, X, Q, k)
            assert np.array_equal(ids, wid), (metric, k)
            same = (vals == wval) | (np.isnan(vals) & np.isnan(wval))
            assert same.all(), (metric, k)
            assert st.widened >= 1  # at least the NaN query goes to the exact scan
    db.close()


@pytest.mark.parametrize("metric", [0, 1, 2])
def test_bf16_large_k_near_ties(S, oracle, metric):
    """k = 33 .. 128: the screen runs without its per-thread running top-k
    (thresholds from the shared bins) and still certifies every query."""
    rng = np.random.default_rng(300 + metric)
    C, X = _mixture(rng, 40000, 128, 16)
    Q = C[rng.integers(0, 16, 30)] + 0.05 * rng.normal(size=(30, 128))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    for k in (33, 48, 64, 65, 100, 128):
        ids, vals, st = _search_both(S, db, Q, k, metric)
        wid, wval = oracle.topk(metric, X, Q, k)
        assert np.array_equal(ids, wid) and np.array_equal(vals, wval), k
        assert st.widened == 0 and st.bound_failures == 0, k
    db.close()


def test_bf16_small_store_and_unscreenable_rows(S, oracle):
    rng = np.random.default_rng(23)
    X = rng.normal(size=(6, 40))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    ids, vals, st = _search_both(S, db, X[:3], 10, 1)  # k > rows: -1 / NaN tail
    wid, wval = oracle.topk(1, X, X[:3], 10)
    assert np.array_equal(ids, wid) and (ids[:, 6:] == -1).all()
    db.insert(np.full(40, 1e200))  # beyond what the BF16 screen can bound
    X2 = np.concatenate([X, np.full((1, 40), 1e200)])
    ids, vals, st = _search_both(S, db, X[:3], 3, 2)
    wid, wval = oracle.topk(2, X2, X[:3], 3)
    assert np.array_equal(ids, wid) and st.widened == 3
    db.close()


def test_bf16_values_within_fp64_tolerance(S, oracle):
    """Reported distances agree with the sequential FP64 formulas to 1e-12 relative."""
    rng = np.random.default_rng(71)
    C, X = _mixture(rng, 8000, 128, 8)
    Q = X[rng.integers(0, 8000, 10)] + 0.01 * rng.normal(size=(10, 128))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    for metric in range(3):
        ids, vals, err = db.search(Q, 10, metric, S.PREC_BF16, with_err=True)
        for qi in range(10):
            for j in range(10):
                s = oracle.fp64(metric, Q[qi], X[ids[qi, j]], seq=True)
                assert abs(vals[qi, j] - s) <= 1e-12 * max(1.0, abs(s))
                assert abs(vals[qi, j] - s) <= err[qi, j] + abs(s) * 2**-52
    db.close()


def test_bf16_cosine_dead_and_zero_rows(S, oracle):
    """The cosine screen masks rows that are deleted, zero (cosine NaN, ranked
    last) or tile padding; none may be emitted or lower a threshold, even while
    the running threshold is still -inf."""
    rng = np.random.default_rng(29)
    X = rng.normal(size=(1000, 64))
    X[[3, 300, 301]] = 0.0
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    host = list(X)
    for _ in range(250):  # empty most of the first 256-row tile
        db.delete(0)
        host.pop(0)
    H = np.stack(host)
    Q = rng.normal(size=(9, 64))
    for k in (1, 5, 32):
        ids, vals, st = _search_both(S, db, Q, k, 0)
        wid, wval = oracle.topk(0, H, Q, k)
        assert np.array_equal(ids, wid) and np.array_equal(vals, wval), k
        assert st.bound_failures == 0
    # tiny store: 10 live rows, 2 of them zero -> the k=10 answer has NaN tails
    small = S.VectorDatabase(0, 3)
    Y = rng.normal(size=(10, 16))
    Y[[2, 7]] = 0.0
    small.insert_batch(Y)
    ids, vals, st = _search_both(S, small, Y[:3] + 0.1, 10, 0)
    wid, wval = oracle.topk(0, Y, Y[:3] + 0.1, 10)
    assert np.array_equal(ids, wid)
    assert ((vals == wval) | (np.isnan(vals) & np.isnan(wval))).all()
    small.close()
    db.close()


@pytest.mark.parametrize("metric", [0, 1, 2])
def test_bf16_grouped_refinement(S, oracle, metric):
    """Batches larger than two queries per SM: queries sorted by survivor
    signature and refined in groups of up to 4 sharing a signature (each
    distinct row read once per group).  Uneven clusters (a few hundred to
    2,600 near-ties: groups past 4,096 survivor entries take the one-query-
    at-a-time path) and queries between two centres (survivors from two
    clusters, so group members' survivor sets differ) on the same batch."""
    rng = np.random.default_rng(700 + metric)
    d = 60
    C = rng.normal(size=(40, d))
    sizes = np.concatenate([rng.integers(100, 900, 34), rng.integers(1500, 2600, 6)])
    X = np.concatenate([C[c] + 0.05 * rng.normal(size=(n, d)) for c, n in enumerate(sizes)])
    X = X[rng.permutation(len(X))]
    which = rng.integers(0, 40, 600)
    Q = C[which] + 0.05 * rng.normal(size=(600, d))
    Q[::7] = 0.5 * (C[which[::7]] + C[(which[::7] + 1) % 40]) + 0.05 * rng.normal(size=(len(Q[::7]), d))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    for k in (1, 10, 32):
        ids, vals, st = _search_both(S, db, Q, k, metric)
        wid, wval = oracle.topk(metric, X, Q, k)
        assert np.array_equal(ids, wid), k
        assert np.array_equal(vals, wval), k
        assert st.bound_failures == 0 and st.widened == 0, k
    db.close()


@pytest.mark.parametrize("metric", [0, 1, 2])
def test_bf16_separated_top_rows_in_first_tiles(S, oracle, metric):
    """Well-separated best rows (gaps far wider than the screen's bound) in the
    first tile and further on, a small store whose segments are single tiles
    (every tile is a warm-up tile): the shared running thresholds must never
    count one row twice, or the second-best row would be cut."""
    rng = np.random.default_rng(11 + metric)
    X = rng.normal(size=(5000, 128))
    q = rng.normal(size=128)
    X[16] = q
    X[3000] = 0.9 * q + 0.05 * rng.normal(size=128)
    X[4900] = 0.8 * q + 0.05 * rng.normal(size=128)
    Q = np.stack([q, q + 1e-3 * rng.normal(size=128)])
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    for k in (2, 3, 5):
        wid, wval = oracle.topk(metric, X, Q, k)
        for _ in range(10):
            ids, vals, st = _search_both(S, db, Q, k, metric)
            assert np.array_equal(ids, wid), (k, ids, wid)
            assert np.array_equal(vals, wval)
            assert st.bound_failures == 0
    db.close()


@pytest.mark.parametrize("d", [768, 1000])
def test_bf16_grouped_refinement_wide_rows(S, oracle, d):
    """Grouped refinement at wide rows (768: 12 float4 per lane; 1000: rows
    padded to 1008, 16 per lane): 400 queries over 20 clusters, ids and
    values identical to the oracle for k = 10 and 100."""
    rng = np.random.default_rng(900 + d)
    C = rng.normal(size=(20, d))
    X = C[rng.integers(0, 20, 6000)] + 0.05 * rng.normal(size=(6000, d))
    Q = C[rng.integers(0, 20, 400)] + 0.05 * rng.normal(size=(400, d))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    for metric in (0, 1):
        for k in (10, 100):
            ids, vals, st = _search_both(S, db, Q, k, metric)
            wid, wval = oracle.topk(metric, X, Q, k)
            assert np.array_equal(ids, wid), (metric, k)
            assert np.array_equal(vals, wval), (metric, k)
            assert st.bound_failures == 0 and st.widened == 0, (metric, k)
    db.close()


@pytest.mark.parametrize("d", [64, 200, 768, 1536])
def test_bf16_streamed_few_queries(S, oracle, d):
    """A single cosine query takes the CUDA-core streamed screen (2 to 5 take
    the tensor-core one): near-tie mixtures, every k class, exact
    duplicates, zero and deleted rows, a partial last tile, and a query that
    is zero (its cosines are NaN: no candidates, answered by the FP64 scan).
    Every single-query cosine search of the other tests takes it too."""
    rng = np.random.default_rng(900 + d)
    C, X = _mixture(rng, 20_000 + 77, d, 16)
    X[[5, 9000]] = 0.0
    X[12000] = X[11999]  # an exact duplicate: ties to the lower index
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    host = list(X)
    for i in (0, 100, 15000):
        db.delete(i)
        host.pop(i)
    H = np.stack(host)
    for nq in (1, 2, 3, 4, 5):
        Q = C[rng.integers(0, 16, nq)] + 0.05 * rng.normal(size=(nq, d))
        if nq == 3:
            Q[1] = H[11998] * 2.0  # the duplicated row's direction: two exact ties at the top
        if nq == 4:
            Q[2] = 0.0
        for k in (1, 10, 33, 100, 128):
            ids, vals, st = _search_both(S, db, Q, k, 0)
            wid, wval = oracle.topk(0, H, Q, k)
            assert np.array_equal(ids, wid), (nq, k, st.widened)
            assert ((vals == wval) | (np.isnan(vals) & np.isnan(wval))).all(), (nq, k)
            assert st.bound_failures == 0
            zero = 1 if nq == 4 else 0
            if k <= 33:  # answered by the screen (not the FP64 scan), but for the zero query
                assert st.widened == zero, (nq, k, st.widened)
            else:
                assert st.widened <= zero + (nq - zero) // 2, (nq, k, st.widened)
    Z = np.zeros((1, d))  # a lone zero query on the streamed path: no candidates, the FP64 scan answers
    ids, vals, st = _search_both(S, db, Z, 10, 0)
    wid, wval = oracle.topk(0, H, Z, 10)
    assert np.array_equal(ids, wid)
    assert ((vals == wval) | (np.isnan(vals) & np.isnan(wval))).all()
    assert st.widened == 1 and st.bound_failures == 0
    db.close()


def test_paired_screen_matches_oracle_in_its_own_process(S):
    """The paired (cta_group::2) screen is opt-in (SVDB_SCREEN_PAIR=1, read
    once per process), so it runs in a child process: BF16 and FP8, cosine and
    Euclidean, batches of 300 and 1024 queries (several pair tiles) on a
    near-tie mixture, against the oracle."""
    import os
    import subprocess
    import sys
    code = r'''
import sys, numpy as np
sys.path[:0] = sys.argv[1:]
import oracle as O, svdb_gb300 as S
o = O.Oracle()
rng = np.random.default_rng(61)
C = rng.normal(size=(40, 256))
X = C[rng.integers(0, 40, 60000)] + 0.05 * rng.normal(size=(60000, 256))
db = S.VectorDatabase(0, 3)
db.insert_batch(X)
db.set_fp8_screen(1)
for nq in (300, 1024):
    Q = C[rng.integers(0, 40, nq)] + 0.05 * rng.normal(size=(nq, 256))
    for metric in (0, 1):
        wi, wv = o.topk(metric, X, Q, 10)
        for prec in (S.PREC_BF16, S.PREC_FP8):
            st = S.SearchStats()
            ids, vals = db.search(Q, 10, metric, prec, stats=st)
            assert np.array_equal(ids, wi) and np.array_equal(vals, wv), (nq, metric, prec)
            assert st.bound_failures == 0 and st.widened < nq
print("paired ok")
'''
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    paths = [os.path.join(root, "oracle"), os.path.join(root, "simple-vector-db_gb300")]
    env = dict(os.environ, SVDB_SCREEN_PAIR="1")
    r = subprocess.run([sys.executable, "-c", code, *paths], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "paired ok" in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]


@pytest.mark.parametrize("metric", [0, 1, 2])
def test_bf16_seeded_thresholds(S, oracle, metric):
    """svdb_set_screen_seeding: the BF16 screen's thresholds start from the
    exact k-th best lower bound of a 1/16 sample of the store; the answers
    are the oracle's either way, and the sample prunes candidates."""
    rng = np.random.default_rng(700 + metric)
    X = rng.uniform(-1, 1, (60_000, 64))  # uniform rows: many near-ties for large k
    Q = rng.uniform(-1, 1, (300, 64))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    wid, wval = oracle.topk(metric, X, Q, 100)
    cands = []
    for mode in (0, 1):
        db.set_screen_seeding(mode)
        for k in (16, 100):
            st = S.SearchStats()
            ids, vals = db.search(Q, k, metric, S.PREC_BF16, stats=st)
            assert np.array_equal(ids, wid[:, :k]), (mode, k)
            assert np.array_equal(vals, wval[:, :k]), (mode, k)
            assert st.bound_failures == 0 and st.widened == 0
            if k == 100:
                cands.append(st.candidates)
    assert cands[1] < cands[0]  # seeded thresholds emit fewer candidates
    db.close()


@pytest.mark.parametrize("metric", [0, 1, 2])
def test_bf16_shallow_store_one_query_tile_on_every_cta(S, oracle, metric):
    """A D = 64 store of 100,000 rows (391 tiles of 256) and a batch of one
    query tile: the two-CTA-per-SM screen splits the tile over ~300 CTAs,
    each writing two candidate sub-lists, so the select's prefix over the
    sub-lists holds ~600 counts.  Answers equal the oracle's."""
    rng = np.random.default_rng(720 + metric)
    C = rng.normal(size=(64, 64))
    X = C[rng.integers(0, 64, 100_000)] + 0.05 * rng.normal(size=(100_000, 64))
    Q = C[rng.integers(0, 64, 5)] + 0.05 * rng.normal(size=(5, 64))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    for k in (1, 10, 100):
        wid, wval = oracle.topk(metric, X, Q, k)
        st = S.SearchStats()
        ids, vals = db.search(Q, k, metric, S.PREC_BF16, stats=st)
        assert np.array_equal(ids, wid) and np.array_equal(vals, wval), k
        assert st.bound_failures == 0
    db.close()
