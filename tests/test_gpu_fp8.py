"""GPU parity of the FP8-E4M3 cosine screen (SVDB_PREC_FP8).

The unit-norm shadow is stored as E4M3 of 256 x/|x|; queries are scaled by a
power of two, so keys are the accumulator times an exact power of two.  Bar:
the same as the BF16 screen -- ids identical to the FP64 oracle (ties to the
lowest index), FP64 values bit-identical to the oracle's canonical order, the
certified bound never failing against the exact value -- on near-tie
mixtures, after mutations, with k up to 128; dot and Euclidean searches with
this precision run the BF16 screen and are exact too; data the FP8 bound
cannot separate (uniform rows) falls back to the exact FP64 scan.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PREC_FP8 = 2


@pytest.fixture(scope="module")
def S(svdb):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return svdb


def _mixture(rng, n, d, centres, sigma=0.05):
    C = rng.normal(size=(centres, d))
    return C, C[rng.integers(0, centres, n)] + sigma * rng.normal(size=(n, d))


def _search(S, db, Q, k, metric=0):
    st = S.SearchStats()
    ids, vals = db.search(Q, k, metric, PREC_FP8, stats=st)
    return ids, vals, st


@pytest.mark.parametrize("d", [64, 128, 200, 768])
def test_fp8_cosine_mixture_near_ties(S, oracle, d):
    rng = np.random.default_rng(80 + d)
    n = 30000 if d <= 200 else 12000
    C, X = _mixture(rng, n, d, 32)
    Q = C[rng.integers(0, 32, 300)] + 0.05 * rng.normal(size=(300, d))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    for k in (1, 10, 100):
        ids, vals, st = _search(S, db, Q, k)
        wid, wval = oracle.topk(0, X, Q, k)
        assert np.array_equal(ids, wid), (k, st.widened)
        assert np.array_equal(vals, wval), k
        assert st.bound_failures == 0
        assert st.widened == 0, (k, st.widened)
    db.close()


def test_fp8_query_tiles_mutations_and_k128(S, oracle):
    rng = np.random.default_rng(81)
    C, X = _mixture(rng, 9000 + 77, 96, 20)
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    rows = list(X)
    for i in (5, 4000, 9000):
        db.delete(i)
        del rows[i]
    for i in (0, 17, 3333):
        v = C[i % 20] + 0.05 * rng.normal(size=96)
        db.update(i, v)
        rows[i] = v
    Xc = np.stack(rows)
    for nq in (1, 127, 129, 520):
        Q = C[rng.integers(0, 20, nq)] + 0.05 * rng.normal(size=(nq, 96))
        for k in (16, 33, 128):
            ids, vals, st = _search(S, db, Q, k)
            wid, wval = oracle.topk(0, Xc, Q, k)
            assert np.array_equal(ids, wid), (nq, k)
            assert np.array_equal(vals, wval), (nq, k)
            assert st.bound_failures == 0
    db.close()


def test_fp8_other_metrics_and_unseparable_data(S, oracle):
    rng = np.random.default_rng(82)
    C, X = _mixture(rng, 8000, 128, 16)
    Q = C[rng.integers(0, 16, 100)] + 0.05 * rng.normal(size=(100, 128))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    for metric in (1, 2):  # the BF16 screen answers these
        ids, vals, st = _search(S, db, Q, 10, metric)
        wid, wval = oracle.topk(metric, X, Q, 10)
        assert np.array_equal(ids, wid) and np.array_equal(vals, wval), metric
        assert st.bound_failures == 0
    db.close()
    U = rng.uniform(-1, 1, (20000, 64))  # no clusters: the FP8 bound admits too much, the exact scan answers
    Qu = rng.uniform(-1, 1, (50, 64))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(U)
    ids, vals, st = _search(S, db, Qu, 10)
    wid, wval = oracle.topk(0, U, Qu, 10)
    assert np.array_equal(ids, wid) and np.array_equal(vals, wval)
    assert st.bound_failures == 0
    db.close()
