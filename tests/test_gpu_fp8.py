"""GPU parity of the FP8-E4M3 screens (SVDB_PREC_FP8).

Cosine screens an E4M3 copy of 256 x/|x|; dot and Euclidean screen an E4M3
copy of x 2^f_i, 2^f_i a per-row power of two (the largest with max |x_j|
2^f_i <= 448).  Queries are scaled by a power of two, so every key is the
accumulator times exact powers of two.  Bar: the same as the BF16 screen --
ids identical to the FP64 oracle (ties to the lowest index), FP64 values
bit-identical to the oracle's canonical order, the certified bound never
failing against the exact value -- on near-tie mixtures, rows of widely
different magnitudes, after mutations, with k up to 128; data the FP8
bound cannot separate (uniform rows) falls back to the exact FP64 scan.
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
    db.set_fp8_screen(1)  # the E4M3 screen at every batch size and k (the default rule picks by both)
    st = S.SearchStats()
    ids, vals = db.search(Q, k, metric, PREC_FP8, stats=st)
    return ids, vals, st


@pytest.mark.parametrize("metric", [0, 1, 2])
@pytest.mark.parametrize("d", [64, 128, 200, 768])
def test_fp8_mixture_near_ties(S, oracle, d, metric):
    rng = np.random.default_rng(80 + d + 7 * metric)
    n = 30000 if d <= 200 else 12000
    C, X = _mixture(rng, n, d, 32)
    Q = C[rng.integers(0, 32, 300)] + 0.05 * rng.normal(size=(300, d))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    for k in (1, 10, 100):
        ids, vals, st = _search(S, db, Q, k, metric)
        wid, wval = oracle.topk(metric, X, Q, k)
        assert np.array_equal(ids, wid), (k, st.widened)
        assert np.array_equal(vals, wval), k
        assert st.bound_failures == 0
        assert st.widened == 0, (k, st.widened)
    db.close()


@pytest.mark.parametrize("metric", [0, 1, 2])
def test_fp8_query_tiles_mutations_and_k128(S, oracle, metric):
    rng = np.random.default_rng(81 + metric)
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
            ids, vals, st = _search(S, db, Q, k, metric)
            wid, wval = oracle.topk(metric, Xc, Q, k)
            assert np.array_equal(ids, wid), (nq, k)
            assert np.array_equal(vals, wval), (nq, k)
            assert st.bound_failures == 0
    db.close()


@pytest.mark.parametrize("metric", [1, 2])
def test_fp8_per_row_scales_on_rows_of_every_magnitude(S, oracle, metric):
    """Rows scaled by 10^U[-12, 12] (their E4M3 scales 2^f span a range of
    2^80), a zero row, and rows of norm 1e-35 (scales clamped at 2^120, so
    their E4M3 copies lose most digits): the per-row scale and residual keep
    every bound valid, and the screen still answers the batch."""
    rng = np.random.default_rng(83 + metric)
    C, X = _mixture(rng, 12000, 96, 24)
    X *= 10.0 ** rng.uniform(-12, 12, (X.shape[0], 1))
    X[7] = 0.0
    X[100:110] *= 1e-35 / np.linalg.norm(X[100:110], axis=1, keepdims=True)
    Q = C[rng.integers(0, 24, 200)] + 0.05 * rng.normal(size=(200, 96))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    for k in (1, 10, 64):
        ids, vals, st = _search(S, db, Q, k, metric)
        wid, wval = oracle.topk(metric, X, Q, k)
        assert np.array_equal(ids, wid), (k, st.widened)
        assert np.array_equal(vals, wval), k
        assert st.bound_failures == 0
        assert st.widened < Q.shape[0], k
    db.close()


@pytest.mark.parametrize("metric", [0, 1, 2])
def test_fp8_unseparable_data_falls_back_exact(S, oracle, metric):
    rng = np.random.default_rng(82 + metric)
    U = rng.uniform(-1, 1, (20000, 64))  # no clusters: the FP8 bound admits too much, the exact scan answers
    Qu = rng.uniform(-1, 1, (50, 64))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(U)
    ids, vals, st = _search(S, db, Qu, 10, metric)
    wid, wval = oracle.topk(metric, U, Qu, 10)
    assert np.array_equal(ids, wid) and np.array_equal(vals, wval)
    assert st.bound_failures == 0
    db.close()


def test_fp8_default_rule_picks_the_screen(S, oracle):
    """svdb_set_fp8_screen(-1), the default: an FP8 search runs the E4M3
    screen only for batches of at least 1,024 queries with k <= 32, and the
    BF16 screen otherwise -- the same survivors and kernels as a BF16 search,
    and the same answers.  Mode 0 always takes the BF16 screen, mode 1 the E4M3 one."""
    rng = np.random.default_rng(90)
    C, X = _mixture(rng, 60_000, 128, 48)
    Q = C[rng.integers(0, 48, 1024)] + 0.05 * rng.normal(size=(1024, 128))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)

    def run(q, k, prec, mode):
        db.set_fp8_screen(mode)
        st = S.SearchStats()
        ids, vals = db.search(q, k, 0, prec, stats=st)
        return ids, vals, (st.survivors, st.kernels)  # (candidates depend on the running thresholds' timing)

    for nq, k, e4m3 in ((1024, 10, True), (1024, 32, True), (1024, 33, False), (300, 10, False), (1, 10, False)):
        wid, wval = oracle.topk(0, X, Q[:nq], k)
        bi, bv, bst = run(Q[:nq], k, S.PREC_BF16, -1)
        di, dv, dst = run(Q[:nq], k, PREC_FP8, -1)
        fi, fv, fst = run(Q[:nq], k, PREC_FP8, 1)
        zi, zv, zst = run(Q[:nq], k, PREC_FP8, 0)
        for ids, vals in ((bi, bv), (di, dv), (fi, fv), (zi, zv)):
            assert np.array_equal(ids, wid) and np.array_equal(vals, wval), (nq, k)
        assert zst == bst, (nq, k)                   # mode 0: the BF16 screen
        assert (dst == fst) if e4m3 else (dst == bst), (nq, k, dst, fst, bst)
        assert fst != bst, (nq, k)                   # mode 1: the E4M3 screen (another funnel)
    db.close()
