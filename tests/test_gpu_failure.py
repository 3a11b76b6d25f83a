"""Failure reporting on the GPU, without a fault: a kernel whose bounded wait
runs out (mbarriers nothing arrives on) and a device allocation the driver
refuses.  Each must come back as a status code and a message, and leave the
context and the store usable -- the same store then answers a search
identical to the oracle's."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S(svdb):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return svdb


def _store(S, rng, n=4000, d=64):
    X = rng.normal(size=(n, d))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    return db, X


def _search_ok(S, oracle, db, X, rng):
    Q = rng.normal(size=(5, X.shape[1]))
    for prec in (S.PREC_BF16, S.PREC_FP64):
        ids, vals = db.search(Q, 10, S.EUCLIDEAN, prec)
        wid, wval = oracle.topk(S.EUCLIDEAN, X, Q, 10)
        assert np.array_equal(ids, wid) and np.array_equal(vals, wval)


def test_bounded_wait_times_out_and_context_survives(S, oracle):
    rng = np.random.default_rng(5)
    db, X = _store(S, rng)
    _search_ok(S, oracle, db, X, rng)
    for limit_us in (20_000, 2_000):
        t0 = time.perf_counter()
        rc, gave_up, msg = db.selftest_bounded_wait(limit_us)
        dt = time.perf_counter() - t0
        assert rc == S.ETIMEOUT, (rc, msg)
        assert gave_up == 3  # the short wait ran out and the long one left through the abort flag
        assert "bounded wait" in msg
        assert dt < 1.5  # far below the 2 s limit of the second wait
        _search_ok(S, oracle, db, X, rng)  # error word cleared, TMEM released
    db.close()


def test_device_allocation_refused_is_enomem(S, oracle):
    rng = np.random.default_rng(6)
    db, X = _store(S, rng)
    for rows in (1 << 36, 1 << 58):  # 36 TB of FP64 rows at d=64, and a count past the address space
        with pytest.raises(S.SvdbError) as ei:
            db.reserve(rows, X.shape[1])
        assert f"({S.ENOMEM})" in str(ei.value)
    _search_ok(S, oracle, db, X, rng)
    more = rng.normal(size=(300, X.shape[1]))
    db.insert_batch(more)  # the store still grows normally afterwards
    _search_ok(S, oracle, db, np.concatenate([X, more]), rng)
    db.close()
