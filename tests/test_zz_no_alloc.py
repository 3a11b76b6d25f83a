"""The search entry point that allocates no device memory.

Some callers cannot call cudaMalloc (an allocator hook or pool that owns every
device byte, a latency-critical path that must not take the driver's
allocation lock).  svdb_search_topk_fp64_noalloc keeps its per-call scratch
in a fixed 16 MiB device array instead; its results must equal the oracle's
exact top-k (ids, and FP64 values bit for bit) and the regular device
search's, on consecutive calls that reuse the array; after a first search has
loaded the kernels' code, calls must leave free device memory unchanged; and
requests larger than the array must be refused.

Collected last (file name) so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S(svdb):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return svdb


def _regular(S, db, qd, k, metric):
    import torch
    nq, d = qd.shape
    ids = torch.empty((nq, k), dtype=torch.int64, device="cuda")
    dists = torch.empty((nq, k), dtype=torch.float64, device="cuda")
    db.search_device(qd.data_ptr(), nq, d, k, metric, S.PREC_FP64, ids.data_ptr(), dists.data_ptr())
    db.wait()
    return ids.cpu().numpy(), dists.cpu().numpy()


def _noalloc(S, db, qd, k, metric):
    import torch
    nq, d = qd.shape
    ids = torch.full((nq, k), -7, dtype=torch.int64, device="cuda")
    dists = torch.full((nq, k), 7.0, dtype=torch.float64, device="cuda")
    db.search_fp64_noalloc(qd.data_ptr(), nq, d, k, metric, ids.data_ptr(), dists.data_ptr())
    db.wait()
    return ids.cpu().numpy(), dists.cpu().numpy()


def test_noalloc_matches_oracle_and_regular_search_on_consecutive_calls(S, oracle):
    import torch
    rng = np.random.default_rng(404)
    X = rng.normal(size=(20000, 96))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    keep = np.ones(X.shape[0], bool)
    for i in range(0, 300, 7):
        db.delete(i)  # positional ids shift, as in the reference
        keep[np.flatnonzero(keep)[i]] = False
    Xl = X[keep]  # the rows in their current positional order
    db.sync()
    torch.cuda.synchronize()
    for call, (nq, k, metric) in enumerate([(17, 10, 0), (33, 32, 1), (5, 100, 2), (17, 10, 0)]):
        Q = rng.normal(size=(nq, 96))
        qd = torch.from_numpy(Q).cuda()
        want_ids, want_d = _regular(S, db, qd, k, metric)
        got_ids, got_d = _noalloc(S, db, qd, k, metric)
        o_ids, o_d = oracle.topk(metric, Xl, Q, k)
        assert np.array_equal(got_ids, o_ids), call  # ids exact, ties to the lowest position
        assert np.array_equal(got_d, o_d), call      # FP64 values bit-identical to the oracle (tolerance 0)
        assert np.array_equal(got_ids, want_ids), call
        assert np.array_equal(got_d, want_d), call
    db.close()


def test_noalloc_allocates_nothing_after_the_first_search(S):
    """Free device memory is the same before and after a run of calls (once
    the scan kernels' code is loaded by a first search), and the results of
    the calls stay identical."""
    import torch
    rng = np.random.default_rng(406)
    X = rng.normal(size=(30000, 128))
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    db.sync()
    nq, k = 24, 16
    qd = torch.from_numpy(rng.normal(size=(nq, 128))).cuda()
    ids = torch.empty((nq, k), dtype=torch.int64, device="cuda")
    dists = torch.empty((nq, k), dtype=torch.float64, device="cuda")
    db.search_fp64_noalloc(qd.data_ptr(), nq, 128, k, 1, ids.data_ptr(), dists.data_ptr())  # loads kernel code
    db.wait()
    first = (ids.cpu().numpy(), dists.cpu().numpy())
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(20):
        for metric in (0, 1, 2):
            db.search_fp64_noalloc(qd.data_ptr(), nq, 128, k, metric, ids.data_ptr(), dists.data_ptr())
    db.wait()
    free1, _ = torch.cuda.mem_get_info()
    db.search_fp64_noalloc(qd.data_ptr(), nq, 128, k, 1, ids.data_ptr(), dists.data_ptr())
    db.wait()
    assert free1 == free0, (free0, free1)
    assert np.array_equal(ids.cpu().numpy(), first[0]) and np.array_equal(dists.cpu().numpy(), first[1])
    db.close()


def test_noalloc_refuses_oversized_requests_and_pending_changes(S):
    import torch
    rng = np.random.default_rng(405)
    db = S.VectorDatabase(0, 3)
    db.insert_batch(rng.normal(size=(5000, 2048)))
    db.sync()
    big = torch.zeros((2048, 2048), dtype=torch.float64, device="cuda")  # 32 MiB of queries alone
    ids = torch.empty((2048, 10), dtype=torch.int64, device="cuda")
    dists = torch.empty((2048, 10), dtype=torch.float64, device="cuda")
    with pytest.raises(S.SvdbError, match="scratch"):
        db.search_fp64_noalloc(big.data_ptr(), 2048, 2048, 10, 0, ids.data_ptr(), dists.data_ptr())
    db.insert(rng.normal(size=2048))  # staged, not yet on the device
    with pytest.raises(S.SvdbError, match="svdb_sync"):
        db.search_fp64_noalloc(big.data_ptr(), 1, 2048, 10, 0, ids.data_ptr(), dists.data_ptr())
    db.sync()
    db.search_fp64_noalloc(big.data_ptr(), 1, 2048, 10, 0, ids.data_ptr(), dists.data_ptr())
    db.wait()
    db.close()
