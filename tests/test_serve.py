"""Serving layer: request layouts, trace generation (CPU) and a mixed request
trace served in batches on the GPU, checked against the oracle's positional
store replaying the same serial order (mutations of a batch in request order,
then its reads)."""
import ctypes as C

import numpy as np
import pytest

ROWS_D = 48


def test_request_layouts_match_the_c_structs(svdb):
    from svdb_gb300 import serve
    assert serve.REQ_DTYPE.itemsize == 48 and serve.RESP_DTYPE.itemsize == 16
    assert [serve.REQ_DTYPE.fields[f][1] for f in ("op", "metric", "k", "a", "b", "vec", "uuid")] == \
        [0, 4, 8, 16, 24, 32, 40]
    assert [serve.RESP_DTYPE.fields[f][1] for f in ("status", "value", "index")] == [0, 4, 8]


def test_trace_is_seeded_and_follows_the_mix(svdb):
    from svdb_gb300 import serve, workloads
    m = workloads.Mixture(16, 5, ncentres=4)
    a = serve.make_trace(m.sample, 500, 40000, 20000.0, 9)
    b = serve.make_trace(m.sample, 500, 40000, 20000.0, 9)
    assert np.array_equal(a.arrival, b.arrival) and np.array_equal(a.req[["op", "metric", "k", "a", "b"]],
                                                                    b.req[["op", "metric", "k", "a", "b"]])
    assert np.array_equal(a.rows, b.rows)
    frac = np.bincount(a.req["op"], minlength=5) / len(a)
    assert np.allclose(frac, serve.DEFAULT_MIX, atol=0.01)
    assert abs(len(a) / a.arrival[-1] - 20000.0) < 600  # Poisson rate
    # every vec pointer lands on a row of the trace's own matrix
    vec = a.req["vec"][a.req["vec"] != 0]
    off = (vec - np.uint64(a.rows.ctypes.data)) // np.uint64(16 * 8)
    assert off.max() < a.rows.shape[0] and len(np.unique(off)) == len(off)


def test_server_needs_a_gpu(svdb):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from svdb_gb300 import serve
    with pytest.raises(svdb.SvdbError, match="CUDA"):
        serve.Server(8, 100)


def _sampler(d, centres=8, seed=0):
    C_ = np.random.default_rng(seed).normal(size=(centres, d))

    def sample(m, stream):
        g = np.random.default_rng([seed, stream])
        return C_[g.integers(0, centres, m)] + 0.05 * g.normal(size=(m, d))
    return sample


def _check_batch(S, oracle, ostore, batch, resp, ids, dists, rows_of):
    from svdb_gb300 import serve
    for r, o in zip(batch, resp):
        op = int(r["op"])
        if op == serve.REQ_INSERT:
            assert o["status"] == 0 and int(o["index"]) == ostore.size
            ostore.insert(rows_of(r))
        elif op in (serve.REQ_UPDATE, serve.REQ_DELETE):
            if int(r["a"]) >= ostore.size:
                assert o["status"] == S.CMP_OUT_OF_BOUNDS
            else:
                assert o["status"] == 0
                if op == serve.REQ_UPDATE:
                    ostore.update(int(r["a"]), rows_of(r))
                else:
                    ostore.delete(int(r["a"]))
    H = ostore.rows()
    for i, (r, o) in enumerate(zip(batch, resp)):
        op = int(r["op"])
        if op == serve.REQ_NEAREST:
            k = int(r["k"])
            wid, wval = oracle.topk(int(r["metric"]), H, rows_of(r)[None], k)
            assert o["status"] == 0
            assert np.array_equal(ids[i, :k], wid[0]), (i, int(r["metric"]), k)
            assert np.array_equal(dists[i, :k], wval[0])
        elif op == serve.REQ_COMPARE:
            a, b, m = int(r["a"]), int(r["b"]), int(r["metric"])
            if a >= len(H) or b >= len(H):
                assert o["status"] == S.CMP_OUT_OF_BOUNDS
            elif m > 2:
                assert o["status"] == S.CMP_UNKNOWN_METHOD
            else:
                w = oracle.ref_metric(m, H[a], H[b])
                assert o["status"] == 0
                assert np.float32(o["value"]).tobytes() == np.float32(w).tobytes(), (a, b, m)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_gpu_server_trace_matches_oracle(svdb, oracle, precision):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from svdb_gb300 import serve
    S = svdb
    d = ROWS_D
    sample = _sampler(d)
    X0 = sample(3000, 1)
    srv = serve.Server(d, 2048)  # smaller than the trace needs: the store grows during the batches
    srv.insert_block(X0)
    tr = serve.make_trace(sample, 3000, 2500, 1e6, seed=3, mix=(0.4, 0.2, 0.2, 0.1, 0.1))
    rng = np.random.default_rng(4)
    near = np.flatnonzero(tr.req["op"] == serve.REQ_NEAREST)
    tr.req["metric"][near] = rng.integers(0, 3, near.size)
    tr.req["k"][near] = rng.choice([1, 10, 32], near.size)
    cmpi = np.flatnonzero(tr.req["op"] == serve.REQ_COMPARE)
    tr.req["a"][cmpi[:5]] = 10**9  # past the end
    tr.req["metric"][cmpi[5:8]] = 7  # unknown method
    muts = np.flatnonzero(np.isin(tr.req["op"], [serve.REQ_UPDATE, serve.REQ_DELETE]))
    tr.req["a"][muts[:4]] = 10**9
    base = tr.rows.ctypes.data

    def rows_of(r):
        return tr.rows[(int(r["vec"]) - base) // (d * 8)]

    ostore = oracle.store(d, 3)
    for row in X0:
        ostore.insert(row)
    i = 0
    st = S.SearchStats()
    while i < len(tr):
        j = min(len(tr), i + int(rng.integers(1, 200)))
        batch = tr.req[i:j]
        resp, ids, dists = srv.execute(batch, precision, 32, st)
        _check_batch(S, oracle, ostore, batch, resp, ids, dists, rows_of)
        assert st.bound_failures == 0
        i = j
    assert srv.size == ostore.size
    H = ostore.rows()
    for p in (0, 1, len(H) // 2, len(H) - 1):
        assert np.array_equal(srv.read(p), H[p])
    srv.close()


@pytest.mark.gpu
def test_gpu_server_replay_in_real_time(svdb):
    """The open-loop replay answers every request of a short trace."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from svdb_gb300 import serve
    sample = _sampler(64)
    srv = serve.Server(64, 1 << 15)
    srv.insert_block(sample(20000, 1))
    tr = serve.make_trace(sample, 20000, 4000, 8000.0, seed=5)
    res = serve.replay(srv, tr)
    assert res["requests"] == len(tr) and res["bound_failures"] == 0
    assert res["p99_ms"] is not None and res["p50_ms"] <= res["p99_ms"]
    assert set(res["statuses"]) <= {0, svdb.CMP_OUT_OF_BOUNDS}
    srv.close()
