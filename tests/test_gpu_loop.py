"""The device-side request loop (svdb_loop_*) against the oracle.

A persistent kernel serves /compare, POST /nearest (the reference's
insertion-order KD tree) and /vector insert / update / delete from a ring in
mapped host memory.  Bar: replaying the same requests in ticket order through
the oracle's positional store (the reference's semantics: delete shifts later
positions, update adds a second KD node, deletes leave the KD tree alone)
gives the same status for every request, bit-identical /compare floats, the
same /nearest indices (stale ones included) and the same final rows.  The
bounded wait is tested by letting the loop run out of requests; shutdown is
tested from the host; admission by the reserved capacity.
"""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REQ_COMPARE, REQ_INSERT, REQ_UPDATE, REQ_DELETE, REQ_KD = 1, 2, 3, 4, 5
OK, OOB, UNKNOWN, ENOMEM = 0, 1, 5, -2


@pytest.fixture(scope="module")
def S(svdb):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return svdb


def _trace(rng, n0, nreq, d):
    """(op, metric, a, b, vec) per request; positions drawn from the size the
    store has at that point (plus some past the end)."""
    out = []
    size = n0
    for _ in range(nreq):
        u = rng.random()
        vec = rng.uniform(-1, 1, d)
        if u < 0.40:
            out.append((REQ_KD, 0, 0, 0, vec))
        elif u < 0.70:
            m = int(rng.integers(0, 3)) if rng.random() > 0.05 else 7
            a, b = (int(x) for x in rng.integers(0, size + 3, 2))
            out.append((REQ_COMPARE, m, a, b, None))
        elif u < 0.85:
            out.append((REQ_INSERT, 0, 0, 0, vec))
            size += 1
        elif u < 0.93:
            out.append((REQ_UPDATE, 0, int(rng.integers(0, size + 2)), 0, vec))
        else:
            a = int(rng.integers(0, size + 2))
            out.append((REQ_DELETE, 0, a, 0, None))
            if a < size:
                size -= 1
    return out


def _replay_oracle(oracle, X0, trace):
    """The oracle's answers for the trace in order: (status, value, index)."""
    st = oracle.store(X0.shape[1], 3)
    rows = [x.copy() for x in X0]
    for x in X0:
        st.insert(x)
    res = []
    for op, m, a, b, vec in trace:
        if op == REQ_KD:
            r = st.nearest(vec)
            res.append((OK, None, 2 ** 64 - 1 if r < 0 else r))
        elif op == REQ_COMPARE:
            if a >= len(rows) or b >= len(rows):
                res.append((OOB, None, None))
            elif m > 2:
                res.append((UNKNOWN, None, None))
            else:
                res.append((OK, oracle.ref_metric(m, rows[a], rows[b]), None))
        elif op == REQ_INSERT:
            st.insert(vec)
            rows.append(vec.copy())
            res.append((OK, None, len(rows) - 1))
        elif op == REQ_UPDATE:
            if a >= len(rows):
                res.append((OOB, None, None))
            else:
                st.update(a, vec)
                rows[a] = vec.copy()
                res.append((OK, None, None))
        else:
            if a >= len(rows):
                res.append((OOB, None, None))
            else:
                st.delete(a)
                del rows[a]
                res.append((OK, None, None))
    return res, rows


def _record(S, op, m, a, b, vec, keep):
    from svdb_gb300 import serve
    r = np.zeros(1, serve.REQ_DTYPE)
    r["op"], r["metric"], r["a"], r["b"] = op, m, a, b
    if vec is not None:
        v = np.ascontiguousarray(vec, np.float64)
        keep.append(v)
        r["vec"] = v.ctypes.data
    return r


def _check(S, got, want):
    for i, ((gs, gv, gi), (ws, wv, wi)) in enumerate(zip(got, want)):
        assert gs == ws, (i, gs, ws)
        if wv is not None:
            assert np.float32(gv).tobytes() == np.float32(wv).tobytes(), (i, gv, wv)
        if wi is not None:
            assert gi == wi, (i, gi, wi)


@pytest.mark.parametrize("chunk", [1, 37, 256])
def test_loop_trace_matches_oracle(S, oracle, chunk):
    rng = np.random.default_rng(chunk)
    d, n0 = 24, 2000
    X0 = rng.uniform(-1, 1, (n0, d))
    trace = _trace(rng, n0, 2500, d)
    loop = S.DeviceLoop(d, 3, n0 + 2000, X0)
    loop.start()
    got, keep = [], []
    for c0 in range(0, len(trace), chunk):  # submit a chunk, then take its answers: batches form as they arrive
        tickets = [loop.submit(_record(S, *req, keep)) for req in trace[c0:c0 + chunk]]
        got += [loop.wait(t) for t in tickets]
        keep.clear()
    want, rows = _replay_oracle(oracle, X0, trace)
    _check(S, got, want)
    loop.stop()
    info = loop.info()
    assert info["state"] == S.LOOP_STOPPED and info["size"] == len(rows) and info["answered"] == len(trace)
    for i in range(0, len(rows), 97):
        row, _ = loop.read(i)
        assert np.array_equal(row, rows[i]), i
    loop.close()


def test_loop_many_submitting_threads(S, oracle):
    """8 host threads submit at once; the ticket order is the serial order."""
    rng = np.random.default_rng(9)
    d, n0 = 16, 1500
    X0 = rng.uniform(-1, 1, (n0, d))
    reqs = _trace(rng, n0, 4000, d)
    loop = S.DeviceLoop(d, 3, n0 + 4000, X0, max_batch=64)
    loop.start()
    lock = threading.Lock()
    order = []  # (ticket, request index)
    answers = {}
    nxt = [0]
    keep = []

    def worker():
        while True:
            with lock:
                i = nxt[0]
                if i >= len(reqs):
                    return
                nxt[0] += 1
                rec = _record(S, *reqs[i], keep)
                t = loop.submit(rec)
                order.append((t, i))
            answers[t] = loop.wait(t)

    ths = [threading.Thread(target=worker) for _ in range(8)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    order.sort()
    trace = [reqs[i] for _, i in order]
    want, rows = _replay_oracle(oracle, X0, trace)
    _check(S, [answers[t] for t, _ in order], want)
    assert loop.info()["batches"] < len(reqs)  # requests were batched
    loop.close()


def test_loop_bounded_idle_wait_and_restart(S, oracle):
    """With nothing to do the kernel returns after idle_us; a later request
    starts it again."""
    rng = np.random.default_rng(3)
    X0 = rng.uniform(-1, 1, (100, 8))
    loop = S.DeviceLoop(8, 3, 200, X0, idle_us=20000)
    loop.start()
    t0 = time.time()
    while loop.info()["state"] != S.LOOP_LEFT_IDLE and time.time() - t0 < 10:
        time.sleep(0.01)
    info = loop.info()
    assert info["state"] == S.LOOP_LEFT_IDLE and info["idle_exits"] == 1, info
    keep = []
    t = loop.submit(_record(S, REQ_COMPARE, 2, 0, 1, None, keep))
    st, v, _ = loop.wait(t)
    assert st == OK and np.float32(v).tobytes() == oracle.ref_metric(2, X0[0], X0[1]).tobytes()
    assert loop.info()["answered"] == 1
    loop.close()


def test_loop_stop_from_host_and_admission(S, oracle):
    rng = np.random.default_rng(4)
    d = 8
    X0 = rng.uniform(-1, 1, (50, d))
    loop = S.DeviceLoop(d, 3, 55, X0)  # room for 5 more rows
    loop.start()
    keep = []
    ins = [loop.submit(_record(S, REQ_INSERT, 0, 0, 0, rng.uniform(-1, 1, d), keep)) for _ in range(8)]
    res = [loop.wait(t) for t in ins]
    assert [r[0] for r in res] == [OK] * 5 + [ENOMEM] * 3
    assert [r[2] for r in res[:5]] == [50, 51, 52, 53, 54]
    loop.stop()
    assert loop.info()["state"] == S.LOOP_STOPPED
    row, _ = loop.read(52)
    assert row.shape == (d,)
    # a request after the stop starts the loop again
    t = loop.submit(_record(S, REQ_DELETE, 0, 0, 0, None, keep))
    assert loop.wait(t)[0] == OK and loop.info()["size"] == 54
    loop.close()


def test_loop_deep_tree_and_empty_store(S, oracle):
    """Rows inserted in sorted order make a degenerate KD tree (height 3000):
    the descent still answers as the reference; an empty store answers
    (size_t)-1."""
    d = 4
    X0 = np.sort(np.random.default_rng(5).uniform(-1, 1, (3000, d)), axis=0)
    loop = S.DeviceLoop(d, 1, 3100, X0)
    o = oracle.kd(1)
    for i, x in enumerate(X0):
        o.insert(x, i)
    keep = []
    Q = np.random.default_rng(6).uniform(-1, 1, (64, d))
    ts = [loop.submit(_record(S, REQ_KD, 0, 0, 0, q, keep)) for q in Q]
    got = [loop.wait(t) for t in ts]
    for q, (st, _, ix) in zip(Q, got):
        assert st == OK and ix == o.nearest(q)
    loop.close()
    empty = S.DeviceLoop(d, 3, 10)
    t = empty.submit(_record(S, REQ_KD, 0, 0, 0, Q[0], keep))
    st, _, ix = empty.wait(t)
    assert st == OK and ix == 2 ** 64 - 1  # kdtree_nearest of an empty tree: (size_t)-1
    empty.close()
