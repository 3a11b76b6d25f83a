"""Serving: batches of mixed requests on a device-resident server store.

`Server` binds svdb_server_* (a store whose rows live only in HBM, with the
reference's positional semantics).  `make_trace` draws a seeded open-loop
request trace -- Poisson arrivals, a mix of /nearest top-k, /compare,
/vector insert, update and delete -- and `replay` serves it the way a
batching front end does: whenever the server is free it takes every request
that has arrived (up to `max_batch`), runs them as one svdb_server_execute
call and stamps each with its completion time, so a request's latency is its
queueing time plus the time of the batch that answered it.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import EUCLIDEAN, PREC_BF16, SearchStats, SvdbError, _check, _dp, _f64, _i64p, last_error, lib, uuid_block

REQ_NEAREST, REQ_COMPARE, REQ_INSERT, REQ_UPDATE, REQ_DELETE = range(5)
REQ_NAMES = ("nearest", "compare", "insert", "update", "delete")

# struct svdb_request / svdb_response (include/svdb_gb300.h)
REQ_DTYPE = np.dtype([("op", "<i4"), ("metric", "<i4"), ("k", "<u4"), ("reserved", "<u4"), ("a", "<u8"),
                      ("b", "<u8"), ("vec", "<u8"), ("uuid", "<u8")])
RESP_DTYPE = np.dtype([("status", "<i4"), ("value", "<f4"), ("index", "<u8")])
assert REQ_DTYPE.itemsize == 48 and RESP_DTYPE.itemsize == 16

# /nearest 70 %, /compare 10 %, insert 15 %, update 3 %, delete 2 %
DEFAULT_MIX = (0.70, 0.10, 0.15, 0.03, 0.02)


class Server:
    """svdb_server_*: rows only in HBM; `reserve_rows` allocated up front."""

    def __init__(self, dim: int, reserve_rows: int, _ptr=None):
        self.dim = dim
        self.ptr = _ptr or lib.svdb_server_create(dim, reserve_rows)
        if not self.ptr:
            raise SvdbError(f"svdb_server_create failed: {last_error()}")

    @classmethod
    def load(cls, filename: str, dim: int, reserve_rows: int = 0) -> "Server":
        """svdb_server_load: a reference-format file straight into HBM."""
        p = lib.svdb_server_load(filename.encode(), dim, reserve_rows)
        if not p:
            raise SvdbError(f"svdb_server_load failed: {last_error()}")
        return cls(dim, 0, _ptr=p)

    def save(self, filename: str) -> None:
        _check(lib.svdb_server_save(self.ptr, filename.encode()), "svdb_server_save")

    def insert_rows(self, rows, uuids=None) -> int:
        r = _f64(rows).reshape(-1, self.dim)
        keys = uuid_block(uuids) if uuids is not None else None
        first = C.c_size_t(0)
        _check(lib.svdb_server_insert_rows(self.ptr, r.ctypes.data_as(_dp), keys, r.shape[0], C.byref(first)),
               "svdb_server_insert_rows")
        return first.value

    def find_uuid(self, uuids) -> np.ndarray:
        keys = uuid_block(uuids)
        out = np.empty(len(uuids), np.int64)
        _check(lib.svdb_server_find_uuid(self.ptr, keys, len(uuids), out.ctypes.data_as(_i64p)),
               "svdb_server_find_uuid")
        return out

    def close(self) -> None:
        if self.ptr:
            lib.svdb_server_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def size(self) -> int:
        return int(lib.svdb_server_size(self.ptr))

    def insert_block(self, rows) -> int:
        r = _f64(rows).reshape(-1, self.dim)
        first = C.c_size_t(0)
        _check(lib.svdb_server_insert_block(self.ptr, r.ctypes.data_as(_dp), r.shape[0], C.byref(first)),
               "svdb_server_insert_block")
        return first.value

    def read(self, index: int) -> np.ndarray:
        out = np.empty(self.dim, np.float64)
        _check(lib.svdb_server_read(self.ptr, index, out.ctypes.data_as(_dp)), "svdb_server_read")
        return out

    def execute(self, req: np.ndarray, precision: int = PREC_BF16, stride: int = 10,
                stats: SearchStats | None = None, out=None):
        """One batch; req is a REQ_DTYPE array whose `vec` fields point at live
        float64 rows.  Returns (responses, ids, dists) with ids/dists
        [len(req), stride]."""
        n = req.shape[0]
        if out is None:
            resp = np.empty(n, RESP_DTYPE)
            ids = np.empty((n, stride), np.int64)
            dists = np.empty((n, stride), np.float64)
        else:
            resp, ids, dists = out
        _check(lib.svdb_server_execute(self.ptr, req.ctypes.data, n, resp.ctypes.data, precision,
                                       ids.ctypes.data_as(_i64p), dists.ctypes.data_as(_dp), stride,
                                       C.byref(stats) if stats is not None else None), "svdb_server_execute")
        return resp, ids, dists


class Trace:
    """A request trace: arrival times (s), requests and the rows they point at."""

    def __init__(self, arrival: np.ndarray, req: np.ndarray, rows: np.ndarray):
        self.arrival, self.req, self.rows = arrival, req, rows

    def __len__(self):
        return self.req.shape[0]

    def counts(self) -> dict:
        return {REQ_NAMES[o]: int((self.req["op"] == o).sum()) for o in range(5)}


def make_trace(sample_rows, n0: int, n_requests: int, rate: float, seed: int, mix=DEFAULT_MIX, k: int = 10,
               nearest_metric: int = EUCLIDEAN) -> Trace:
    """Seeded open-loop trace of `n_requests` requests at `rate` per second
    (exponential gaps) against a store that holds n0 rows when it starts.
    `sample_rows(m, stream)` draws m rows (queries and new rows come from the
    store's own distribution).  Positions are uniform over the rows the store
    holds at that point of the trace."""
    g = np.random.Generator(np.random.PCG64(np.random.SeedSequence([seed, 7])))
    arrival = np.cumsum(g.exponential(1.0 / rate, n_requests))
    ops = g.choice(5, size=n_requests, p=np.asarray(mix, np.float64) / np.sum(mix)).astype(np.int32)
    req = np.zeros(n_requests, REQ_DTYPE)
    req["op"] = ops
    need_vec = (ops == REQ_NEAREST) | (ops == REQ_INSERT) | (ops == REQ_UPDATE)
    rows = np.ascontiguousarray(sample_rows(int(need_vec.sum()), seed), np.float64)
    vec_at = np.cumsum(need_vec) - 1
    base = rows.ctypes.data
    req["vec"] = np.where(need_vec, base + vec_at.astype(np.uint64) * np.uint64(rows.shape[1] * 8), 0)
    metrics = g.integers(0, 3, n_requests)
    u = g.random((n_requests, 2))
    size = n0
    for i in range(n_requests):
        o = ops[i]
        if o == REQ_NEAREST:
            req["metric"][i] = nearest_metric
            req["k"][i] = k
        elif o == REQ_COMPARE:
            req["metric"][i] = metrics[i]
            req["a"][i] = int(u[i, 0] * size)
            req["b"][i] = int(u[i, 1] * size)
        elif o == REQ_INSERT:
            size += 1
        elif o == REQ_UPDATE:
            req["a"][i] = int(u[i, 0] * size)
        elif size > 0:  # delete
            req["a"][i] = int(u[i, 0] * size)
            size -= 1
    return Trace(arrival, req, rows)


def replay(server: Server, trace: Trace, precision: int = PREC_BF16, max_batch: int = 4096, stride: int = 10,
           time_limit: float | None = None, keep_results: bool = False) -> dict:
    """Serve `trace` open-loop in real time; returns latencies (ms) of the
    requests answered, the batch sizes, the wall time and the per-request
    results when keep_results."""
    n = len(trace)
    arrival = trace.arrival
    lat = np.full(n, np.nan)
    resp = np.empty(n, RESP_DTYPE)
    ids = np.empty((n, stride), np.int64)
    dists = np.empty((n, stride), np.float64)
    batches = []
    st = SearchStats()
    tot = {"widened": 0, "bound_failures": 0}
    i = 0
    t0 = time.perf_counter()
    while i < n:
        now = time.perf_counter() - t0
        if time_limit is not None and now > time_limit:
            break
        if arrival[i] > now:
            wait = arrival[i] - now
            if wait > 2e-4:
                time.sleep(wait - 1e-4)
            while time.perf_counter() - t0 < arrival[i]:
                pass
            now = time.perf_counter() - t0
        j = min(int(np.searchsorted(arrival, now, side="right")), i + max_batch)
        j = max(j, i + 1)
        out = (resp[i:j], ids[i:j], dists[i:j])
        server.execute(trace.req[i:j], precision, stride, st, out)
        done = time.perf_counter() - t0
        lat[i:j] = (done - arrival[i:j]) * 1e3
        tot["widened"] += st.widened
        tot["bound_failures"] += st.bound_failures
        batches.append(j - i)
        i = j
    wall = time.perf_counter() - t0
    served = lat[:i]
    res = {
        "requests": int(i),
        "offered": int(n),
        "wall_s": wall,
        "served_per_s": i / wall if i else 0.0,
        "p50_ms": float(np.percentile(served, 50)) if i else None,
        "p99_ms": float(np.percentile(served, 99)) if i else None,
        "max_ms": float(served.max()) if i else None,
        "batches": len(batches),
        "mean_batch": float(np.mean(batches)) if batches else 0.0,
        "widened": tot["widened"],
        "bound_failures": tot["bound_failures"],
        "statuses": {int(s): int(c) for s, c in zip(*np.unique(resp["status"][:i], return_counts=True))},
    }
    if keep_results:
        res["results"] = (resp[:i].copy(), ids[:i].copy(), dists[:i].copy(), np.asarray(batches))
    return res
