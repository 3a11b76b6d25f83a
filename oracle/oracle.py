"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg,
never by the shipped library.  Two back ends:

* ``Oracle``    -- oracle/_build/liboracle.so, the C restatement of the
  reference's arithmetic (svdb_oracle.c); builds anywhere.
* ``RefLib``    -- oracle/_ref/libsvdb_ref.so, the reference's own
  src/vector_database.c + src/kdtree.c compiled unmodified; only where the
  reference sources exist (its recipe is oracle/Makefile).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsvdb_ref.so")
REF_O2_SO = os.path.join(HERE, "_ref", "libsvdb_ref_O2.so")
REF_SRC = os.environ.get("SVDB_REFERENCE_DIR", "/root/reference")

COSINE, EUCLIDEAN, DOT = 0, 1, 2
METRICS = {"cosine_similarity": COSINE, "euclidean_distance": EUCLIDEAN, "dot_product": DOT}

_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)


def build(ref: bool | None = None) -> None:
    """Compile the restatement, and the reference where its sources exist."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref is None:
        ref = os.path.isfile(os.path.join(REF_SRC, "src", "kdtree.c"))
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}"], check=True,
                       stderr=subprocess.DEVNULL)


def _ptr(a: np.ndarray, t=_dp):
    return a.ctypes.data_as(t)


class Oracle:
    def __init__(self, path: str = ORACLE_SO):
        if not os.path.isfile(path):
            build(ref=False)
        L = C.CDLL(path)
        for n in ("orc_ref_cosine", "orc_ref_euclidean", "orc_ref_dot"):
            getattr(L, n).restype = C.c_float
            getattr(L, n).argtypes = [_dp, _dp, C.c_size_t]
        L.orc_ref_metric.restype = C.c_float
        L.orc_ref_metric.argtypes = [C.c_int, _dp, C.c_size_t, _dp, C.c_size_t]
        for n in ("orc_fp64_canon", "orc_fp64_seq"):
            getattr(L, n).restype = C.c_double
            getattr(L, n).argtypes = [C.c_int, _dp, _dp, C.c_size_t]
        L.orc_canon_sumsq.restype = C.c_double
        L.orc_canon_sumsq.argtypes = [_dp, C.c_size_t]
        L.orc_topk.restype = C.c_int
        L.orc_topk.argtypes = [C.c_int, C.c_int, _dp, C.c_size_t, C.c_size_t, _dp, C.c_size_t,
                               C.c_size_t, _i64p, _dp, C.c_int]
        L.orc_kd_create.restype = C.c_void_p
        L.orc_kd_create.argtypes = [C.c_size_t]
        L.orc_kd_free.argtypes = [C.c_void_p]
        L.orc_kd_insert.restype = C.c_int
        L.orc_kd_insert.argtypes = [C.c_void_p, _dp, C.c_size_t]
        L.orc_kd_nearest.restype = C.c_size_t
        L.orc_kd_nearest.argtypes = [C.c_void_p, _dp]
        L.orc_store_create.restype = C.c_void_p
        L.orc_store_create.argtypes = [C.c_size_t, C.c_size_t]
        L.orc_store_free.argtypes = [C.c_void_p]
        L.orc_store_insert.restype = C.c_size_t
        L.orc_store_insert.argtypes = [C.c_void_p, _dp]
        L.orc_store_update.argtypes = [C.c_void_p, C.c_size_t, _dp]
        L.orc_store_delete.argtypes = [C.c_void_p, C.c_size_t]
        L.orc_store_size.restype = C.c_size_t
        L.orc_store_size.argtypes = [C.c_void_p]
        L.orc_store_rows.restype = _dp
        L.orc_store_rows.argtypes = [C.c_void_p]
        L.orc_store_nearest.restype = C.c_size_t
        L.orc_store_nearest.argtypes = [C.c_void_p, _dp]
        L.orc_decode_body.restype = C.c_int
        L.orc_decode_body.argtypes = [C.c_char_p, C.c_size_t, C.c_size_t, _dp]
        L.orc_format_number.restype = C.c_int
        L.orc_format_number.argtypes = [C.c_double, C.c_char_p]
        L.orc_format_compare.restype = C.c_size_t
        L.orc_format_compare.argtypes = [C.c_int, C.c_float, C.c_char_p]
        L.orc_format_nearest.restype = C.c_size_t
        L.orc_format_nearest.argtypes = [C.c_int, C.c_uint64, _dp, C.c_size_t, C.c_char_p, C.c_char_p]
        L.orc_find_uuid.restype = C.c_int
        L.orc_find_uuid.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t, _i64p, C.c_int]
        self.L = L

    # -- POST /nearest body: cJSON_Parse + the handler's checks -------------
    def decode_body(self, body: bytes, dim: int):
        """(status, values): 0 ok, 1 Invalid JSON, 2 Vector size mismatch,
        3 Invalid vector data (src/compare_handler.c:300-390)."""
        out = np.full(max(dim, 1), np.nan)
        st = self.L.orc_decode_body(body, len(body), dim, _ptr(out))
        return st, out[:dim]

    # -- response bodies as cJSON_PrintUnformatted writes them -------------
    def format_number(self, d: float) -> bytes:
        buf = C.create_string_buffer(64)
        n = self.L.orc_format_number(float(d), buf)
        return buf.raw[:n]

    def format_compare(self, metric: int, value) -> bytes:
        buf = C.create_string_buffer(128)
        n = self.L.orc_format_compare(metric, float(np.float32(value)), buf)
        return buf.raw[:n]

    def format_nearest(self, found: int, index: int, row, uuid37: bytes) -> bytes:
        """found 1: the row; 0: no neighbour; -1: an index that reads no row."""
        r = np.ascontiguousarray(row if row is not None else np.zeros(0), np.float64)
        buf = C.create_string_buffer(64 + 26 * r.size + 6 * 37 + 64)
        u = C.create_string_buffer(bytes(uuid37).ljust(37, b"\0")[:37], 38)
        n = self.L.orc_format_nearest(found, index, _ptr(r), r.size, u, buf)
        return buf.raw[:n]

    # -- GET /vector?uuid=: the reference's linear strncmp scan -------------
    def find_uuid(self, table: bytes, keys: bytes, threads: int = 1) -> np.ndarray:
        """table, keys: n x 37 and nk x 37 bytes (char uuid[37] each)."""
        n, nk = len(table) // 37, len(keys) // 37
        out = np.empty(nk, np.int64)
        if self.L.orc_find_uuid(table, n, keys, nk, _ptr(out, _i64p), threads) != 0:
            raise RuntimeError("orc_find_uuid: thread start failed")
        return out

    # -- /compare metrics, reference-exact (float accumulation) -------------
    def ref_metric(self, metric: int, a: np.ndarray, b: np.ndarray) -> np.float32:
        a = np.ascontiguousarray(a, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        return np.float32(self.L.orc_ref_metric(metric, _ptr(a), a.size, _ptr(b), b.size))

    def fp64(self, metric: int, a: np.ndarray, b: np.ndarray, seq: bool = False) -> float:
        a = np.ascontiguousarray(a, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        f = self.L.orc_fp64_seq if seq else self.L.orc_fp64_canon
        return f(metric, _ptr(a), _ptr(b), a.size)

    def topk(self, metric: int, x: np.ndarray, q: np.ndarray, k: int, seq: bool = False,
             threads: int | None = None):
        x = np.ascontiguousarray(x, np.float64)
        q = np.ascontiguousarray(q, np.float64).reshape(-1, x.shape[1])
        ids = np.empty((q.shape[0], k), np.int64)
        vals = np.empty((q.shape[0], k), np.float64)
        threads = threads or os.cpu_count() or 1
        rc = self.L.orc_topk(metric, int(seq), _ptr(x), x.shape[0], x.shape[1], _ptr(q), q.shape[0],
                             k, _ptr(ids, _i64p), _ptr(vals), threads)
        assert rc == 0
        return ids, vals

    # -- insertion-order KD tree / positional store --------------------------
    def kd(self, dim: int) -> "OracleKD":
        return OracleKD(self, dim)

    def store(self, d: int, kd_dim: int) -> "OracleStore":
        return OracleStore(self, d, kd_dim)


class OracleKD:
    def __init__(self, o: Oracle, dim: int):
        self.L = o.L
        self.h = o.L.orc_kd_create(dim)

    def insert(self, p: np.ndarray, index: int) -> None:
        p = np.ascontiguousarray(p, np.float64)
        self.L.orc_kd_insert(self.h, _ptr(p), index)

    def nearest(self, q: np.ndarray) -> int:
        q = np.ascontiguousarray(q, np.float64)
        r = self.L.orc_kd_nearest(self.h, _ptr(q))
        return -1 if r == 2**64 - 1 else int(r)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_kd_free(self.h)
            self.h = None


class OracleStore:
    def __init__(self, o: Oracle, d: int, kd_dim: int):
        self.L = o.L
        self.d = d
        self.h = o.L.orc_store_create(d, kd_dim)

    def insert(self, v):
        v = np.ascontiguousarray(v, np.float64)
        return int(self.L.orc_store_insert(self.h, _ptr(v)))

    def update(self, i, v):
        v = np.ascontiguousarray(v, np.float64)
        self.L.orc_store_update(self.h, i, _ptr(v))

    def delete(self, i):
        self.L.orc_store_delete(self.h, i)

    @property
    def size(self):
        return int(self.L.orc_store_size(self.h))

    def rows(self) -> np.ndarray:
        n = self.size
        if n == 0:
            return np.zeros((0, self.d))
        return np.ctypeslib.as_array(self.L.orc_store_rows(self.h), shape=(n * self.d,)).reshape(n, self.d).copy()

    def nearest(self, q) -> int:
        q = np.ascontiguousarray(q, np.float64)
        r = self.L.orc_store_nearest(self.h, _ptr(q))
        return -1 if r == 2**64 - 1 else int(r)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_store_free(self.h)
            self.h = None


# ---------------------------------------------------------------------------
# The reference itself (compiled unmodified), driven through its C API.
# ---------------------------------------------------------------------------
class RefVector(C.Structure):
    """include/vector_database.h:14-18"""
    _fields_ = [("uuid", C.c_char * 37), ("dimension", C.c_size_t), ("data", _dp)]


class RefLib:
    def __init__(self, path: str = REF_SO):
        if not os.path.isfile(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        L.vector_db_init.restype = C.c_void_p
        L.vector_db_init.argtypes = [C.c_size_t, C.c_size_t]
        L.vector_db_free.argtypes = [C.c_void_p]
        L.vector_db_insert.restype = C.c_size_t
        L.vector_db_insert.argtypes = [C.c_void_p, RefVector]
        L.vector_db_read.restype = C.POINTER(RefVector)
        L.vector_db_read.argtypes = [C.c_void_p, C.c_size_t]
        L.vector_db_update.argtypes = [C.c_void_p, C.c_size_t, RefVector]
        L.vector_db_read_by_uuid.restype = C.POINTER(RefVector)
        L.vector_db_read_by_uuid.argtypes = [C.c_void_p, C.c_char_p]
        L.vector_db_delete.argtypes = [C.c_void_p, C.c_size_t]
        for n in ("cosine_similarity", "euclidean_distance", "dot_product"):
            getattr(L, n).restype = C.c_float
            getattr(L, n).argtypes = [RefVector, RefVector]
        L.kdtree_nearest.restype = C.c_size_t
        L.kdtree_nearest.argtypes = [C.c_void_p, _dp]
        L.kdtree_create.restype = C.c_void_p
        L.kdtree_create.argtypes = [C.c_size_t]
        L.kdtree_insert.argtypes = [C.c_void_p, _dp, C.c_size_t]
        L.kdtree_free.argtypes = [C.c_void_p]
        self.L = L
        self.libc = C.CDLL(None)
        self.libc.malloc.restype = C.c_void_p
        self.libc.malloc.argtypes = [C.c_size_t]

    def make_vector(self, v: np.ndarray, uuid: bytes = b"") -> RefVector:
        """A Vector whose data is malloc'd, as the reference's handlers build it
        (the store takes ownership and later free()s it)."""
        v = np.ascontiguousarray(v, np.float64)
        p = self.libc.malloc(max(v.size, 1) * 8)
        C.memmove(p, v.ctypes.data, v.size * 8)
        vec = RefVector()
        vec.uuid = uuid[:36]
        vec.dimension = v.size
        vec.data = C.cast(p, _dp)
        return vec

    def metric(self, metric: int, a: np.ndarray, b: np.ndarray) -> np.float32:
        a = np.ascontiguousarray(a, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        va, vb = RefVector(), RefVector()
        va.dimension, va.data = a.size, _ptr(a)
        vb.dimension, vb.data = b.size, _ptr(b)
        f = (self.L.cosine_similarity, self.L.euclidean_distance, self.L.dot_product)[metric]
        return np.float32(f(va, vb))


class RefStore:
    """The reference's VectorDatabase, used through vector_db_* exactly as
    the handlers do (src/post_handler.c:333, src/put_handler.c:247,
    src/delete_handler.c:96, src/compare_handler.c:403-411)."""

    def __init__(self, ref: RefLib, kd_dim: int, capacity: int = 0):
        self.r = ref
        self.db = ref.L.vector_db_init(capacity, kd_dim)

    def _kdtree(self):
        # VectorDatabase layout (include/vector_database.h:24-30):
        # Vector* vectors; size_t size; size_t capacity; KDTree* kdtree; ...
        return C.cast(self.db + 24, C.POINTER(C.c_void_p))[0]

    @property
    def size(self):
        return C.cast(self.db + 8, C.POINTER(C.c_size_t))[0]

    def insert(self, v, uuid=b""):
        r = self.r.L.vector_db_insert(self.db, self.r.make_vector(v, uuid))
        return -1 if r == 2**64 - 1 else int(r)

    def update(self, i, v, uuid=b""):
        self.r.L.vector_db_update(self.db, i, self.r.make_vector(v, uuid))

    def find_uuid(self, key: bytes) -> int:
        """vector_db_read_by_uuid (src/vector_database.c:145-158) -> the row's
        position (pointer minus the array base over sizeof(Vector) = 56), -1
        for NULL."""
        p = self.r.L.vector_db_read_by_uuid(self.db, key)
        if not p:
            return -1
        base = C.cast(self.db, C.POINTER(C.c_void_p))[0]
        return (C.cast(p, C.c_void_p).value - base) // C.sizeof(RefVector)

    def delete(self, i):
        self.r.L.vector_db_delete(self.db, i)

    def read(self, i):
        p = self.r.L.vector_db_read(self.db, i)
        if not p:
            return None
        v = p.contents
        return np.ctypeslib.as_array(v.data, shape=(v.dimension,)).copy()

    def nearest(self, q) -> int:
        q = np.ascontiguousarray(q, np.float64)
        r = self.r.L.kdtree_nearest(self._kdtree(), _ptr(q))
        return -1 if r == 2**64 - 1 else int(r)

    def free(self):
        if self.db:
            self.r.L.vector_db_free(self.db)
            self.db = None


# ---------------------------------------------------------------------------
# uuid lookup (numpy restatement of src/vector_database.c:145-158)
# ---------------------------------------------------------------------------
def uuid_record(u: bytes) -> np.ndarray:
    """char uuid[37] as strncmp(.., 37) sees it: the bytes up to the first NUL
    (at most 37), zero padded to 37."""
    b = bytes(u)[:37]
    b = b.split(b"\0", 1)[0]
    return np.frombuffer(b.ljust(37, b"\0"), np.uint8)


def uuid_first(table: np.ndarray, key: bytes) -> int:
    """Position of the first row of `table` (n x 37 records) whose uuid equals
    `key` under strncmp(.., 37) -- the reference's linear scan -- or -1."""
    if table.shape[0] == 0:
        return -1
    hit = np.flatnonzero((table == uuid_record(key)).all(axis=1))
    return int(hit[0]) if hit.size else -1
