"""Python binding of libsvdb_gb300.so (the C ABI declared in include/).

Mirrors the reference's C API one to one -- ``vector_db_init``,
``vector_db_insert``, ``vector_db_read``, ``vector_db_update``,
``vector_db_delete``, ``vector_db_save``/``vector_db_load``,
``cosine_similarity``/``euclidean_distance``/``dot_product`` and
``kdtree_nearest`` (reference include/vector_database.h, include/kdtree.h)
-- plus the batch entry points of include/svdb_gb300.h.  There is no
Python compute path: every metric and search runs in the CUDA library, and
importing this module fails if the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.environ.get("SVDB_LIB", os.path.join(_PKG, "_build", "libsvdb_gb300.so"))

COSINE, EUCLIDEAN, DOT = 0, 1, 2
PREC_FP64, PREC_BF16, PREC_FP8 = 0, 1, 2
# status codes (include/svdb_gb300.h)
OK, EINVAL, ENOMEM, ECUDA, ETIMEOUT, ENODEV = 0, -1, -2, -3, -4, -5
METRIC_URLS = {"/compare/cosine_similarity": COSINE, "/compare/euclidean_distance": EUCLIDEAN,
               "/compare/dot_product": DOT}
CMP_OK, CMP_OUT_OF_BOUNDS, CMP_NOT_FOUND, CMP_DIFF_DIM, CMP_SIZE_MISMATCH, CMP_UNKNOWN_METHOD = range(6)
# error bodies of compare_handler_callback (src/compare_handler.c:88-163)
CMP_ERRORS = {
    CMP_OUT_OF_BOUNDS: (400, "Index out of bounds"),
    CMP_NOT_FOUND: (404, "Vector not found"),
    CMP_DIFF_DIM: (400, "Vectors have different dimensions"),
    CMP_SIZE_MISMATCH: (400, "Vector size mismatch"),
    CMP_UNKNOWN_METHOD: (400, "Unknown comparison method"),
}
NOT_FOUND = 2**64 - 1  # (size_t)-1
STAGE_PREP, STAGE_SCREEN, STAGE_SELECT, STAGE_REFINE, STAGE_RERANK = range(5)
NSTAGES = 5

_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)


class Vector(C.Structure):
    """include/vector_database.h (reference include/vector_database.h:14-18)."""
    _fields_ = [("uuid", C.c_char * 37), ("dimension", C.c_size_t), ("data", _dp)]


class SearchStats(C.Structure):
    _fields_ = [("candidates", C.c_uint64), ("survivors", C.c_uint64), ("reranked", C.c_uint64),
                ("widened", C.c_uint32), ("kernels", C.c_uint32), ("bound_failures", C.c_uint32),
                ("reserved", C.c_uint32), ("max_err_bound", C.c_double)]


class RaggedPart(C.Structure):
    """svdb_ragged_part (include/svdb_gb300.h)."""
    _fields_ = [("db", C.c_void_p), ("nq", C.c_size_t), ("dim", C.c_size_t), ("d_queries", C.c_void_p),
                ("k", C.POINTER(C.c_uint32)), ("d_ids", C.c_void_p), ("d_dists", C.c_void_p),
                ("stride", C.c_size_t)]


class RaggedInfo(C.Structure):
    """svdb_ragged_info (include/svdb_gb300.h)."""
    _fields_ = [("grouping", C.c_int32), ("concurrent", C.c_int32), ("graph", C.c_int32), ("searches", C.c_int32),
                ("tuned_ms", C.c_float * 4), ("captures", C.c_uint32), ("fp8_stores", C.c_uint32),
                ("swap_ms", C.c_float * 8), ("fused", C.c_int32), ("fused_launches", C.c_int32),
                ("fused_ms", C.c_float * 2), ("weight_ms", C.c_float * 3), ("epi_weight", C.c_float),
                ("seeded", C.c_int32), ("seed_ms", C.c_float)]


class LoopConfig(C.Structure):
    """svdb_loop_config (include/svdb_gb300.h)."""
    _fields_ = [("dim", C.c_size_t), ("kd_dim", C.c_size_t), ("capacity", C.c_size_t), ("kd_capacity", C.c_size_t),
                ("ring", C.c_size_t), ("max_batch", C.c_uint32), ("idle_us", C.c_uint32)]


class LoopInfo(C.Structure):
    """svdb_loop_info (include/svdb_gb300.h)."""
    _fields_ = [("state", C.c_uint32), ("reserved", C.c_uint32), ("size", C.c_uint64), ("answered", C.c_uint64),
                ("batches", C.c_uint64), ("idle_exits", C.c_uint64)]


LOOP_NOT_STARTED, LOOP_RUNNING, LOOP_LEFT_IDLE, LOOP_STOPPED, LOOP_LEAVING = range(5)
REQ_KD_NEAREST = 5

RAGGED_AUTOTUNE, RAGGED_NO_GRAPH, RAGGED_FUSED, RAGGED_BY_K_CLASS, RAGGED_SEED = 1, 2, 4, 8, 16
SAVE_EXACT_COUNT = 1


class SvdbError(RuntimeError):
    pass


def _load():
    if not os.path.isfile(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with simple-vector-db_gb300/build.py")
    L = C.CDLL(LIB_PATH)
    vp, sz = C.c_void_p, C.c_size_t
    sig = {
        "vector_db_init": (vp, [sz, sz]),
        "vector_db_free": (None, [vp]),
        "vector_db_insert": (sz, [vp, Vector]),
        "vector_db_read": (C.POINTER(Vector), [vp, sz]),
        "vector_db_read_by_uuid": (C.POINTER(Vector), [vp, C.c_char_p]),
        "vector_db_update": (None, [vp, sz, Vector]),
        "vector_db_delete": (None, [vp, sz]),
        "vector_db_save": (None, [vp, C.c_char_p]),
        "vector_db_load": (vp, [C.c_char_p, sz]),
        "cosine_similarity": (C.c_float, [Vector, Vector]),
        "euclidean_distance": (C.c_float, [Vector, Vector]),
        "dot_product": (C.c_float, [Vector, Vector]),
        "kdtree_create": (vp, [sz]),
        "kdtree_insert": (None, [vp, _dp, sz]),
        "kdtree_free": (None, [vp]),
        "kdtree_nearest": (sz, [vp, _dp]),
        "svdb_compare_batch": (C.c_int, [vp, C.c_int, _i64p, _i64p, sz, sz, C.POINTER(C.c_float),
                                         C.POINTER(C.c_int32)]),
        "svdb_nearest_batch": (C.c_int, [vp, _dp, sz, sz, _i64p]),
        "svdb_search_topk": (C.c_int, [vp, _dp, sz, sz, sz, C.c_int, C.c_int, _i64p, _dp, _dp,
                                       C.POINTER(SearchStats)]),
        "svdb_search_topk_device": (C.c_int, [vp, vp, sz, sz, sz, C.c_int, C.c_int, vp, vp, vp,
                                              C.POINTER(SearchStats)]),
        "svdb_insert_batch": (C.c_int, [vp, _dp, sz, sz, C.c_char_p, C.POINTER(C.c_size_t)]),
        "svdb_reserve": (C.c_int, [vp, sz, sz]),
        "svdb_sync": (C.c_int, [vp]),
        "svdb_stream": (vp, [vp]),
        "svdb_wait": (C.c_int, [vp]),
        "svdb_last_error": (C.c_char_p, []),
        "svdb_profile": (C.c_int, [vp, C.c_int]),
        "svdb_set_screen_seeding": (C.c_int, [vp, C.c_int]),
        "svdb_set_fp8_screen": (C.c_int, [vp, C.c_int]),
        "svdb_selftest_bounded_wait": (C.c_int, [vp, C.c_uint32, C.POINTER(C.c_uint32)]),
        "svdb_save": (C.c_int, [vp, C.c_char_p, C.c_uint]),
        "svdb_format_compare": (C.c_int, [C.POINTER(C.c_int32), C.POINTER(C.c_float), C.POINTER(C.c_int32), sz,
                                          vp, sz, C.POINTER(C.c_uint64)]),
        "svdb_format_nearest": (C.c_int, [vp, _i64p, sz, vp, sz, C.POINTER(C.c_uint64)]),
        "svdb_loop_create": (vp, [C.POINTER(LoopConfig), _dp, sz, C.c_char_p]),
        "svdb_loop_start": (C.c_int, [vp]),
        "svdb_loop_submit": (C.c_int, [vp, vp, C.POINTER(C.c_uint64)]),
        "svdb_loop_wait": (C.c_int, [vp, C.c_uint64, vp, C.c_uint32]),
        "svdb_loop_stop": (C.c_int, [vp]),
        "svdb_loop_get_info": (C.c_int, [vp, C.POINTER(LoopInfo)]),
        "svdb_loop_read": (C.c_int, [vp, sz, _dp, C.c_char_p]),
        "svdb_loop_destroy": (None, [vp]),
        "svdb_debug_screen_accumulators": (C.c_int, [vp, _dp, sz, sz, C.c_int, C.c_int, sz,
                                                     C.POINTER(C.c_float), vp, vp, C.POINTER(C.c_size_t)]),
        "svdb_server_create": (vp, [sz, sz]),
        "svdb_server_destroy": (None, [vp]),
        "svdb_server_size": (sz, [vp]),
        "svdb_server_insert_block": (C.c_int, [vp, _dp, sz, C.POINTER(C.c_size_t)]),
        "svdb_server_read": (C.c_int, [vp, sz, _dp]),
        "svdb_server_execute": (C.c_int, [vp, vp, sz, vp, C.c_int, _i64p, _dp, sz, C.POINTER(SearchStats)]),
        "svdb_merge_topk": (C.c_int, [C.c_int, _i64p, _dp, sz, sz, sz, _i64p, _dp]),
        "svdb_search_topk_fp64_noalloc": (C.c_int, [vp, vp, sz, sz, sz, C.c_int, vp, vp]),
        "svdb_profile_read": (C.c_int, [vp, _dp, C.c_int]),
        "svdb_find_uuid_batch": (C.c_int, [vp, C.c_char_p, sz, _i64p]),
        "svdb_decode_vectors": (C.c_int, [C.c_char_p, C.POINTER(C.c_uint64), sz, sz, _dp, C.POINTER(C.c_int32)]),
        "svdb_nearest_batch_median": (C.c_int, [vp, _dp, sz, sz, _i64p]),
        "svdb_server_insert_rows": (C.c_int, [vp, _dp, C.c_char_p, sz, C.POINTER(C.c_size_t)]),
        "svdb_server_find_uuid": (C.c_int, [vp, C.c_char_p, sz, _i64p]),
        "svdb_server_save": (C.c_int, [vp, C.c_char_p]),
        "svdb_server_load": (vp, [C.c_char_p, sz, sz]),
        "svdb_ragged_create": (vp, [C.POINTER(RaggedPart), sz, C.c_int, C.c_int, C.c_uint]),
        "svdb_ragged_run": (C.c_int, [vp]),
        "svdb_ragged_wait": (C.c_int, [vp]),
        "svdb_ragged_stream": (vp, [vp]),
        "svdb_ragged_get_info": (C.c_int, [vp, C.POINTER(RaggedInfo)]),
        "svdb_ragged_get_search_stats": (C.c_int, [vp, C.POINTER(C.c_uint64), C.c_size_t]),
        "svdb_ragged_destroy": (None, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype, f.argtypes = res, args
    return L


lib = _load()
_libc = C.CDLL(None)
_libc.malloc.restype = C.c_void_p
_libc.malloc.argtypes = [C.c_size_t]


def last_error() -> str:
    return (lib.svdb_last_error() or b"").decode(errors="replace")


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise SvdbError(f"{what} failed ({rc}): {last_error()}")


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def make_vector(data, uuid: bytes | str = b"", owned: bool = True) -> Vector:
    """A Vector as the handlers build it.  owned=True mallocs the data (the
    store takes ownership on insert/update and free()s it later); owned=False
    points at the numpy buffer (for the metric functions, which only read)."""
    a = _f64(data).ravel()
    v = Vector()
    if isinstance(uuid, str):
        uuid = uuid.encode()
    v.uuid = uuid[:36]
    v.dimension = a.size
    if owned:
        p = _libc.malloc(max(a.size, 1) * 8)
        if not p:
            raise MemoryError
        C.memmove(p, a.ctypes.data, a.size * 8)
        v.data = C.cast(p, _dp)
    else:
        v.data = a.ctypes.data_as(_dp)
        v._keep = a
    return v


def uuid_block(uuids) -> bytes:
    """n uuids (str or bytes) as n x 37 bytes, each NUL-padded the way
    char uuid[37] holds a shorter string (longer ones keep 37 bytes)."""
    out = bytearray()
    for u in uuids:
        b = u.encode() if isinstance(u, str) else bytes(u)
        out += b[:37].ljust(37, b"\0")
    return bytes(out)


def decode_vectors(bodies, dim: int):
    """svdb_decode_vectors: POST /nearest bodies (bytes each) decoded on the
    device -> (values [n, dim] float64, status [n] int32, SVDB_DEC_*)."""
    text = b"".join(bodies)
    off = np.zeros(len(bodies) + 1, np.uint64)
    off[1:] = np.cumsum([len(b) for b in bodies])
    out = np.empty((len(bodies), dim), np.float64)
    st = np.empty(len(bodies), np.int32)
    _check(lib.svdb_decode_vectors(text, off.ctypes.data_as(C.POINTER(C.c_uint64)), len(bodies), dim,
                                   out.ctypes.data_as(_dp), st.ctypes.data_as(C.POINTER(C.c_int32))),
           "svdb_decode_vectors")
    return out, st


DEC_OK, DEC_INVALID_JSON, DEC_SIZE_MISMATCH, DEC_INVALID_DATA = range(4)


def cosine_similarity(a, b) -> np.float32:
    return np.float32(lib.cosine_similarity(make_vector(a, owned=False), make_vector(b, owned=False)))


def euclidean_distance(a, b) -> np.float32:
    return np.float32(lib.euclidean_distance(make_vector(a, owned=False), make_vector(b, owned=False)))


def dot_product(a, b) -> np.float32:
    return np.float32(lib.dot_product(make_vector(a, owned=False), make_vector(b, owned=False)))


def _format(call, n):
    off = np.zeros(n + 1, np.uint64)
    _check(call(None, 0, off), "svdb_format")
    buf = C.create_string_buffer(max(int(off[-1]), 1))
    _check(call(buf, len(buf), off), "svdb_format")
    raw = buf.raw
    return [raw[int(off[i]):int(off[i + 1])] for i in range(n)]


def format_compare(metric, value, status=None) -> list:
    """svdb_format_compare: GET /compare response bodies (bytes each)."""
    m = np.ascontiguousarray(metric, np.int32)
    v = np.ascontiguousarray(value, np.float32)
    s = np.zeros(m.size, np.int32) if status is None else np.ascontiguousarray(status, np.int32)
    u64 = C.POINTER(C.c_uint64)
    return _format(lambda out, cap, off: lib.svdb_format_compare(
        m.ctypes.data_as(C.POINTER(C.c_int32)), v.ctypes.data_as(C.POINTER(C.c_float)),
        s.ctypes.data_as(C.POINTER(C.c_int32)), m.size, out, cap, off.ctypes.data_as(u64)), m.size)


class VectorDatabase:
    """Owner of one ``VectorDatabase*`` (vector_db_init / vector_db_load)."""

    def __init__(self, initial_capacity: int = 0, kd_dimension: int = 3, _ptr=None):
        self.ptr = _ptr if _ptr is not None else lib.vector_db_init(initial_capacity, kd_dimension)
        if not self.ptr:
            raise SvdbError("vector_db_init failed")
        self.kd_dimension = kd_dimension

    @classmethod
    def load(cls, filename: str, kd_dimension: int = 3) -> "VectorDatabase":
        p = lib.vector_db_load(filename.encode(), kd_dimension)
        if not p:
            raise SvdbError(f"vector_db_load({filename}) failed")
        return cls(_ptr=p, kd_dimension=kd_dimension)

    def close(self) -> None:
        if self.ptr:
            lib.vector_db_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- struct fields the handlers read (include/vector_database.h:24-30) --
    @property
    def size(self) -> int:
        return C.cast(self.ptr + 8, C.POINTER(C.c_size_t))[0]

    @property
    def kdtree(self) -> int:
        return C.cast(self.ptr + 24, C.POINTER(C.c_void_p))[0]

    # -- vector_db_* ---------------------------------------------------------
    def insert(self, data, uuid: bytes | str = b"") -> int:
        r = lib.vector_db_insert(self.ptr, make_vector(data, uuid))
        if r == NOT_FOUND:
            raise SvdbError(f"vector_db_insert failed: {last_error()}")
        return int(r)

    def insert_batch(self, rows, uuids: bytes | None = None) -> int:
        rows = _f64(rows)
        first = C.c_size_t(0)
        _check(lib.svdb_insert_batch(self.ptr, rows.ctypes.data_as(_dp), rows.shape[0], rows.shape[1], uuids,
                                     C.byref(first)), "svdb_insert_batch")
        return first.value

    def read(self, index: int):
        p = lib.vector_db_read(self.ptr, index)
        if not p:
            return None
        v = p.contents
        return np.ctypeslib.as_array(v.data, shape=(v.dimension,)).copy() if v.dimension else np.zeros(0)

    def uuid(self, index: int) -> bytes | None:
        p = lib.vector_db_read(self.ptr, index)
        return bytes(p.contents.uuid).split(b"\0")[0] if p else None

    def find_uuid(self, uuids) -> np.ndarray:
        """svdb_find_uuid_batch: position of the first row with each uuid
        (strncmp over 37 bytes, as the reference compares), -1 if none."""
        keys = uuid_block(uuids)
        out = np.empty(len(uuids), np.int64)
        _check(lib.svdb_find_uuid_batch(self.ptr, keys, len(uuids), out.ctypes.data_as(_i64p)),
               "svdb_find_uuid_batch")
        return out

    def read_by_uuid(self, uuid: bytes | str):
        if isinstance(uuid, str):
            uuid = uuid.encode()
        p = lib.vector_db_read_by_uuid(self.ptr, uuid)
        if not p:
            return None
        v = p.contents
        return np.ctypeslib.as_array(v.data, shape=(v.dimension,)).copy()

    def update(self, index: int, data, uuid: bytes | str = b"") -> None:
        lib.vector_db_update(self.ptr, index, make_vector(data, uuid))

    def delete(self, index: int) -> None:
        lib.vector_db_delete(self.ptr, index)

    def save(self, filename: str, exact_count: bool = False) -> None:
        """vector_db_save (the reference's bytes), or svdb_save with
        SVDB_SAVE_EXACT_COUNT: the row count written is the rows written."""
        if exact_count:
            _check(lib.svdb_save(self.ptr, filename.encode(), SAVE_EXACT_COUNT), "svdb_save")
        else:
            lib.vector_db_save(self.ptr, filename.encode())

    def sync(self) -> None:
        _check(lib.svdb_sync(self.ptr), "svdb_sync")

    def reserve(self, rows: int, dim: int) -> None:
        _check(lib.svdb_reserve(self.ptr, rows, dim), "svdb_reserve")

    def set_fp8_screen(self, mode: int) -> None:
        """svdb_set_fp8_screen: which screen PREC_FP8 searches run; -1 the
        default rule (E4M3 for >= 1,024 queries and k <= 32), 0 BF16, 1 E4M3."""
        _check(lib.svdb_set_fp8_screen(self.ptr, int(mode)), "svdb_set_fp8_screen")

    def set_screen_seeding(self, mode: int) -> None:
        """svdb_set_screen_seeding: -1 default (FP8 only), 0 never, 1 always."""
        _check(lib.svdb_set_screen_seeding(self.ptr, int(mode)), "svdb_set_screen_seeding")

    def profile(self, enable: bool = True) -> None:
        _check(lib.svdb_profile(self.ptr, int(enable)), "svdb_profile")

    def profile_read(self, reset: bool = True):
        """(searches covered, device ms per stage: prep, screen, select, refine, rerank)."""
        ms = np.zeros(NSTAGES, np.float64)
        n = lib.svdb_profile_read(self.ptr, ms.ctypes.data_as(_dp), int(reset))
        if n < 0:
            raise SvdbError(f"svdb_profile_read failed ({n}): {last_error()}")
        return n, ms

    def stream(self) -> int:
        return lib.svdb_stream(self.ptr) or 0

    def wait(self) -> None:
        _check(lib.svdb_wait(self.ptr), "svdb_wait")

    # -- /nearest (KD tree) --------------------------------------------------
    def kdtree_nearest(self, q) -> int:
        """kdtree_nearest(db->kdtree, q) as src/compare_handler.c:403 calls it;
        -1 for (size_t)-1."""
        q = _f64(q)
        r = lib.kdtree_nearest(self.kdtree, q.ctypes.data_as(_dp))
        return -1 if r == NOT_FOUND else int(r)

    def nearest_batch(self, queries) -> np.ndarray:
        q = _f64(queries)
        q = q.reshape(-1, q.shape[-1])
        out = np.empty(q.shape[0], np.int64)
        _check(lib.svdb_nearest_batch(self.ptr, q.ctypes.data_as(_dp), q.shape[0], q.shape[1],
                                      out.ctypes.data_as(_i64p)), "svdb_nearest_batch")
        return out

    def nearest_batch_median(self, queries) -> np.ndarray:
        """svdb_nearest_batch_median: exact 1-NN over the KD prefix by a
        median-split tree of the current rows, ties to the lowest position."""
        q = _f64(queries)
        q = q.reshape(-1, q.shape[-1])
        out = np.empty(q.shape[0], np.int64)
        _check(lib.svdb_nearest_batch_median(self.ptr, q.ctypes.data_as(_dp), q.shape[0], q.shape[1],
                                             out.ctypes.data_as(_i64p)), "svdb_nearest_batch_median")
        return out

    # -- /compare ------------------------------------------------------------
    def compare_batch(self, metric: int, index1, index2, expected_dim: int = 0):
        i1 = np.ascontiguousarray(index1, np.int64)
        i2 = np.ascontiguousarray(index2, np.int64)
        out = np.empty(i1.size, np.float32)
        st = np.empty(i1.size, np.int32)
        _check(lib.svdb_compare_batch(self.ptr, metric, i1.ctypes.data_as(_i64p), i2.ctypes.data_as(_i64p), i1.size,
                                      expected_dim, out.ctypes.data_as(C.POINTER(C.c_float)),
                                      st.ctypes.data_as(C.POINTER(C.c_int32))), "svdb_compare_batch")
        return out, st

    def compare(self, url: str, index1: int, index2: int, expected_dim: int = 0):
        """GET /compare/<metric>?index1=&index2= -> (status, body dict)."""
        metric = METRIC_URLS.get(url, -1)
        out, st = self.compare_batch(metric, [index1], [index2], expected_dim)
        if st[0] != CMP_OK:
            code, msg = CMP_ERRORS[int(st[0])]
            return code, {"error": msg}
        return 200, {url.rsplit("/", 1)[1]: float(out[0])}

    # -- top-k ---------------------------------------------------------------
    def search(self, queries, k: int, metric: int = COSINE, precision: int = PREC_FP64, with_err: bool = False,
               stats: SearchStats | None = None, out=None):
        """Exact top-k (svdb_search_topk).  `out` = (ids, dists) preallocated
        [nq, k] int64 / float64 arrays; page-locked host buffers (queries and
        outputs) are read and written by DMA without a staging copy."""
        q = _f64(queries)
        q = q.reshape(-1, q.shape[-1])
        nq = q.shape[0]
        if out is not None:
            ids, dists = out
            assert ids.shape == (nq, k) and dists.shape == (nq, k) and ids.dtype == np.int64
            assert dists.dtype == np.float64 and ids.flags.c_contiguous and dists.flags.c_contiguous
        else:
            ids = np.empty((nq, k), np.int64)
            dists = np.empty((nq, k), np.float64)
        err = np.empty((nq, k), np.float64) if with_err else None
        _check(lib.svdb_search_topk(self.ptr, q.ctypes.data_as(_dp), nq, q.shape[1], k, metric, precision,
                                    ids.ctypes.data_as(_i64p), dists.ctypes.data_as(_dp),
                                    err.ctypes.data_as(_dp) if with_err else None,
                                    C.byref(stats) if stats is not None else None), "svdb_search_topk")
        return (ids, dists, err) if with_err else (ids, dists)

    def search_fp64_noalloc(self, q_ptr: int, nq: int, dim: int, k: int, metric: int, ids_ptr: int,
                            dists_ptr: int) -> None:
        """Exact FP64 top-k that allocates no device memory (device pointers,
        queued on self.stream()); for callers that cannot call cudaMalloc."""
        _check(lib.svdb_search_topk_fp64_noalloc(self.ptr, q_ptr, nq, dim, k, metric, ids_ptr, dists_ptr),
               "svdb_search_topk_fp64_noalloc")

    def format_nearest(self, index) -> list:
        """svdb_format_nearest: POST /nearest response bodies (bytes each) for
        the indices kdtree_nearest returned (-1 for none)."""
        ix = np.ascontiguousarray(index, np.int64)
        u64 = C.POINTER(C.c_uint64)
        return _format(lambda out, cap, off: lib.svdb_format_nearest(
            self.ptr, ix.ctypes.data_as(_i64p), ix.size, out, cap, off.ctypes.data_as(u64)), ix.size)

    def selftest_bounded_wait(self, limit_us: int = 20000):
        """(status, gave_up bits, message) of svdb_selftest_bounded_wait; a
        working failure path gives (ETIMEOUT, 3, ...)."""
        g = C.c_uint32(0)
        rc = lib.svdb_selftest_bounded_wait(self.ptr, limit_us, C.byref(g))
        return rc, g.value, last_error()

    def screen_accumulators(self, queries, metric: int, precision: int, rows: int):
        """svdb_debug_screen_accumulators (1..256 queries; more than 128 run
        the paired screen) -> (acc [nq, rows] float32, query operands
        [nq, op_bytes] uint8, row operands [rows, op_bytes] uint8)."""
        q = _f64(queries)
        q = q.reshape(-1, q.shape[-1])
        nq, d = q.shape
        ob = (d + 63) // 64 * 128 if precision == PREC_BF16 else (d + 127) // 128 * 128
        acc = np.empty((nq, rows), np.float32)
        qo = np.empty((nq, ob), np.uint8)
        ro = np.empty((rows, ob), np.uint8)
        got = C.c_size_t(0)
        _check(lib.svdb_debug_screen_accumulators(self.ptr, q.ctypes.data_as(_dp), nq, d, metric, precision, rows,
                                                  acc.ctypes.data_as(C.POINTER(C.c_float)), qo.ctypes.data,
                                                  ro.ctypes.data, C.byref(got)), "svdb_debug_screen_accumulators")
        assert got.value == ob, (got.value, ob)
        return acc, qo, ro

    def search_device(self, q_ptr: int, nq: int, dim: int, k: int, metric: int, precision: int, ids_ptr: int,
                      dists_ptr: int, err_ptr: int = 0, stats: SearchStats | None = None) -> None:
        """Device-pointer variant (queued on self.stream(); does not wait)."""
        _check(lib.svdb_search_topk_device(self.ptr, q_ptr, nq, dim, k, metric, precision, ids_ptr, dists_ptr,
                                           err_ptr or None, C.byref(stats) if stats is not None else None),
               "svdb_search_topk_device")


class RaggedPlan:
    """svdb_ragged_create / _run / _wait / _destroy: one uneven batch of
    top-k queries over several stores (different dimensions allowed), each
    query with its own k, answered by one CUDA-graph launch per run.

    ``parts`` is a list of (db, q_ptr, nq, dim, ks, ids_ptr, dists_ptr,
    stride): device pointers (torch tensors' data_ptr()), ks a host sequence
    of nq ints.  The buffers stay bound to the plan."""

    def __init__(self, parts, metric: int, precision: int, flags: int = RAGGED_AUTOTUNE):
        arr = (RaggedPart * len(parts))()
        self._ks = []
        for i, (db, q_ptr, nq, dim, ks, ids_ptr, dists_ptr, stride) in enumerate(parts):
            k = np.ascontiguousarray(ks, dtype=np.uint32)
            assert k.shape == (nq,)
            self._ks.append(k)
            arr[i] = RaggedPart(db.ptr, nq, dim, q_ptr, k.ctypes.data_as(C.POINTER(C.c_uint32)), ids_ptr,
                                dists_ptr, stride)
        self.ptr = lib.svdb_ragged_create(arr, len(parts), metric, precision, flags)
        if not self.ptr:
            raise SvdbError(f"svdb_ragged_create failed: {last_error()}")

    def run(self) -> None:
        _check(lib.svdb_ragged_run(self.ptr), "svdb_ragged_run")

    def wait(self) -> None:
        _check(lib.svdb_ragged_wait(self.ptr), "svdb_ragged_wait")

    def stream(self) -> int:
        return lib.svdb_ragged_stream(self.ptr) or 0

    def info(self) -> dict:
        inf = RaggedInfo()
        _check(lib.svdb_ragged_get_info(self.ptr, C.byref(inf)), "svdb_ragged_get_info")
        return {"grouping": inf.grouping, "concurrent": inf.concurrent, "graph": inf.graph,
                "searches": inf.searches, "tuned_ms": [float(x) for x in inf.tuned_ms], "captures": inf.captures,
                "fp8_stores": inf.fp8_stores, "swap_ms": [float(x) for x in inf.swap_ms], "fused": inf.fused,
                "fused_launches": inf.fused_launches, "fused_ms": [float(x) for x in inf.fused_ms],
                "weight_ms": [float(x) for x in inf.weight_ms], "epi_weight": float(inf.epi_weight),
                "seeded": inf.seeded, "seed_ms": float(inf.seed_ms)}

    def search_stats(self) -> np.ndarray:
        """svdb_ragged_get_search_stats: [searches, 12] uint64 (part, k, queries,
        fused, candidates, survivors, re-ranked, widened, bound failures,
        widened by candidate / survivor / re-rank overflow)."""
        n = self.info()["searches"]
        out = np.zeros((n, 12), np.uint64)
        _check(lib.svdb_ragged_get_search_stats(self.ptr, out.ctypes.data_as(C.POINTER(C.c_uint64)), n),
               "svdb_ragged_get_search_stats")
        return out

    def close(self) -> None:
        if getattr(self, "ptr", None):
            lib.svdb_ragged_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def merge_topk(metric: int, ids, vals):
    """Exact global top-k from per-shard lists ([shard, query, k], global ids);
    ties to the lowest global id (svdb_merge_topk)."""
    ids = np.ascontiguousarray(ids, np.int64)
    vals = np.ascontiguousarray(vals, np.float64)
    nsh, nq, k = ids.shape
    oi = np.empty((nq, k), np.int64)
    ov = np.empty((nq, k), np.float64)
    _check(lib.svdb_merge_topk(metric, ids.ctypes.data_as(_i64p), vals.ctypes.data_as(_dp), nsh, nq, k,
                               oi.ctypes.data_as(_i64p), ov.ctypes.data_as(_dp)), "svdb_merge_topk")
    return oi, ov


class KDTree:
    """Standalone kdtree_* (reference include/kdtree.h:32-57)."""

    def __init__(self, dimension: int):
        self.ptr = lib.kdtree_create(dimension)
        self.dimension = dimension

    def insert(self, point, index: int) -> None:
        p = _f64(point)
        lib.kdtree_insert(self.ptr, p.ctypes.data_as(_dp), index)

    def nearest(self, q) -> int:
        q = _f64(q)
        r = lib.kdtree_nearest(self.ptr, q.ctypes.data_as(_dp))
        return -1 if r == NOT_FOUND else int(r)

    def close(self):
        if self.ptr:
            lib.kdtree_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceLoop:
    """svdb_loop_*: the request path as a device-side loop over its own store
    (rows x dim initial rows, KD prefix kd_dim).  submit() takes a request
    record (serve.REQ_DTYPE layout) and returns a ticket; wait() its answer
    (status, value, index)."""

    def __init__(self, dim: int, kd_dim: int, capacity: int, rows=None, uuids=None, ring: int = 4096,
                 max_batch: int = 256, idle_us: int = 1_000_000, kd_capacity: int = 0):
        cfg = LoopConfig(dim, kd_dim, capacity, kd_capacity, ring, max_batch, idle_us)
        r = np.zeros((0, dim)) if rows is None else _f64(rows).reshape(-1, dim)
        self._rows = r
        keys = uuid_block(uuids) if uuids is not None else None
        self.ptr = lib.svdb_loop_create(C.byref(cfg), r.ctypes.data_as(_dp), r.shape[0], keys)
        if not self.ptr:
            raise SvdbError(f"svdb_loop_create failed: {last_error()}")
        self.dim = dim

    def start(self) -> None:
        _check(lib.svdb_loop_start(self.ptr), "svdb_loop_start")

    def submit(self, req) -> int:
        """req: one record of serve.REQ_DTYPE (a numpy void or 1-element array)."""
        t = C.c_uint64(0)
        _check(lib.svdb_loop_submit(self.ptr, req.ctypes.data if hasattr(req, "ctypes") else req, C.byref(t)),
               "svdb_loop_submit")
        return t.value

    def wait(self, ticket: int, timeout_us: int = 10_000_000):
        out = np.zeros(1, np.dtype([("status", "<i4"), ("value", "<f4"), ("index", "<u8")]))
        _check(lib.svdb_loop_wait(self.ptr, ticket, out.ctypes.data, timeout_us), "svdb_loop_wait")
        return int(out["status"][0]), np.float32(out["value"][0]), int(out["index"][0])

    def stop(self) -> None:
        _check(lib.svdb_loop_stop(self.ptr), "svdb_loop_stop")

    def info(self) -> dict:
        i = LoopInfo()
        _check(lib.svdb_loop_get_info(self.ptr, C.byref(i)), "svdb_loop_get_info")
        return {"state": i.state, "size": i.size, "answered": i.answered, "batches": i.batches,
                "idle_exits": i.idle_exits}

    def read(self, position: int):
        row = np.empty(self.dim, np.float64)
        u = C.create_string_buffer(38)
        _check(lib.svdb_loop_read(self.ptr, position, row.ctypes.data_as(_dp), u), "svdb_loop_read")
        return row, u.raw[:37].split(b"\0")[0]

    def close(self) -> None:
        if getattr(self, "ptr", None):
            lib.svdb_loop_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
