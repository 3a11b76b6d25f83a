"""C-ABI boundary checks that need no GPU: the library loads, exports every
function include/*.h declares, and the host-side store logic (positional
indices, ownership, uuid, the save/load file format, /compare request
validation) behaves as the reference's does."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(inc, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        src = re.sub(r"#[^\n]*", "", src)
        for m in re.finditer(r"([A-Za-z_]\w*)\s*\([^;{}]*\)\s*;", src):
            names.add(m.group(1))
    return names


def test_exports_every_declared_symbol(svdb):
    names = declared_functions()
    assert {"vector_db_init", "kdtree_nearest", "cosine_similarity", "svdb_search_topk"} <= names
    out = subprocess.run(["nm", "-D", "--defined-only", svdb.LIB_PATH], capture_output=True, text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if l.strip()}
    missing = names - exported
    assert not missing, missing
    lib = C.CDLL(svdb.LIB_PATH)
    for n in names:
        assert getattr(lib, n) is not None


def test_struct_layout_matches_reference(svdb):
    # include/vector_database.h:14-18 on LP64: uuid[37] + pad -> 40, dimension, data
    assert C.sizeof(svdb.Vector) == 56
    assert svdb.Vector.dimension.offset == 40 and svdb.Vector.data.offset == 48


def test_positional_store_semantics_host(svdb):
    """insert / read / update / delete as src/vector_database.c:81-195 (host
    side; no GPU call is made).  read_by_uuid is answered by the device's
    uuid index (tests/test_gpu_uuid.py)."""
    db = svdb.VectorDatabase(0, 3)
    rows = [np.full(8, float(i)) for i in range(6)]
    for i, r in enumerate(rows):
        assert db.insert(r, f"uuid-{i}") == i
    assert db.size == 6
    db.delete(2)  # shifts later rows left (src/vector_database.c:189-191)
    assert db.size == 5
    assert np.array_equal(db.read(2), rows[3])
    assert db.uuid(2) == b"uuid-3"
    db.delete(99)  # ignored
    db.update(99, np.zeros(8))  # ignored
    assert db.size == 5
    db.update(0, np.full(8, 42.0))
    assert np.array_equal(db.read(0), np.full(8, 42.0))
    assert db.read(5) is None
    db.close()


def test_compare_validation_host(svdb):
    """Error branches of compare_handler_callback (src/compare_handler.c:86-170)
    for requests that never reach the arithmetic."""
    db = svdb.VectorDatabase(0, 3)
    db.insert(np.ones(4))
    db.insert(np.ones(5))
    db.insert(np.ones(4))
    assert db.compare("/compare/cosine_similarity", 0, 3) == (400, {"error": "Index out of bounds"})
    assert db.compare("/compare/cosine_similarity", -1, 0) == (400, {"error": "Index out of bounds"})
    assert db.compare("/compare/dot_product", 0, 1) == (400, {"error": "Vectors have different dimensions"})
    assert db.compare("/compare/dot_product", 0, 2, expected_dim=5) == (400, {"error": "Vector size mismatch"})
    assert db.compare("/compare/manhattan", 0, 2) == (400, {"error": "Unknown comparison method"})
    db.close()


def test_save_load_roundtrip_and_format(svdb, tmp_path):
    """vector_db_save writes the reference's format (src/vector_database.c:
    212-223): size_t n, then uuid[37], size_t dim, double[dim] per row."""
    db = svdb.VectorDatabase(0, 3)
    r = np.random.default_rng(0)
    X = r.uniform(-1, 1, (7, 5))
    for i, x in enumerate(X):
        db.insert(x, f"{i:036d}")
    f = str(tmp_path / "a.db")
    db.save(f)
    raw = open(f, "rb").read()
    assert len(raw) == 8 + 7 * (37 + 8 + 5 * 8)
    assert int.from_bytes(raw[:8], "little") == 7
    assert raw[8:8 + 36] == b"0" * 36
    assert np.array_equal(np.frombuffer(raw[8 + 45:8 + 45 + 40], np.float64), X[0])
    db2 = svdb.VectorDatabase.load(f, 3)
    assert db2.size == 7
    for i in range(7):
        assert np.array_equal(db2.read(i), X[i])
        assert db2.uuid(i) == f"{i:036d}".encode()
    db.close()
    db2.close()


def test_save_exact_count_option(svdb, tmp_path):
    """A row without data is skipped by the reference's save but still
    counted (src/vector_database.c:213-218): vector_db_save keeps that count,
    svdb_save(SVDB_SAVE_EXACT_COUNT) writes the rows actually written, with
    the same row bytes; both files load back to the complete rows."""
    db = svdb.VectorDatabase(0, 3)
    r = np.random.default_rng(8)
    X = r.uniform(-1, 1, (5, 4))
    for i, x in enumerate(X):
        db.insert(x, f"{i:036d}")
    db.insert(np.zeros(0), "no-data")  # dimension 0: skipped by the save
    db.insert(X[0] + 1.0, "last")
    assert db.size == 7
    f1, f2 = str(tmp_path / "counted.db"), str(tmp_path / "exact.db")
    db.save(f1)
    db.save(f2, exact_count=True)
    raw1, raw2 = open(f1, "rb").read(), open(f2, "rb").read()
    row = 37 + 8 + 4 * 8
    assert len(raw1) == len(raw2) == 8 + 6 * row
    assert int.from_bytes(raw1[:8], "little") == 7  # the reference's count: one row more than the file holds
    assert int.from_bytes(raw2[:8], "little") == 6
    assert raw1[8:] == raw2[8:]
    for f in (f1, f2):  # the drop-in load keeps every complete row of either file
        d2 = svdb.VectorDatabase.load(f, 3)
        assert d2.size == 6
        for i in range(5):
            assert np.array_equal(d2.read(i), X[i])
        assert np.array_equal(d2.read(5), X[0] + 1.0) and d2.uuid(5) == b"last"
        d2.close()
    assert svdb.lib.svdb_save(db.ptr, str(tmp_path / "x.db").encode(), 2) == svdb.EINVAL  # unknown flag
    db.close()


def test_save_file_identical_to_reference(svdb, refstore, tmp_path):
    import oracle as O
    r = np.random.default_rng(5)
    X = r.uniform(-1, 1, (9, 6))
    rs = O.RefStore(refstore, 3)
    db = svdb.VectorDatabase(0, 3)
    for i, x in enumerate(X):
        u = f"{i:08d}-0000-0000-0000-000000000000".encode()
        rs.insert(x, u)
        db.insert(x, u)
    rs.delete(3)
    db.delete(3)
    fr, fo = str(tmp_path / "r.db"), str(tmp_path / "o.db")
    refstore.L.vector_db_save.argtypes = [C.c_void_p, C.c_char_p]
    refstore.L.vector_db_save(rs.db, fr.encode())
    db.save(fo)
    assert open(fr, "rb").read() == open(fo, "rb").read()
    rs.free()
    db.close()


def test_dropin_calls_from_many_threads_host_logic(svdb):
    """The drop-in per-call path's host side (row registry, call combiner,
    grouping by store) driven from 16 threads on stored rows, free vectors
    and rows of two stores at once.  With no GPU every call must come back
    as the failure the reference's callers can see (NaN, or -1.0f for a
    dimension mismatch) -- and nothing may crash or hang."""
    import threading
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present (the GPU test checks the values)")
    r = np.random.default_rng(3)
    dbs = [svdb.VectorDatabase(0, 3), svdb.VectorDatabase(0, 3)]
    for d in dbs:
        for x in r.uniform(-1, 1, (300, 16)):
            d.insert(x)  # staged on the host (no GPU here)
    rows = [[svdb.lib.vector_db_read(d.ptr, i).contents for i in range(300)] for d in dbs]
    free = [svdb.make_vector(r.uniform(-1, 1, 16), owned=False) for _ in range(8)]
    short = svdb.make_vector(np.ones(5), owned=False)
    fns = (svdb.lib.cosine_similarity, svdb.lib.euclidean_distance, svdb.lib.dot_product)
    bad = []

    def work(t):
        g = np.random.default_rng(t)
        for j in range(60):
            m, a, b = int(g.integers(0, 3)), int(g.integers(0, 300)), int(g.integers(0, 300))
            kind = j % 4
            if kind == 0:
                v = fns[m](rows[t % 2][a], rows[t % 2][b])
            elif kind == 1:
                v = fns[m](rows[0][a], rows[1][b])  # rows of two stores
            elif kind == 2:
                v = fns[m](free[a % 8], rows[0][b])
            else:
                v = fns[m](short, rows[0][b])
                if v != np.float32(-1.0):
                    bad.append((t, j, v))
                continue
            if not np.isnan(v):
                bad.append((t, j, v))

    ths = [threading.Thread(target=work, args=(t,)) for t in range(16)]
    for th in ths:
        th.start()
    for th in ths:
        th.join(timeout=120)
        assert not th.is_alive()
    assert not bad, bad[:5]
    for d in dbs:
        d.close()


def test_library_fails_loudly_without_gpu(svdb):
    """No CPU fallback: without a usable GPU every compute call errors."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    db = svdb.VectorDatabase(0, 3)
    db.insert(np.ones(4))
    with pytest.raises(svdb.SvdbError):
        db.search(np.ones(4), 1)
    assert db.kdtree_nearest(np.ones(4)) == -1
    assert np.isnan(svdb.cosine_similarity(np.ones(4), np.ones(4)))
    assert db.read_by_uuid("") is None
    with pytest.raises(svdb.SvdbError):
        db.find_uuid(["a"])
    db.close()


def test_binding_structs_match_the_header(svdb, tmp_path):
    """The Python mirrors of the header's structs (ctypes classes and the
    serving NumPy dtypes) have the C compiler's sizes and field offsets."""
    import shutil

    from svdb_gb300 import serve

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    here = os.path.dirname(os.path.abspath(__file__))
    inc = os.path.join(here, os.pardir, "include")
    mirrors = {
        "svdb_search_stats": svdb.SearchStats,
        "svdb_ragged_part": svdb.RaggedPart,
        "svdb_ragged_info": svdb.RaggedInfo,
    }
    dtypes = {"svdb_request": serve.REQ_DTYPE, "svdb_response": serve.RESP_DTYPE}
    lines = []
    for name, cls in mirrors.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for f in cls._fields_:
            lines.append(f'printf("{name}.{f[0]} %zu\\n", offsetof({name}, {f[0]}));')
    for name, dt in dtypes.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for f in dt.names:
            lines.append(f'printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    src = tmp_path / "layout.c"
    src.write_text("#include <stddef.h>\n#include <stdio.h>\n#include \"svdb_gb300.h\"\nint main(void) {\n" +
                   "\n".join(lines) + "\nreturn 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", inc, str(src), "-o", str(exe)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], check=True, capture_output=True,
                                                  text=True).stdout.splitlines())
    for name, cls in mirrors.items():
        assert int(got[name]) == C.sizeof(cls), name
        for f in cls._fields_:
            assert int(got[f"{name}.{f[0]}"]) == getattr(cls, f[0]).offset, (name, f[0])
    for name, dt in dtypes.items():
        assert int(got[name]) == dt.itemsize, name
        for f in dt.names:
            assert int(got[f"{name}.{f}"]) == dt.fields[f][1], (name, f)
