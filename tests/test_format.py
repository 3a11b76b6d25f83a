"""Response bodies printed on the GPU, against the oracle.

The handlers answer GET /compare and POST /nearest with
cJSON_PrintUnformatted (src/compare_handler.c:180-185, :409-424).  cJSON is
not vendored; its published number rule is restated in the oracle with the C
library's own printf ("%1.15g" / "%1.17g") and strtod, exactly as cJSON calls
them, and pinned here against an independent Python restatement of the same
rule (Python's "%.Ng" formatting and float() are correctly rounded, like
glibc's).  On the GPU, svdb_format_compare / svdb_format_nearest must produce
the oracle's bytes exactly: numbers of every magnitude (normal, subnormal,
near the int range, exact decimal ties at 15 and 17 digits), NaN and
infinities ("null"), -0, uuids needing escapes, rows of another dimension,
rows without data, and the two error bodies of /nearest.
"""
import math

import numpy as np
import pytest


def _py_number(d: float) -> bytes:
    """cJSON's number rule, restated in Python (independent of the oracle)."""
    if math.isnan(d) or math.isinf(d):
        return b"null"
    vi = 2147483647 if d >= 2147483647.0 else (-2147483648 if d <= -2147483648.0 else int(d))
    if d == float(vi):
        return b"%d" % vi
    t = "%.15g" % d
    b = float(t)
    if not abs(b - d) <= max(abs(b), abs(d)) * 2.220446049250313e-16:
        t = "%.17g" % d
    return t.encode()


def _corpus(seed: int, n_random: int) -> np.ndarray:
    r = np.random.default_rng(seed)
    vals = [r.normal(size=n_random),
            r.normal(size=n_random) * 10.0 ** r.integers(-300, 300, n_random),
            np.frombuffer(r.integers(0, 2 ** 63, n_random, dtype=np.int64).tobytes(), np.float64),
            np.frombuffer(r.integers(1, 2 ** 52, 256, dtype=np.int64).tobytes(), np.float64),  # subnormals
            -np.frombuffer(r.integers(1, 2 ** 52, 256, dtype=np.int64).tobytes(), np.float64)]
    ties = [(2.0 ** 53 - k) / 4 for k in range(1, 40)]          # 18 digits ending in 5: ties at 17
    ties += [(2.0 ** 48 + 2 * k + 1) / 2 for k in range(40)]     # x.5 with 15 integer digits: ties at 15
    ties += [123456789012345.5, 1234567890123455.0, 2.5, 0.5, 0.125, 1e22, 1e23, 5e-324, 2.2250738585072014e-308,
             1.7976931348623157e308, 0.1, 1 / 3, 2 / 3, 1e-5, 1e-4, 9.9999999999999995e-5, 123456.0, 1e15, 1e16,
             1e17, 2147483647.0, -2147483648.0, 2147483648.0, -2147483649.0, 2147483646.5, 0.0, -0.0, 1.0, -1.0,
             3.0, 1e-7, 99999999999999.99, 999999999999999.9, 1e100, 123e-310]
    vals.append(np.array(ties))
    v = np.concatenate(vals)
    return v[np.isfinite(v)]


def test_oracle_numbers_pinned_to_printf_rule(oracle):
    """The oracle (C printf + strtod, as cJSON) equals the Python restatement."""
    vals = list(_corpus(1, 20000)) + [float("nan"), float("inf"), -float("inf")]
    bad = [(v, oracle.format_number(v), _py_number(v)) for v in vals
           if oracle.format_number(v) != _py_number(v)]
    assert not bad, bad[:5]


def test_oracle_bodies_layout(oracle):
    assert oracle.format_compare(0, np.float32(0.5)) == b'{"cosine_similarity":0.5}'
    assert oracle.format_compare(1, np.float32("nan")) == b'{"euclidean_distance":null}'
    assert oracle.format_compare(2, np.float32(3.0)) == b'{"dot_product":3}'
    assert oracle.format_nearest(1, 3, np.array([1.5, -2.0, 1e-7]), b'a"b\\c\x01\n\x7f\xc3\xa9') == \
        b'{"index":3,"vector":[1.5,-2,1e-07],"uuid":"a\\"b\\\\c\\u0001\\n\x7f\xc3\xa9"}'
    assert oracle.format_nearest(1, 0, np.zeros(0), b"") == b'{"index":0,"vector":[],"uuid":""}'
    assert oracle.format_nearest(0, 0, None, b"") == b'{"error":"No nearest neighbor found"}'
    assert oracle.format_nearest(-1, 9, None, b"") == b'{"error":"Nearest neighbor not found"}'


@pytest.fixture(scope="module")
def S(svdb):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return svdb


@pytest.mark.gpu
@pytest.mark.parametrize("d", [1, 64, 768, 1500])
def test_device_nearest_bodies_equal_oracle(S, oracle, d):
    vals = _corpus(10 + d, 40000)
    rows = max(8, vals.size // d)
    X = np.resize(vals, rows * d).reshape(rows, d)
    r = np.random.default_rng(d)
    X = X[r.permutation(rows)]
    specials = [b"", b"plain-uuid-0000", b'quote"back\\slash', bytes(range(1, 32))[:36], b"\xff\xfe high bytes",
                b"a" * 37]
    db = S.VectorDatabase(0, 3)
    for i in range(rows):
        db.insert(X[i], specials[i % len(specials)])
    got = db.format_nearest(np.arange(rows))
    stored = [db.uuid(i) for i in range(len(specials))]  # as the store keeps them (a 37-byte uuid has no NUL)
    for i in range(rows):
        want = oracle.format_nearest(1, i, X[i], stored[i % len(specials)])
        assert got[i] == want, (i, got[i][:200], want[:200])
    db.close()


@pytest.mark.gpu
def test_device_nearest_special_rows_and_errors(S, oracle):
    db = S.VectorDatabase(0, 3)
    X = np.array([[float("nan"), float("inf"), -float("inf"), -0.0, 0.0, 2147483647.0, 5e-324, 0.1]])
    db.insert(X[0], "specials")
    db.insert(np.array([1.0, 2.0, 3.5]), "other-dimension")  # not in the device store (dimension 3 != 8)
    db.insert(np.zeros(0), "no-data")                          # dimension 0
    db.insert(X[0] * 3.0, "last")
    db.delete(1)  # positions shift; index 3 now reads past the end (a stale KD node's index)
    rows = [X[0], np.zeros(0), X[0] * 3.0]
    uu = [b"specials", b"no-data", b"last"]
    got = db.format_nearest([0, 1, 2, -1, 3, 57])
    for i in range(3):
        assert got[i] == oracle.format_nearest(1, i, rows[i], uu[i]), i
    assert got[3] == b'{"error":"No nearest neighbor found"}'
    assert got[4] == got[5] == b'{"error":"Nearest neighbor not found"}'
    db.insert(np.array([4.0, 5.0, 6.25]), "odd")  # a row of another dimension, now found
    got = db.format_nearest([3])
    assert got[0] == oracle.format_nearest(1, 3, np.array([4.0, 5.0, 6.25]), b"odd")
    db.close()


@pytest.mark.gpu
def test_device_compare_bodies_equal_oracle(S, oracle):
    r = np.random.default_rng(5)
    v = np.concatenate([r.normal(size=3000).astype(np.float32),
                        (r.normal(size=3000) * 10.0 ** r.integers(-40, 38, 3000)).astype(np.float32),
                        np.frombuffer(r.integers(0, 2 ** 31, 2000, dtype=np.int64).astype(np.uint32).tobytes(),
                                      np.float32),
                        np.array([np.nan, np.inf, -np.inf, 0.0, -0.0, 1.0, 0.5, 1e-45, 3.4028235e38, 16777217.0],
                                 np.float32)])
    m = r.integers(0, 3, v.size)
    st = np.zeros(v.size, np.int32)
    st[::97] = r.integers(1, 6, st[::97].size)  # the handler's error statuses
    got = S.format_compare(m, v, st)
    errs = {1: b'{"error": "Index out of bounds"}', 2: b'{"error": "Vector not found"}',
            3: b'{"error": "Vectors have different dimensions"}', 4: b'{"error": "Vector size mismatch"}',
            5: b'{"error": "Unknown comparison method"}'}
    for i in range(v.size):
        want = errs[int(st[i])] if st[i] else oracle.format_compare(int(m[i]), v[i])
        assert got[i] == want, (i, v[i], got[i], want)
