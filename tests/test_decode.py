"""POST /nearest bodies decoded on the device (svdb_decode_vectors).

The reference parses a body with cJSON and strtod (src/compare_handler.c:
300-390); cJSON is not part of the reference's sources and its version is not
pinned, so the oracle restates its published grammar (oracle/svdb_oracle.c,
orc_decode_body) and takes numbers from the C library's strtod, as cJSON
does.  CPU tests pin the oracle: every number it decodes equals Python's
correctly rounded float() of the same text, and on standard JSON its
accept/reject decisions match Python's json module.  GPU tests hold the
device decoder to the oracle bit for bit (values and statuses) on a seeded
corpus of every error branch and number style, and at 4,096 bodies of 768
numbers.
"""
import json

import numpy as np
import pytest

from decode_corpus import bodies, number_texts

DIM = 16


def _reject(name):
    raise ValueError(name)


def test_oracle_numbers_are_correctly_rounded(oracle):
    rng = np.random.default_rng(1)
    texts = number_texts(rng, 5000)
    for t in texts:
        st, v = oracle.decode_body(b"[" + t + b"]", 1)
        if st == 0:
            want = float(t.decode()) if not t.startswith(b"-.") else -float(t[1:].decode())
            assert v[0].tobytes() == np.float64(want).tobytes(), t


def test_oracle_grammar_matches_json_on_standard_text(oracle):
    for b in bodies(seed=2, n=1500, dim=DIM):
        try:
            val = json.loads(b.decode("utf-8"), parse_constant=_reject)  # no NaN / Infinity literals
        except (ValueError, UnicodeDecodeError):
            continue  # cJSON's leniencies (BOM, trailing text, control bytes, "-.5") are not standard JSON
        if b"\\u" in b:
            continue  # cJSON rejects lone surrogate escapes that Python's json accepts
        st, v = oracle.decode_body(b, DIM)
        if b.startswith(b"[[[[["):  # cJSON's nesting limit (1,000 containers); Python's json has none
            depth = len(b) - len(b.lstrip(b"["))
            assert st == (1 if depth > 1000 else 3)
            continue
        assert st != 1, b[:80]  # valid JSON is never "Invalid JSON"
        kids = list(val.values()) if isinstance(val, dict) else val if isinstance(val, list) else []
        if len(kids) != DIM:
            assert st == 2
        elif not all(isinstance(x, (int, float)) and not isinstance(x, bool) for x in kids):
            assert st == 3
        else:
            assert st == 0 and np.array_equal(v, np.array(kids, np.float64))


@pytest.mark.gpu
def test_device_decode_matches_oracle_on_corpus(svdb, oracle):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    bs = bodies(seed=3, n=3000, dim=DIM)
    out, st = svdb.decode_vectors(bs, DIM)
    seen = set()
    for i, b in enumerate(bs):
        ost, ov = oracle.decode_body(b, DIM)
        assert st[i] == ost, (i, b[:120], st[i], ost)
        seen.add(ost)
        if ost == 0:
            assert out[i].tobytes() == ov.tobytes(), (i, b[:120])
        else:
            assert np.isnan(out[i]).all()
    assert seen == {0, 1, 2, 3}


@pytest.mark.gpu
def test_device_decode_at_scale(svdb):
    """4,096 bodies of 768 numbers written with %.17g (cJSON's own print
    format for doubles that need it): every value round-trips exactly."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    rng = np.random.default_rng(4)
    X = rng.normal(size=(4096, 768)) * 10.0 ** rng.integers(-8, 8, (4096, 1))
    bs = [("[" + ",".join("%.17g" % x for x in row) + "]").encode() for row in X]
    out, st = svdb.decode_vectors(bs, 768)
    assert (st == 0).all()
    assert out.tobytes() == X.tobytes()
