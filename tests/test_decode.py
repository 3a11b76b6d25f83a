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


def _el_numbers(seed):
    """Decimal numbers w x 10^q with 1 to 19 significant digits at every
    decimal exponent from -350 to 315 (the fast conversion's whole table,
    underflow and overflow on both sides), exact ties between two doubles
    that need at most 19 digits, exact ties written with every digit (20 to
    57 characters: the first 19 digits leave the rounding open), and the
    numbers one unit either side of each tie."""
    import random
    from fractions import Fraction
    R = random.Random(seed)
    texts = []
    for q in range(-350, 316):
        for nd in (1, 3, 8, 15, 16, 17, 18, 19):
            w = R.randrange(10 ** (nd - 1), 10 ** nd)
            texts.append(("-" if R.random() < 0.3 else "") + "%de%d" % (w, q))
    for k in range(-3, 10):  # doubles in [2^(53+k), 2^(54+k)) are 2^(k+1) apart
        for _ in range(40):
            n = R.randrange(2 ** 52, 2 ** 53) * 2 ** (k + 1) if k >= -1 else Fraction(R.randrange(2 ** 52, 2 ** 53), 2 ** (-k - 1))
            mid = Fraction(n) + Fraction(2) ** k
            e = min(k, 0)
            W = int(mid * 10 ** (-e))
            for d in (-1, 0, 1):
                texts.append("%de%d" % (W + d, e))
    for j in list(range(0, 10)) + list(range(64, 121, 8)):  # doubles in [2^j, 2^(j+1))
        for _ in range(20):
            t = 53 - j  # the tie is (2m + 1) x 2^-t
            odd = 2 * R.randrange(2 ** 52, 2 ** 53) + 1
            D, e = (odd * 5 ** t, -t) if t > 0 else (odd * 2 ** -t, 0)
            for d in (-1, 0, 1):
                texts.append("%de%d" % (D + d, e))
    return [t.encode() for t in texts]


def test_oracle_numbers_at_every_exponent(oracle):
    """The oracle (cJSON's run + the C library's strtod) on the exponent and
    tie corpus equals Python's correctly rounded float() bit for bit."""
    texts = _el_numbers(5)
    for i in range(0, len(texts), 64):
        chunk = texts[i:i + 64]
        st, v = oracle.decode_body(b"[" + b",".join(chunk) + b"]", len(chunk))
        assert st == 0
        want = np.array([float(t) for t in chunk], np.float64)
        assert v.tobytes() == want.tobytes(), i


@pytest.mark.gpu
def test_device_numbers_at_every_exponent(svdb, oracle):
    """The fast conversion (128-bit powers of five) and the exact fallback it
    hands undecided cases to: every value equals strtod's (the oracle) and
    Python's correctly rounded float()."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    texts = _el_numbers(5)
    texts += [b"0"] * (-len(texts) % 64)
    bs = [b"[" + b",".join(texts[i:i + 64]) + b"]" for i in range(0, len(texts), 64)]
    out, st = svdb.decode_vectors(bs, 64)
    for i, b in enumerate(bs):
        ost, ov = oracle.decode_body(b, 64)
        assert st[i] == ost == 0, (i, st[i], ost)
        want = np.array([float(t) for t in texts[64 * i:64 * i + 64]], np.float64)
        assert ov.tobytes() == want.tobytes()
        bad = np.nonzero(out[i].view(np.int64) != ov.view(np.int64))[0]
        assert bad.size == 0, [(texts[64 * i + j], out[i][j], ov[j]) for j in bad[:5]]


def _long_bodies(dim):
    rng = np.random.default_rng(6)
    errors = [b"1.5.3", b"--1", b"+1", b".5", b"1e", b",", b"", b"1 2", b"9" * 70]
    handover = [b'"x"', b"null", b"[1]", b"{}", b"1\x00", b"\xc3\xa9"]
    bs = []
    for i in range(600):
        nums = number_texts(rng, dim)
        kind = i % 6
        if kind >= 1:
            j = int(rng.integers(0, dim))
            nums[j] = errors[int(rng.integers(0, len(errors)))] if kind in (1, 3) else nums[j]
            j2 = int(rng.integers(0, dim))
            if kind in (2, 3):
                nums[j2] = handover[int(rng.integers(0, len(handover)))]
            if kind == 4:
                nums = nums[:-1]  # size mismatch
            if kind == 5:
                nums = nums + [b"1"]
        sep = [b",", b" ,", b", ", b"\t,\n"][i % 4]
        bs.append(b" " * (i % 7) + b"[" + sep.join(nums) + b"]" + [b"", b"]", b" tail", b"\x00x"][i % 4])
    return bs


@pytest.mark.gpu
def test_device_long_bodies_errors_and_handover(svdb, oracle):
    """Bodies of 300 numbers (many 512-byte steps of the one-warp decoder)
    with an error, a byte only the general parser handles, or both in either
    order, at seeded positions: the first event in the text decides, as in
    cJSON's sequential parse."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    dim = 300
    bs = _long_bodies(dim)
    out, st = svdb.decode_vectors(bs, dim)
    # the same bodies eight times over (4,800 bodies, 25 MB of text: decoded in two chunks on two streams)
    out8, st8 = svdb.decode_vectors(bs * 8, dim)
    assert np.array_equal(st8, np.tile(st, 8))
    assert out8.tobytes() == np.tile(out, (8, 1)).tobytes()
    seen = set()
    for i, b in enumerate(bs):
        ost, ov = oracle.decode_body(b, dim)
        assert st[i] == ost, (i, st[i], ost)
        seen.add(ost)
        if ost == 0:
            assert out[i].tobytes() == ov.tobytes(), i
        else:
            assert np.isnan(out[i]).all(), i
    assert seen == {0, 1, 2, 3}
