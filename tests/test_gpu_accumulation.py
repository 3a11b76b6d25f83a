"""The screen's accumulation model, measured.

The exact top-k rests on one assumption about hardware the vendor does not
document: the tensor core's FP32 accumulation of K products stays within
c_acc |bq| |bx| of their exact sum, with

    BF16 (kind::f16):     c_acc = (ldb / 16 + 1) x 20 x 2^-23
    E4M3 (kind::f8f6f4):  c_acc = (ldb8 / 32 + 1) x 40 x 2^-13

(bq, bx the operands the MMAs read).  These tests run the screen kernel in
its diagnostic form (same pipeline, the epilogue stores the raw
accumulators), in both its single-CTA (M = 128) and paired (cta_group::2,
M = 256) forms, and compare every accumulator with the exact sum of the same
products, computed in FP64 from the returned operands (products of BF16 or
E4M3 values are exact in FP64; the FP64 sum's own rounding is below 2^-44 of
|bq| |bx| here).  Inputs are chosen to stress the accumulation: heavy
cancellation (sums that are exactly zero after partial sums of the full
magnitude), exponents spread over 2^-20 .. 2^20, many equal-sign addends,
large products first and small ones after, at D up to 1536.  The largest
observed error as a fraction of the modelled bound is printed at the end of
the run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S(svdb):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return svdb


def _bf16_to_f64(b):
    u = b.view(np.uint16).astype(np.uint32) << 16
    return u.view(np.float32).astype(np.float64)


_E4M3 = np.zeros(256)
for _c in range(256):
    _s, _e, _m = _c >> 7, (_c >> 3) & 15, _c & 7
    _v = (_m / 8.0) * 2.0 ** -6 if _e == 0 else (1 + _m / 8.0) * 2.0 ** (_e - 7)
    _E4M3[_c] = np.nan if (_e == 15 and _m == 7) else (-_v if _s else _v)


def _cases(rng, d, n):
    """Row blocks and query blocks of each stress pattern (n rows / queries each)."""
    h = d // 2
    rows, qs = [], []
    # plain Gaussian
    rows.append(rng.normal(size=(n, d)))
    qs.append(rng.normal(size=(n, d)))
    # cancellation: q = [v, -v], x = [u, u] -> every q.x is exactly 0 after
    # partial sums as large as |q| |x| / 2
    u = rng.normal(size=(n, h))
    v = rng.normal(size=(n, h))
    rows.append(np.hstack([u, u]))
    qs.append(np.hstack([v, -v]))
    # exponents spread over 2^-20 .. 2^20, random signs
    rows.append(rng.choice([-1.0, 1.0], (n, d)) * 2.0 ** rng.uniform(-20, 20, (n, d)))
    qs.append(rng.choice([-1.0, 1.0], (n, d)) * 2.0 ** rng.uniform(-20, 20, (n, d)))
    # many equal-sign addends of similar size (the running sum grows linearly)
    rows.append(1.0 + 0.01 * rng.random((n, d)))
    qs.append(1.0 + 0.01 * rng.random((n, d)))
    # large products first, then many small ones of the same sign
    big = np.where(np.arange(d) < 16, 2.0 ** 12, 2.0 ** -6)
    rows.append(big * (1.0 + 0.1 * rng.random((n, d))))
    qs.append(big * (1.0 + 0.1 * rng.random((n, d))))
    # a large positive block cancelled by a large negative block, with small terms between
    w = np.where(np.arange(d) < h, 1.0, -1.0) * (2.0 ** 8) * (1.0 + 0.05 * rng.random((n, d)))
    w[:, h - 8:h + 8] = 2.0 ** -8 * rng.normal(size=(n, 16))
    rows.append(np.abs(w))
    qs.append(w)
    return np.vstack(rows), np.vstack(qs)


def _measure(S, d, metric, prec, seed):
    rng = np.random.default_rng(seed)
    X, Qall = _cases(rng, d, 128)
    db = S.VectorDatabase(0, 3)
    db.insert_batch(X)
    db.sync()
    worst = 0.0
    worst_units = 0.0
    # blocks of 256 queries run the paired form (cta_group::2, M = 256 over two
    # SMs), blocks of 128 the single-CTA form (M = 128): both are measured
    for q0, q1 in ((0, 256), (256, 384), (384, 640), (640, 768)):
        Q = Qall[q0:q1]
        acc, qo, ro = db.screen_accumulators(Q, metric, prec, X.shape[0])
        if prec == S.PREC_BF16:
            bq, bx = _bf16_to_f64(qo), _bf16_to_f64(ro)
            c_acc = (qo.shape[1] // 2 // 16 + 1) * 20 * 2.0 ** -23
        else:
            bq, bx = _E4M3[qo], _E4M3[ro]
            c_acc = (qo.shape[1] // 32 + 1) * 40 * 2.0 ** -13
        assert np.isfinite(bq).all() and np.isfinite(bx).all()
        exact = bq @ bx.T
        scale = np.linalg.norm(bq, axis=1)[:, None] * np.linalg.norm(bx, axis=1)[None, :]
        ok = scale > 0
        err = np.abs(acc.astype(np.float64) - exact)
        assert (err[~ok] == 0).all()
        rel = np.where(ok, err / np.where(ok, scale, 1.0), 0.0)
        assert np.isfinite(acc).all()
        assert (rel <= c_acc).all(), (rel.max() / c_acc, np.unravel_index(rel.argmax(), rel.shape))
        worst = max(worst, rel.max() / c_acc)
        worst_units = max(worst_units, rel.max() / 2.0 ** -23)
    db.close()
    return worst, worst_units


@pytest.mark.parametrize("d", [64, 768, 1536])
@pytest.mark.parametrize("metric", [0, 2])
def test_bf16_accumulation_within_model(S, parity_report, d, metric):
    worst, units = _measure(S, d, metric, S.PREC_BF16, 1000 + d + metric)
    parity_report.append(f"kind::f16 accumulation, D={d} {('cosine (unit-norm shadow)', '', 'dot (plain shadow)')[metric]}"
                         f": largest |acc - exact| = {units:.3g} x 2^-23 |bq||bx| = {worst:.3g} of the modelled c_acc")


@pytest.mark.parametrize("d", [64, 768, 1536])
@pytest.mark.parametrize("metric", [0, 2])
def test_e4m3_accumulation_within_model(S, parity_report, d, metric):
    worst, units = _measure(S, d, metric, S.PREC_FP8, 2000 + d + metric)
    shadow = ("cosine (E4M3 unit-norm shadow)", "", "dot (E4M3 shadow, per-row power of two)")[metric]
    parity_report.append(f"kind::f8f6f4 accumulation, D={d} {shadow}: largest |acc - exact| = "
                         f"{units:.3g} x 2^-23 |bq||bx| = {worst:.3g} of the modelled c_acc")
