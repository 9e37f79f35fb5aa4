"""Runs the same query through the GPU engine (C ABI) and the C oracle and compares.

Parity bar: bitmasks, materialized values and min/max bit-exact; sums bit-exact
for BUFF (exact integer arithmetic in both) and within a stated relative
tolerance for the codecs whose reference sum is a sequential f64 sum.
"""
from __future__ import annotations

import math

import numpy as np

import ebi_gb300 as E
from oracle import oracle as O

# Relative tolerance of compensated GPU sums against the reference's sequential
# f64 sum (Gorilla, Chimp, Chimp128, RLE, Uncompressed), relative to the sum of
# magnitudes of the summed values (the scale of the sequential sum's own error).
SUM_RTOL = 1e-12
# The GPU sum is a double-double (TwoSum/TwoProd) reduction: against the exact
# sum of the same values (math.fsum) it is off by at most a few ulps.
SUM_EXACT_ULPS = 2


def to_oracle_pred(p: E.Predicate) -> O.Pred:
    if p.kind == 0:
        return O.eq(p.value)
    if p.kind == 1:
        return O.ne(p.value)
    return O.rng(p.rng.start.kind, p.rng.start.value, p.rng.end.kind, p.rng.end.value)


def mask_np(t) -> np.ndarray:
    return t.detach().cpu().numpy().view(np.uint64)


def same_f64(a, b) -> bool:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def same_scalar(a: float, b: float) -> bool:
    """Equal as values (+0 == -0), NaN == NaN."""
    return (a == b) or (np.isnan(a) and np.isnan(b))


def sum_ok(g: float, o: float, exact: bool, vals=None) -> bool:
    """GPU sum g against the oracle's o; vals = the values summed (for the compensated bound)."""
    if exact:
        return same_scalar(g, o)
    if np.isnan(o) or np.isinf(o):
        return same_scalar(g, o)
    if g == o:
        return True
    scale = abs(o)
    if vals is not None and len(vals):
        a = np.abs(np.asarray(vals, dtype=np.float64))
        if np.all(np.isfinite(a)):
            scale = max(scale, float(a.sum()))
            fs = math.fsum(np.asarray(vals, dtype=np.float64).tolist())
            if abs(g - fs) > SUM_EXACT_ULPS * np.spacing(abs(fs)) + 1e-300:
                return False
    return abs(g - o) <= SUM_RTOL * max(scale, 1e-300)


def call(fn, *a, **k):
    """(result, error_code) of fn; error_code 0 on success."""
    try:
        return fn(*a, **k), 0
    except E.DecoderError as e:
        return None, e.code
    except O.OracleError as e:
        return None, e.code


def check_query_suite(data: bytes, preds, masks=(None,), chunk_ids=(None,), exact_sum=None, precision=None):
    """Every operator of the Decoder over every (mask, chunk_id, predicate) combination."""
    g = E.Decoder(data)
    o = O.Decoder(data)
    if precision is not None:
        g.with_precision(precision)
        o.with_precision(precision)
    if exact_sum is None:
        exact_sum = o.scheme == O.BUFF
    try:
        for cid in chunk_ids:
            for m in masks:
                gm, ge = call(g.materialize, m, cid)
                om, oe = call(o.materialize, m, cid)
                assert ge == oe, ("materialize status", ge, oe, cid)
                mat_vals = None if oe else om
                if not ge:
                    assert same_f64(gm.cpu().numpy(), om), ("materialize", cid)
                for name in ("sum", "min", "max"):
                    gv, ge = call(getattr(g, name), m, cid)
                    ov, oe = call(getattr(o, name), m, cid)
                    assert ge == oe, (name, "status", ge, oe)
                    if ge:
                        continue
                    if name == "sum":
                        assert sum_ok(gv, ov, exact_sum, mat_vals), (name, gv, ov, cid)
                    else:
                        assert same_scalar(gv, ov), (name, gv, ov, cid)
                for p in preds:
                    op = to_oracle_pred(p)
                    gf, ge = call(g.filter, p, m, cid)
                    of, oe = call(o.filter, op, m, cid)
                    assert ge == oe, ("filter status", p, ge, oe)
                    if ge:
                        continue
                    assert np.array_equal(mask_np(gf)[: len(of)], of), ("filter", p, cid)
                    gfm, ge = call(g.filter_materialize, p, m, cid)
                    ofm, oe = call(o.filter_materialize, op, m, cid)
                    assert ge == oe
                    assert same_f64(gfm.cpu().numpy(), ofm), ("filter_materialize", p, cid)
                    (gmk, gs, gmn, gmx, gn), ge = call(g.filter_agg, p, m, cid)
                    (omk, os_, omn, omx), oe = call(o.filter_agg, op, m, cid)
                    assert ge == oe
                    assert np.array_equal(mask_np(gmk)[: len(omk)], omk)
                    assert sum_ok(gs, os_, exact_sum, ofm), ("filter_agg sum", p, gs, os_)
                    assert same_scalar(gmn, omn) and same_scalar(gmx, omx), ("filter_agg min/max", p, gmn, omn, gmx, omx)
                    # rows selected = values filter_materialize returns (decoded rows may overlap
                    # the next chunk's in a corrupt file, so this is not always the bitmask's popcount)
                    assert gn == len(ofm), ("filter_agg count", p, gn, len(ofm))
    finally:
        g.close()
        o.close()


def oracle_filter_agg(o: "O.Decoder", p):
    """One filter + aggregate query on the oracle: (bitmask, sum, min, max, count, selected values),
    sum / min / max over the filter's bitmask as the reference's second call computes them."""
    op = to_oracle_pred(p) if isinstance(p, E.Predicate) else p
    m, s, mn, mx = o.filter_agg(op)
    sel = o.filter_materialize(op)
    return m, s, mn, mx, len(sel), sel


def oracle_request(odecs, ids, p):
    """A serving request (one predicate over the columns `ids`) answered by the oracle and combined
    as a request is: per-column sums added in column order, fmin / fmax, counts added.
    Returns (sum, min, max, count, sum of |selected value|)."""
    s, mn, mx, cnt, mag = 0.0, math.inf, -math.inf, 0, 0.0
    for i in ids:
        _, si, mni, mxi, ni, sel = oracle_filter_agg(odecs[i], p)
        s += si
        mn = float(np.fmin(mn, mni))
        mx = float(np.fmax(mx, mxi))
        cnt += ni
        mag += float(np.abs(sel).sum()) if len(sel) else 0.0
    return s, mn, mx, cnt, mag


def combined_sum_ok(g: float, o: float, mag: float) -> bool:
    """A sum combined from several columns' sums: within 1e-12 of the summed magnitudes of the oracle's."""
    if np.isnan(o) or np.isinf(o):
        return same_scalar(g, o)
    return abs(g - o) <= SUM_RTOL * max(mag, 1e-300)


def random_mask(n, density, rng):
    rows = np.nonzero(rng.random(n) < density)[0]
    return O.mask_from_rows(rows.tolist(), n)


def random_preds(values, rng, k=4):
    lo, hi = float(np.min(values)), float(np.max(values))
    span = hi - lo if hi > lo else 1.0
    ps = []
    for _ in range(k):
        a, b = sorted(rng.uniform(lo - 0.1 * span, hi + 0.1 * span, 2))
        kinds = [E.RangeValue.inclusive, E.RangeValue.exclusive, lambda v: E.RangeValue.NONE]
        s = kinds[rng.integers(3)](a)
        e = kinds[rng.integers(3)](b)
        ps.append(E.Predicate.range(s, e))
    v = float(values[rng.integers(len(values))]) if len(values) else 0.0
    ps += [E.Predicate.eq(v), E.Predicate.ne(v), E.Predicate.eq(lo - 1.0)]
    return ps
