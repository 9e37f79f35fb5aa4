"""The benchmark configurations at their full sizes, on the GPU against the oracle.

Each configuration's own column (the seeded generators the bench uses, at the
bench's row count and chunking) is queried through the C ABI and through the
oracle's Decoder on the same EBI1 bytes, the way ebi's differential tests run
one decoder against another (ebi/tests/query.rs:69-111,
ebi/tests/aggregation.rs:246-300):

  * bitmasks, materialized values, min/max and selected-row counts: bit for bit;
  * BUFF sums: bit for bit (exact integer sums on both sides);
  * Gorilla / Chimp128 / RLE sums: relative error against the oracle's
    sequential f64 sum, |gpu - oracle| / |oracle|, at most 1e-12 (and within
    the general bound of tests/parity.py: 1e-12 of the sum of magnitudes and
    2 ulps of the exactly rounded sum).

The oracle runs chunk-parallel on every host core, so each configuration takes
seconds.
"""
import math
import os

import numpy as np
import pytest

import ebi_gb300 as E
from ebi_gb300 import workloads as W
from oracle import oracle as O
from tests.parity import mask_np, same_f64, same_scalar, sum_ok

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
REL_TOL = 1e-12  # compensated sums vs the oracle's sequential sum, relative to |sum|


def incl(a, b):
    return (E.Predicate.range(E.RangeValue.inclusive(a), E.RangeValue.inclusive(b)),
            O.rng(O.BOUND_INCLUSIVE, a, O.BOUND_INCLUSIVE, b))


def check_sum(g, o, exact, vals):
    if exact:
        assert same_scalar(g, o), (g, o)
        return 0.0
    assert sum_ok(g, o, False, vals), (g, o)
    rel = abs(g - o) / abs(o) if o else abs(g)
    assert rel <= REL_TOL, (g, o, rel)
    # the exactly rounded sum of the same values, for the record
    assert abs(g - math.fsum(vals.tolist())) <= 2 * np.spacing(abs(o)) + 1e-300
    return rel


def check_filter_agg(g, o, gp, op, exact, aggs=("sum", "min", "max")):
    """filter + aggregates over its bitmask: the fused GPU call against the oracle's
    filter, filter_materialize and sum / min / max over the filter's bitmask."""
    gm, gs, gmn, gmx, gn = g.filter_agg(gp, aggregates=aggs)
    om = o.filter(op)
    assert np.array_equal(mask_np(gm)[: len(om)], om)
    sel = o.filter_materialize(op)
    assert gn == len(sel) == int(np.unpackbits(om.view(np.uint8)).sum())
    rel = None
    if "sum" in aggs:
        rel = check_sum(gs, o.sum(om), exact, sel)
    if "min" in aggs:
        assert same_scalar(gmn, o.min(om)), (gmn, o.min(om))
    if "max" in aggs:
        assert same_scalar(gmx, o.max(om)), (gmx, o.max(om))
    # the same query through the reference's two calls on the GPU: filter, then the aggregates
    m2 = g.filter(gp)
    assert np.array_equal(mask_np(m2)[: len(om)], om)
    if "max" in aggs:
        assert same_scalar(g.max(m2), gmx)
    return rel


def open_both(values, codec, chunk, scale=1):
    data = E.encode(values, codec, ("record_count", chunk), scale)
    # the oracle's encoder writes the same file
    assert data == O.encode(values, codec, O.CHUNK_RECORD_COUNT, chunk, scale)
    return E.Decoder(data), O.Decoder(data, threads=THREADS)


def check_materialize(g, o, values=None):
    got = g.materialize().cpu().numpy()
    want = o.materialize()
    assert same_f64(got, want)
    if values is not None:  # lossless codecs: encode -> decode is the identity
        assert same_f64(got, values)
    return got


def test_c1_gorilla_1m():
    # 1,048,576-value random walk (x0 = 30, N(0, 0.5) steps, 2 decimals), 8,192-value chunks:
    # decode all, filter 10 <= x <= 50 to a bitmask, sum / min / max over it and unfiltered
    v = W.gorilla_walk(1_048_576)
    g, o = open_both(v, "gorilla", 8192)
    assert g.n_chunks == 128
    check_materialize(g, o, v)
    gp, op = incl(10.0, 50.0)
    check_filter_agg(g, o, gp, op, exact=False)
    check_sum(g.sum(), o.sum(), False, v)
    assert same_scalar(g.min(), o.min()) and same_scalar(g.max(), o.max())


@pytest.fixture(scope="module")
def c2():
    v = W.buff_uniform(67_108_864)
    g, o = open_both(v, "buff", 65_536, 1000)
    yield g, o
    g.close()
    o.close()


@pytest.mark.parametrize("sel", list(W.BUFF_RANGES))
def test_c2_buff_67m_filter_sum(c2, sel):
    # 67,108,864 values U[-1000, 1000] at 3 decimals, 65,536-value chunks, scale 1000:
    # the headline query (filter to a bitmask + sum) at 1 %, 10 % and 50 % selectivity
    g, o = c2
    assert g.n_chunks == 1024
    a = W.BUFF_RANGES[sel]
    gp, op = incl(-a, a)
    check_filter_agg(g, o, gp, op, exact=True)


def test_c2_buff_67m_materialize(c2):
    # full materialize: the fixed-point values trunc(x * 2^11) / 2^11, as the reference decodes them
    g, o = c2
    got = check_materialize(g, o)
    assert len(got) == 67_108_864
    check_sum(g.sum(), o.sum(), True, None)
    assert same_scalar(g.min(), o.min()) and same_scalar(g.max(), o.max())


def test_c3a_chimp128_16m():
    # 16,777,216-value sensor series (20 + 10 sin(2 pi i / 1440) + N(0, 0.1), 4 decimals),
    # 8,192-value chunks: decode + max, decode + filter 15 <= x <= 25
    v = W.sensor(16_777_216)
    g, o = open_both(v, "chimp128", 8192)
    check_materialize(g, o, v)
    assert same_scalar(g.max(), o.max())
    gp, op = incl(15.0, 25.0)
    check_filter_agg(g, o, gp, op, exact=False, aggs=("max",))
    check_filter_agg(g, o, gp, op, exact=False)


def test_c3b_rle_16m():
    # 16,777,216-value step series (Geometric(1/64) runs, levels moving by U{-5..5} * 0.1):
    # decode + max, decode + filter over the middle 30 % of the values
    v = W.steps(16_777_216)
    g, o = open_both(v, "rle", 8192)
    check_materialize(g, o, v)
    assert same_scalar(g.max(), o.max())
    lo, hi = (float(x) for x in np.quantile(v, [0.35, 0.65]))
    gp, op = incl(lo, hi)
    check_filter_agg(g, o, gp, op, exact=False, aggs=("max",))
    check_filter_agg(g, o, gp, op, exact=False)


@pytest.mark.parametrize("codec", ["elf", "elf_on_chimp", "chimp"])
def test_sensor_16m_other_xor_codecs(codec):
    # the Elf workloads of the bench (C3a's series and query through the Elf codecs) and plain Chimp
    v = W.sensor(16_777_216)
    g, o = open_both(v, codec, 8192)
    check_materialize(g, o, v)
    gp, op = incl(15.0, 25.0)
    check_filter_agg(g, o, gp, op, exact=False)
