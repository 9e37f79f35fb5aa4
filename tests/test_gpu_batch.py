"""ebi_batch (one persistent mixed-codec launch for many queries) against the
oracle and against the single-column ebi_filter_agg: every query's bitmask,
min, max and count equal the oracle's Decoder on the same bytes bit for bit,
its sum is exact (BUFF) or within the compensated-sum bound of the oracle's
sequential sum, and all of them are bit-identical to the same query run alone."""
import json

import numpy as np
import pytest

import ebi_gb300 as E
from oracle import oracle as O
from tests.parity import mask_np, oracle_filter_agg, random_preds, same_scalar, sum_ok

pytestmark = pytest.mark.gpu


def make_columns(rng, n_cols):
    cols = []
    codecs = ["buff", "gorilla", "chimp128", "rle", "chimp", "uncompressed", "elf", "elf_on_chimp"]
    for i in range(n_cols):
        codec = codecs[i % len(codecs)]
        n = int(rng.integers(1, 60_000)) if i % 5 else int(rng.integers(60_000, 300_000))
        walk = np.round(30 + np.cumsum(rng.normal(0, 0.5, n)), 2) + 0.0
        if codec == "buff":
            v = np.round(rng.uniform(-1000, 1000, n), 3) + 0.0
            data = E.encode(v, "buff", ("record_count", [65536, 8192, 1000][i % 3]), 1000)
        elif codec == "rle":
            v = np.repeat(np.round(rng.normal(0, 5, n // 30 + 1), 1), 30)[:n] + 0.0
            data = E.encode(v, "rle", ("record_count", 8192))
        else:
            v = walk
            data = E.encode(v, codec, ("record_count", [8192, 4096, 20000][i % 3]))
        cols.append((E.Decoder(data), v, O.Decoder(data), codec))
    return cols


def alone(d, p, aggs):
    m, s, mn, mx, n = d.filter_agg(p, aggregates=aggs)
    return m, s, mn, mx, n


def same(a, b):
    return a is None and b is None or a == b or (np.isnan(a) and np.isnan(b))


@pytest.mark.parametrize("seed", [1, 2])
def test_batch_matches_single_queries(seed):
    rng = np.random.default_rng(seed)
    cols = make_columns(rng, 30)
    queries, expect = [], []
    for k in range(45):  # some columns appear in several queries
        d, v = cols[k % len(cols)][:2]
        p = random_preds(v, rng, k=1)[int(rng.integers(4))]
        aggs = [("sum", "min", "max"), ("sum",), ("max",)][k % 3]
        queries.append((d, p, aggs))
    b = E.Batch(queries, want_masks=True)
    for rnd in range(2):
        if rnd == 1:  # new predicates, same graph
            preds = []
            for k, (d, p, aggs) in enumerate(queries):
                preds.append(random_preds(cols[k % len(cols)][1], rng, k=1)[0])
            queries = [(d, p, a) for (d, _, a), p in zip(queries, preds)]
            got = b.run(preds)
        else:
            got = b.run()
        for k, (d, p, aggs) in enumerate(queries):
            m, s, mn, mx, n = alone(d, p, aggs)
            gs, gmn, gmx, gn = got[k]
            _, _, o, codec = cols[k % len(cols)]
            om, os_, omn, omx, on, sel = oracle_filter_agg(o, p)
            assert gn == on, (k, gn, on)
            assert np.array_equal(mask_np(b.masks[k])[: len(om)], om), k
            if "sum" in aggs:
                assert sum_ok(gs, os_, codec == "buff", sel), (k, codec, gs, os_)
            if "min" in aggs:
                assert same_scalar(gmn, omn), (k, gmn, omn)
            if "max" in aggs:
                assert same_scalar(gmx, omx), (k, gmx, omx)
            assert gn == n, (k, gn, n)
            assert same(gs, s) and same(gmn, mn) and same(gmx, mx), (k, gs, s, gmn, mn, gmx, mx)
            assert np.array_equal(mask_np(b.masks[k]), mask_np(m)), k
    info = b.info()
    assert info["shape"] >= 0 and info["queries"] == 45
    b.close()


def test_batch_reports_a_failing_query():
    rng = np.random.default_rng(4)
    good = E.Decoder(E.encode(np.round(rng.normal(0, 1, 5000), 3), "gorilla", ("record_count", 1000)))
    data = bytearray(E.encode(np.round(rng.uniform(-1, 1, 5000), 3), "buff", ("record_count", 1000), 1000))
    phys, size, _, _ = E.Decoder(bytes(data)).chunk_info(2)
    data[phys + 12] = 40  # the chunk's header claims more bits than its bytes hold
    bad = E.Decoder(bytes(data))
    p = E.Predicate.range(E.RangeValue.inclusive(-0.5), E.RangeValue.inclusive(0.5))
    b = E.Batch([(good, p), (bad, p)])
    with pytest.raises(E.UnexpectedEndOfChunk):
        b.run()
    st = b.statuses()
    assert st[0] == 0 and st[1] == E.UnexpectedEndOfChunk.code
    b.close()


def test_tiling_is_tuned_cached_and_exact(tmp_path):
    # Columns of every codec family in the two smaller size buckets: the first run
    # times the launch shapes and then the tiles per item of each (family, bucket)
    # present; whatever it picks, every query equals the oracle and the query run
    # alone.  A second batch of the same column shape takes the choice from the
    # tuning cache (no timing) and gives the same bits.
    rng = np.random.default_rng(9)
    cols = make_columns(rng, 24)
    queries = []
    for k, (d, v, _, _) in enumerate(cols):
        aggs = [("sum", "min", "max"), ("sum",), ("min",), ("max",)][k % 4]
        queries.append((d, random_preds(v, rng, k=1)[0], aggs))
    path = tmp_path / "tuning.json"
    E.Batch.set_tuning_cache(path)
    try:
        b = E.Batch(queries, want_masks=True)
        got = b.run()
        info = b.info()
        knobs = {t["knob"] for t in info["trials"]}
        assert {"shape", "buff_tiles", "value_chunks", "gorilla_chunks"} <= knobs, knobs
        assert not info["from_cache"] and info["items"] > 0 and info["best_ms"] > 0
        assert sum(t["kept"] for t in info["trials"] if t["knob"] == "shape") == 1
        for k, (d, p, aggs) in enumerate(queries):
            m, s, mn, mx, n = alone(d, p, aggs)
            gs, gmn, gmx, gn = got[k]
            om, os_, omn, omx, on, sel = oracle_filter_agg(cols[k][2], p)
            assert gn == on == n, k
            assert np.array_equal(mask_np(b.masks[k])[: len(om)], om), k
            assert same(gs, s) and same(gmn, mn) and same(gmx, mx), k
            if "sum" in aggs:
                assert sum_ok(gs, os_, cols[k][3] == "buff", sel), k
            if "min" in aggs:
                assert same_scalar(gmn, omn), k
            if "max" in aggs:
                assert same_scalar(gmx, omx), k
        cache = json.loads(path.read_text())
        assert len(cache) == 1
        entry = next(iter(cache.values()))
        assert entry["buff_tiles"] == info["buff_tiles"] and entry["gorilla_chunks"] == info["gorilla_chunks"]
        assert entry["value_chunks"] == info["value_chunks"] and entry["ctas_per_sm"] == info["ctas_per_sm"]
        b2 = E.Batch(queries)
        got2 = b2.run()
        info2 = b2.info()
        assert info2["from_cache"] and not info2["trials"]
        assert info2["buff_tiles"] == info["buff_tiles"] and info2["value_chunks"] == info["value_chunks"]
        for a, c in zip(got, got2):
            assert all(same(x, y) for x, y in zip(a, c))
        b.close()
        b2.close()
    finally:
        E.Batch.set_tuning_cache(None)


def test_queries_on_one_column_share_decodes():
    # Twelve queries on each of four columns, interleaved: the batch runs them grouped by
    # column, so a Chimp128 chunk is decoded once for all twelve and a Gorilla chunk group is
    # walked twice (8 + 4 queries); results come back in the caller's order and equal the
    # oracle and the queries run alone, also after new predicates are set.
    rng = np.random.default_rng(12)
    cols = []
    for codec in ("chimp128", "gorilla", "buff", "rle"):
        n = 70_000
        if codec == "buff":
            v = np.round(rng.uniform(-1000, 1000, n), 3) + 0.0
            data = E.encode(v, "buff", ("record_count", 65536), 1000)
        elif codec == "rle":
            v = np.repeat(np.round(rng.normal(0, 5, n // 30 + 1), 1), 30)[:n] + 0.0
            data = E.encode(v, "rle", ("record_count", 8192))
        else:
            v = np.round(30 + np.cumsum(rng.normal(0, 0.5, n)), 2) + 0.0
            data = E.encode(v, codec, ("record_count", 8192))
        cols.append((E.Decoder(data), v, O.Decoder(data), codec))
    queries = []
    for k in range(48):
        d, v, _, _ = cols[k % 4]
        queries.append((d, random_preds(v, rng, k=1)[0], [("sum", "min", "max"), ("sum",), ("min",), ("max",)][k % 4]))
    b = E.Batch(queries)
    for rnd in range(2):
        if rnd == 1:
            preds = [random_preds(cols[k % 4][1], rng, k=1)[0] for k in range(48)]
            queries = [(d, p, a) for (d, _, a), p in zip(queries, preds)]
            got = b.run(preds)
        else:
            got = b.run()
        for k, (d, p, aggs) in enumerate(queries):
            m, s, mn, mx, n = alone(d, p, aggs)
            gs, gmn, gmx, gn = got[k]
            om, os_, omn, omx, on, sel = oracle_filter_agg(cols[k % 4][2], p)
            assert gn == on == n, k
            assert same(gs, s) and same(gmn, mn) and same(gmx, mx), k
            if "sum" in aggs:
                assert sum_ok(gs, os_, cols[k % 4][3] == "buff", sel), k
            if "min" in aggs:
                assert same_scalar(gmn, omn), k
            if "max" in aggs:
                assert same_scalar(gmx, omx), k
    b.close()
