"""The continuous-batching server: every request's result, answered in the
mix (batched with whatever arrived around it, batches overlapping on the
device), equals the same request answered alone with plain per-column
filter_agg calls, bit for bit, and equals the oracle's answer on the same
columns (count, min and max bit for bit; the sum within the compensated-sum
bound of the oracle's sequential sums, added in column order)."""
import numpy as np
import pytest

import ebi_gb300 as E
from oracle import oracle as O
from tests.parity import combined_sum_ok, oracle_request

pytestmark = pytest.mark.gpu


def columns(rng, n_cols, codecs=("buff", "gorilla", "chimp128", "rle", "elf"), lo=2_000, hi=200_000):
    """(device Decoder, values, oracle Decoder) per column."""
    out = []
    for i in range(n_cols):
        codec = codecs[i % len(codecs)]
        n = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        if codec == "buff":
            v = np.round(rng.uniform(-1000, 1000, n), 3) + 0.0
            data = E.encode(v, "buff", ("record_count", 65536), 1000)
        elif codec == "rle":
            v = np.repeat(np.round(50 + np.cumsum(rng.integers(-5, 6, n // 40 + 1) * 0.1), 1), 40)[:n] + 0.0
            data = E.encode(v, "rle", ("record_count", 8192))
        else:
            v = np.round(30 + np.cumsum(rng.normal(0, 0.5, n)), 2) + 0.0
            data = E.encode(v, codec, ("record_count", 8192))
        out.append((E.Decoder(data), v, O.Decoder(data)))
    return out


def requests(rng, cols, n):
    reqs = []
    for _ in range(n):
        k = int(rng.integers(1, min(8, len(cols)) + 1))
        ids = [int(x) for x in rng.choice(len(cols), size=k, replace=False)]
        vals = np.concatenate([cols[i][1] for i in ids])
        a, b = np.sort(rng.choice(vals, 2))
        p = E.Predicate.range(E.RangeValue.inclusive(float(a)), E.RangeValue.inclusive(float(b)))
        aggs = [("sum", "min", "max"), ("sum",), ("min",), ("max",)][int(rng.integers(4))]
        reqs.append((ids, p, aggs))
    return reqs


def same(x, y):
    return x == y or (np.isnan(x) and np.isnan(y))


def check_oracle(cols, reqs, got):
    odecs = [o for _, _, o in cols]
    for i, ((ids, p, aggs), m) in enumerate(zip(reqs, got)):
        s, mn, mx, cnt, mag = oracle_request(odecs, ids, p)
        assert m["count"] == cnt, (i, m, cnt)
        if "sum" in aggs:
            assert combined_sum_ok(m["sum"], s, mag), (i, m["sum"], s)
        if "min" in aggs:
            assert same(m["min"], mn), (i, m["min"], mn)
        if "max" in aggs:
            assert same(m["max"], mx), (i, m["max"], mx)


@pytest.mark.parametrize("rate", [5_000, 50_000, None])
def test_results_equal_alone_and_in_the_mix(rate):
    rng = np.random.default_rng(7)
    cols = columns(rng, 24)
    decs = [d for d, _, _ in cols]
    reqs = requests(rng, cols, 400)
    alone = E.run_plain(decs, reqs)
    srv = E.Server(decs, slots=4, max_queries=512, max_chunks=1 << 16, max_items=1 << 17)
    arrivals = None
    if rate:
        arrivals = np.cumsum(rng.exponential(1e9 / rate, len(reqs)))
    mixed = srv.replay(reqs, arrivals)
    st = srv.stats()
    srv.close()
    assert st["requests"] == len(reqs)
    for i, (a, m) in enumerate(zip(alone, mixed)):
        assert a["status"] == 0 and m["status"] == 0, i
        assert a["count"] == m["count"], (i, a, m)
        assert same(a["sum"], m["sum"]) and same(a["min"], m["min"]) and same(a["max"], m["max"]), (i, a, m)
        assert m["done_ns"] >= m["launch_ns"] >= m["submit_ns"]
    check_oracle(cols, reqs, mixed)
    if rate is None:  # everything queued at once: requests share batches
        assert st["batches"] < len(reqs)


@pytest.mark.parametrize("codecs", [("chimp128", "gorilla", "chimp"), ("elf", "elf_on_chimp", "gorilla")])
def test_shared_decodes_match_oracle(codecs):
    # Three columns and 300 requests queued at once: every batch holds many queries per
    # column, so a Chimp-family chunk is decoded once for up to 32 of them and a Gorilla
    # chunk group is walked once for up to 8 (up to 3 with the walk's state in registers,
    # more with it in shared memory).  Each answer is checked against the oracle.
    rng = np.random.default_rng(17)
    cols = columns(rng, 3, codecs=codecs, lo=30_000, hi=120_000)
    decs = [d for d, _, _ in cols]
    reqs = []
    for k in range(300):
        ids = [k % 3] if k % 4 else [0, 1, 2]
        vals = np.concatenate([cols[i][1] for i in ids])
        a, b = np.sort(rng.choice(vals, 2))
        p = E.Predicate.range(E.RangeValue.inclusive(float(a)), E.RangeValue.inclusive(float(b)))
        reqs.append((ids, p, [("sum", "min", "max"), ("sum",), ("min",), ("max",)][k % 4]))
    srv = E.Server(decs, slots=2, max_queries=512, max_chunks=1 << 16, max_items=1 << 17)
    mixed = srv.replay(reqs)
    st = srv.stats()
    srv.close()
    assert st["batches"] * 10 <= len(reqs)  # batches of tens of requests: queries share chunks
    for m in mixed:
        assert m["status"] == 0
    check_oracle(cols, reqs, mixed)
    alone = E.run_plain(decs, reqs)
    for a, m in zip(alone, mixed):
        assert a["count"] == m["count"] and same(a["sum"], m["sum"]) and same(a["min"], m["min"]) and same(a["max"], m["max"])


def test_poll_interface():
    rng = np.random.default_rng(3)
    cols = columns(rng, 6)
    decs = [d for d, _, _ in cols]
    srv = E.Server(decs, slots=2, max_queries=64, max_chunks=1 << 14, max_items=1 << 15)
    reqs = requests(rng, cols, 20)
    tickets = [srv.submit(*r) for r in reqs]
    got = {}
    import time
    t0 = time.time()
    while len(got) < len(reqs) and time.time() - t0 < 30:
        for r in srv.poll():
            got[r["ticket"]] = r
    srv.close()
    alone = E.run_plain(decs, reqs)
    assert sorted(got) == sorted(tickets)
    check_oracle(cols, reqs, [got[t] for t in tickets])
    for t, a in zip(tickets, alone):
        m = got[t]
        assert a["count"] == m["count"] and same(a["sum"], m["sum"]) and same(a["min"], m["min"]) and same(a["max"], m["max"])


@pytest.mark.parametrize("tiling", [(1, 1, 8), (16, 16, 64), (3, 5, 24)])
def test_every_tiling_gives_the_same_answers(tiling):
    # BUFF tiles, RLE / Uncompressed chunks and Gorilla chunks per work item change
    # only how the work is cut, never a result: each setting answers as the plain
    # per-column calls do, bit for bit, and as the oracle does.
    rng = np.random.default_rng(23)
    cols = columns(rng, 12, codecs=("buff", "gorilla", "rle", "chimp128"), lo=20_000, hi=400_000)
    decs = [d for d, _, _ in cols]
    reqs = requests(rng, cols, 120)
    bt, vc, gc = tiling
    srv = E.Server(decs, slots=2, max_queries=512, max_chunks=1 << 16, max_items=1 << 17, buff_tiles=bt,
                   value_chunks=vc, gorilla_chunks=gc)
    mixed = srv.replay(reqs)
    st = srv.stats()
    srv.close()
    assert st["items"] > 0
    alone = E.run_plain(decs, reqs)
    for a, m in zip(alone, mixed):
        assert m["status"] == 0
        assert a["count"] == m["count"] and same(a["sum"], m["sum"]) and same(a["min"], m["min"]) and same(a["max"], m["max"])
    check_oracle(cols, reqs, mixed)
