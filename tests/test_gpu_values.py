"""RLE, Uncompressed, Gorilla, Chimp, Chimp128, Elf and ElfOnChimp on the GPU
against the oracle.

Values, bitmasks and min/max are bit-exact; sums are compensated within each
chunk and combined exactly across chunks, and checked against the oracle's sequential sum (relative 1e-12 of the sum of
magnitudes) and against math.fsum of the same values (2 ulps).
"""
import numpy as np
import pytest

import ebi_gb300 as E
from oracle import oracle as O
from tests.kat import KAT, chunk_option, round_at
from tests.parity import check_query_suite, mask_np, random_mask, random_preds, same_f64, sum_ok

pytestmark = pytest.mark.gpu

VALUE_CODECS = ["uncompressed", "rle", "gorilla", "chimp", "chimp128", "elf_on_chimp", "elf"]
KIND_NAMES = {O.CHUNK_RECORD_COUNT: "record_count", O.CHUNK_BYTE_SIZE: "byte_size", O.CHUNK_FULL: "full"}


def to_pred(spec):
    if spec[0] == "eq":
        return E.Predicate.eq(spec[1])
    if spec[0] == "ne":
        return E.Predicate.ne(spec[1])
    mk = {"none": lambda v: E.RangeValue.NONE, "incl": E.RangeValue.inclusive, "excl": E.RangeValue.exclusive}
    (sk, sv), (ek, ev) = spec[1], spec[2]
    return E.Predicate.range(mk[sk](sv), mk[ek](ev))


@pytest.mark.parametrize("codec", VALUE_CODECS)
@pytest.mark.parametrize("idx", range(len(KAT["filter_cases"])))
def test_kat_filter_cases(codec, idx):
    case = KAT["filter_cases"][idx]
    kind, val = chunk_option(case["chunk"])
    data = E.encode(case["values"], codec, (KIND_NAMES[kind], val))
    d = E.Decoder(data)
    mask = O.mask_from_rows(case["bitmask"], d.n_records) if "bitmask" in case else None
    got = O.rows_from_mask(mask_np(d.filter(to_pred(case["pred"]), mask, case.get("chunk_id"))), d.n_records)
    assert got == case["expect"], case["src"]
    fm = d.filter_materialize(to_pred(case["pred"]), mask, case.get("chunk_id")).cpu().numpy()
    assert same_f64(fm, np.asarray(case["values"], dtype=np.float64)[case["expect"]])
    check_query_suite(data, [to_pred(case["pred"])], masks=(None, mask) if mask is not None else (None,),
                      chunk_ids=(None, case.get("chunk_id")) if "chunk_id" in case else (None,))


@pytest.mark.parametrize("codec", VALUE_CODECS)
@pytest.mark.parametrize("idx", range(len(KAT["agg_cases"])))
def test_kat_agg_cases(codec, idx):
    case = KAT["agg_cases"][idx]
    kind, val = chunk_option(case["chunk"])
    data = E.encode(case["values"], codec, (KIND_NAMES[kind], val))
    d = E.Decoder(data)
    mask = O.mask_from_rows(case["bitmask"], d.n_records) if "bitmask" in case else None
    got = getattr(d, case["op"])(mask)
    assert round_at(got, 100) == round_at(case["expect"], 100), case["src"]


def columns(rng, n):
    walk = np.round(30 + np.cumsum(rng.normal(0, 0.5, n)), 2) + 0.0
    i = np.arange(n)
    sensor = np.round(20 + 10 * np.sin(2 * np.pi * i / 1440) + rng.normal(0, 0.1, n), 4) + 0.0
    lens = rng.geometric(1 / 64, n)
    steps = np.repeat(np.round(50 + np.cumsum(rng.integers(-5, 6, n) * 0.1), 1), lens)[:n] + 0.0
    return {
        "walk": walk,
        "sensor": sensor,
        "steps": steps,
        "uniform": rng.uniform(-1e6, 1e6, n),
        "few": rng.choice([-2.5, 0.0, 1.0, 7.25, 1e300], n),  # repeats, copies from the ring
        "long_runs": np.repeat(rng.normal(0, 1, n // 600 + 1), 600)[:n],  # RLE runs past 255
    }


@pytest.mark.parametrize("codec", VALUE_CODECS)
@pytest.mark.parametrize("kind", ["walk", "sensor", "steps", "uniform", "few", "long_runs"])
@pytest.mark.parametrize("chunk", [("record_count", 8192), ("record_count", 1000), ("byte_size", 20000)])
def test_random_columns(codec, kind, chunk):
    rng = np.random.default_rng(abs(hash((codec, kind, chunk))) % 2**32)
    n = 30_011
    v = columns(rng, n)[kind]
    data = E.encode(v, codec, chunk)
    masks = (None, random_mask(n, 0.3, rng), random_mask(n, 0.001, rng), O.mask_from_rows([], n))
    n_chunks = O.Decoder(data).n_chunks
    check_query_suite(data, random_preds(v, rng), masks=masks,
                      chunk_ids=(None, int(rng.integers(n_chunks)), n_chunks + 3))


@pytest.mark.parametrize("codec", VALUE_CODECS)
def test_full_chunk_sequential_path(codec):
    # one chunk of 20,000 values: more records than the shared-memory decode holds
    rng = np.random.default_rng(11)
    v = np.round(30 + np.cumsum(rng.normal(0, 0.5, 20_000)), 2) + 0.0
    data = E.encode(v, codec, ("full", 0))
    check_query_suite(data, random_preds(v, rng, k=2), masks=(None, random_mask(len(v), 0.4, rng)))


XOR_CODECS = ["gorilla", "chimp", "chimp128", "elf_on_chimp", "elf"]


@pytest.mark.parametrize("codec", XOR_CODECS)
def test_nan_truncates_stream(codec):
    # the XOR readers stop at the first value whose bits equal f64::NAN (parity hazard kept on purpose)
    v = np.round(np.random.default_rng(5).normal(10, 3, 5000), 2)
    v[1234] = np.nan
    v[4100] = np.nan
    data = E.encode(v, codec, ("record_count", 1000))
    check_query_suite(data, [E.Predicate.range(E.RangeValue.inclusive(5.0), E.RangeValue.exclusive(12.0))],
                      masks=(None, random_mask(len(v), 0.5, np.random.default_rng(1))))


@pytest.mark.parametrize("codec", VALUE_CODECS)
def test_tiny_and_empty(codec):
    for v in ([], [1.5], [0.0, -0.0, 0.0], [np.inf, -np.inf, 3.0], [5e-324, -5e-324, 1.0]):
        data = E.encode(np.asarray(v, dtype=np.float64), codec, ("record_count", 2))
        check_query_suite(data, [E.Predicate.eq(0.0), E.Predicate.ne(3.0),
                                 E.Predicate.range(E.RangeValue.NONE, E.RangeValue.inclusive(1.0))])


@pytest.mark.parametrize("codec", VALUE_CODECS)
def test_corrupt_chunks_match_oracle(codec):
    # flipped bits and truncated chunk payloads: same status (or same results) as the oracle
    rng = np.random.default_rng(3)
    v = np.round(30 + np.cumsum(rng.normal(0, 0.5, 6000)), 2) + 0.0
    base = bytes(E.encode(v, codec, ("record_count", 1000)))
    d = O.Decoder(base)
    for trial in range(12):
        data = bytearray(base)
        c = int(rng.integers(d.n_chunks))
        phys, size, _, _ = d.chunk_info(c)
        for _ in range(1 + trial % 3):
            k = phys + int(rng.integers(size))
            data[k] ^= 1 << int(rng.integers(8))
        check_query_suite(bytes(data), [E.Predicate.range(E.RangeValue.inclusive(25.0), E.RangeValue.NONE)],
                          masks=(None,), chunk_ids=(None, c))


@pytest.mark.parametrize("codec", VALUE_CODECS)
def test_full_size_properties(codec):
    # 1,048,576-value random walk in 8,192-value chunks: encode -> decode is the
    # identity, the filter count and min/max equal numpy's, the sum is exact to 2 ulps
    rng = np.random.default_rng(1)
    v = np.round(30.0 + np.cumsum(rng.normal(0.0, 0.5, 1 << 20)), 2) + 0.0
    d = E.Decoder(E.encode(v, codec, ("record_count", 8192)))
    assert same_f64(d.materialize().cpu().numpy(), v)
    p = E.Predicate.range(E.RangeValue.inclusive(10.0), E.RangeValue.inclusive(50.0))
    sel = (v >= 10.0) & (v <= 50.0)
    mask, s, mn, mx, cnt = d.filter_agg(p)
    rows = np.nonzero(np.unpackbits(mask_np(mask).view(np.uint8), bitorder="little")[: len(v)])[0]
    assert np.array_equal(rows, np.nonzero(sel)[0])
    assert cnt == int(sel.sum())
    assert mn == v[sel].min() and mx == v[sel].max()
    assert sum_ok(s, float(np.sum(v[sel])), False, v[sel])
    assert sum_ok(d.sum(), float(np.sum(v)), False, v)


@pytest.mark.parametrize("codec", XOR_CODECS)
@pytest.mark.parametrize("kind", ["walk", "sensor", "few"])
def test_many_small_chunks(codec, kind):
    # >= 1,024 chunks of 64 values: short streams, many CTAs
    rng = np.random.default_rng(abs(hash((codec, kind, "lanes"))) % 2**32)
    n = 80_000
    v = columns(rng, n)[kind]
    data = E.encode(v, codec, ("record_count", 64))
    n_chunks = O.Decoder(data).n_chunks
    assert n_chunks >= 1024
    check_query_suite(data, random_preds(v, rng, k=2), masks=(None, random_mask(n, 0.3, rng)),
                      chunk_ids=(None, int(rng.integers(n_chunks))))


@pytest.mark.parametrize("codec", ["uncompressed", "rle", "gorilla", "chimp128"])
@pytest.mark.parametrize("corrupt", [False, True])
@pytest.mark.parametrize("n", [150_000, 300_000])
def test_fold_over_many_slices(codec, corrupt, n):
    # 2,344 / 4,688 chunks of 64 values: 37 / 74 slices of 64 chunks, so the
    # single-column fold runs over a grid of CTAs with a ticket (and the batch
    # in one CTA)
    rng = np.random.default_rng(23)
    v = columns(rng, n)["walk"]
    data = bytearray(E.encode(v, codec, ("record_count", 64)))
    d = O.Decoder(bytes(data))
    assert d.n_chunks > 32 * 64
    if corrupt:
        for c in (1500, 2100, 2300):  # failing chunks in different slices and CTAs
            phys, size, _, _ = d.chunk_info(c)
            data[phys + size // 2] ^= 0x10
    preds = random_preds(v, rng, k=2)
    check_query_suite(bytes(data), preds, masks=(None, random_mask(n, 0.3, rng)))
    if not corrupt:
        # the batch folds the same slices in one CTA per query: the same bits
        g = E.Decoder(bytes(data))
        got = E.Batch([(g, p, ("sum", "min", "max")) for p in preds]).run()
        for p, (s, mn, mx, cnt) in zip(preds, got):
            _, s1, mn1, mx1, cnt1 = g.filter_agg(p)
            assert same_f64(np.array([s, mn, mx]), np.array([s1, mn1, mx1])) and cnt == cnt1, (p, s, s1)


@pytest.mark.parametrize("codec", VALUE_CODECS)
@pytest.mark.parametrize("chunk", [512, 1000])
def test_output_mask_fully_written(codec, chunk):
    # the output bitmask starts as all ones: every word, the padding past the
    # last row included, must come back as the oracle's (512-row chunks: each
    # chunk's CTA zeroes its own words; 1,000-row chunks share words: a memset)
    rng = np.random.default_rng(31)
    n = 32 * 937 - 5  # an odd number of u32 words: the last u64 word's upper half holds no row
    v = columns(rng, n)["walk"]
    check_mask_words(E.encode(v, codec, ("record_count", chunk)), (None, random_mask(n, 0.2, rng)))


def check_mask_words(data, masks, lo=25.0, hi=35.0):
    """filter / filter_agg into an all-ones output equal the oracle's bitmask in every word."""
    g, o = E.Decoder(data), O.Decoder(data)
    p = E.Predicate.range(E.RangeValue.inclusive(lo), E.RangeValue.inclusive(hi))
    op = O.rng(O.BOUND_INCLUSIVE, lo, O.BOUND_INCLUSIVE, hi)
    for m in masks:
        out = g.new_mask()
        out.fill_(-1)
        g.filter(p, m, out=out)
        want = o.filter(op, m)
        got = mask_np(out)
        assert np.array_equal(got[: len(want)], want) and not got[len(want):].any()
        out.fill_(-1)
        g.filter_agg(p, m, out=out)
        assert np.array_equal(mask_np(out)[: len(want)], want)


def test_rle_runs_past_chunk_rows():
    # a chunk whose run lengths add up to more than its rows: the extra rows
    # take the next chunk's row ids, in the bitmask too, as the reader's do
    rng = np.random.default_rng(37)
    n = 4096
    v = np.repeat(np.round(rng.uniform(20, 40, n // 16), 1), 16)[:n] + 0.0
    data = bytearray(E.encode(v, "rle", ("record_count", 512)))
    d = O.Decoder(bytes(data))
    phys, _, _, _ = d.chunk_info(2)
    data[phys + 8] = 200  # the chunk's first run: 16 -> 200 rows
    check_mask_words(bytes(data), (None, random_mask(n, 0.5, rng)))


@pytest.mark.parametrize("codec", ["chimp", "chimp128", "elf_on_chimp", "elf"])
def test_many_small_chunks_corrupt(codec):
    rng = np.random.default_rng(9)
    v = np.round(30 + np.cumsum(rng.normal(0, 0.5, 70_000)), 2) + 0.0
    base = bytes(E.encode(v, codec, ("record_count", 64)))
    d = O.Decoder(base)
    for trial in range(4):
        data = bytearray(base)
        for _ in range(3):
            c = int(rng.integers(d.n_chunks))
            phys, size, _, _ = d.chunk_info(c)
            data[phys + int(rng.integers(size))] ^= 1 << int(rng.integers(8))
        check_query_suite(bytes(data), [E.Predicate.range(E.RangeValue.inclusive(25.0), E.RangeValue.NONE)],
                          masks=(None,))


def elf_edge_columns(rng, n):
    from tests.test_cpu_abi import mixed_decimals
    near = 10.0 ** rng.integers(-300, 300, n).astype(np.float64)
    near = np.nextafter(near, np.where(rng.random(n) < 0.5, 0.0, np.inf))
    return {
        "decimals": mixed_decimals(rng, n),
        # get_sp's log10 path and the power-of-ten flag (both sides of 10^k)
        "near_powers": np.where(rng.random(n) < 0.5, near, np.round(rng.normal(0, 1, n), 2)),
        "digits": np.round(rng.normal(0, 1e3, n), 1) * 10.0 ** rng.integers(-8, 8, n),
    }


@pytest.mark.parametrize("codec", ["elf_on_chimp", "elf"])
@pytest.mark.parametrize("kind", ["decimals", "near_powers", "digits"])
@pytest.mark.parametrize("chunk", [("record_count", 8192), ("record_count", 777)])
def test_elf_decimal_restoration(codec, kind, chunk):
    # restored values equal the oracle's bit for bit, including the values the
    # reference's power-of-ten test turns into 10^k
    rng = np.random.default_rng(abs(hash((codec, kind, chunk))) % 2**32)
    n = 25_000
    v = elf_edge_columns(rng, n)[kind]
    data = E.encode(v, codec, chunk)
    assert bytes(data) == O.encode(v, codec, O.CHUNK_RECORD_COUNT, chunk[1])
    got = E.Decoder(data).materialize().cpu().numpy()
    assert same_f64(got, O.Decoder(bytes(data)).materialize(None))
    check_query_suite(data, random_preds(v[np.isfinite(v)], rng, k=2), masks=(None, random_mask(n, 0.3, rng)))
