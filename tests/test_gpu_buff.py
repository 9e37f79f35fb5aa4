"""BUFF on the GPU against the oracle (parity tests, need a GB300)."""
import numpy as np
import pytest
import torch

import ebi_gb300 as E
from oracle import oracle as O
from tests.kat import KAT, chunk_option, round_at
from tests.parity import check_query_suite, mask_np, random_mask, random_preds, same_f64

pytestmark = pytest.mark.gpu

KIND_NAMES = {O.CHUNK_RECORD_COUNT: "record_count", O.CHUNK_BYTE_SIZE: "byte_size", O.CHUNK_FULL: "full"}


def enc(values, chunk, scale):
    return E.encode(values, "buff", chunk, scale)


def to_pred(spec):
    if spec[0] == "eq":
        return E.Predicate.eq(spec[1])
    if spec[0] == "ne":
        return E.Predicate.ne(spec[1])
    mk = {"none": lambda v: E.RangeValue.NONE, "incl": E.RangeValue.inclusive, "excl": E.RangeValue.exclusive}
    (sk, sv), (ek, ev) = spec[1], spec[2]
    return E.Predicate.range(mk[sk](sv), mk[ek](ev))


@pytest.mark.parametrize("idx", range(len(KAT["filter_cases"])))
def test_kat_filter_cases(idx):
    case = KAT["filter_cases"][idx]
    kind, val = chunk_option(case["chunk"])
    data = enc(case["values"], (KIND_NAMES[kind], val), KAT["filter_buff_scale"])
    d = E.Decoder(data)
    mask = O.mask_from_rows(case["bitmask"], d.n_records) if "bitmask" in case else None
    got = O.rows_from_mask(mask_np(d.filter(to_pred(case["pred"]), mask, case.get("chunk_id"))), d.n_records)
    assert got == case["expect"], case["src"]
    fm = d.filter_materialize(to_pred(case["pred"]), mask, case.get("chunk_id")).cpu().numpy()
    want = np.asarray(case["values"])[case["expect"]]
    np.testing.assert_array_equal(round_at(fm, 100), round_at(want, 100))
    check_query_suite(data, [to_pred(case["pred"])], masks=(None, mask) if mask is not None else (None,),
                      chunk_ids=(None, case.get("chunk_id")) if "chunk_id" in case else (None,))


@pytest.mark.parametrize("idx", range(len(KAT["agg_cases"])))
def test_kat_agg_cases(idx):
    case = KAT["agg_cases"][idx]
    kind, val = chunk_option(case["chunk"])
    data = enc(case["values"], (KIND_NAMES[kind], val), KAT["agg_buff_scale"])
    d = E.Decoder(data)
    mask = O.mask_from_rows(case["bitmask"], d.n_records) if "bitmask" in case else None
    got = getattr(d, case["op"])(mask)
    if case["op"] == "sum":
        assert abs(got - case["expect"]) < 0.5 * len(case["values"])
    else:
        assert round_at(got, 100) == round_at(case["expect"], 100)


# Columns that exercise every BUFF layout: constant (bits 0), tail only
# (bits < 8), exactly one plane, planes + tail, and wide (> 32 bits).
def layouts(rng, n):
    return {
        "const": np.full(n, -12.5),
        "narrow": np.round(rng.integers(0, 100, n) / 1000.0 + 5.0, 3),
        "one_plane": np.round(rng.integers(0, 200, n) / 100.0, 2),
        "planes_tail": np.round(rng.uniform(-1000, 1000, n), 3),
        "wide": np.round(rng.uniform(-2.0e7, 2.0e7, n), 3),
        "walk": np.round(30 + np.cumsum(rng.normal(0, 0.5, n)), 2),
    }


@pytest.mark.parametrize("layout", ["const", "narrow", "one_plane", "planes_tail", "wide", "walk"])
@pytest.mark.parametrize("chunk", [("record_count", 65536), ("record_count", 1000), ("record_count", 8197),
                                   ("byte_size", 30000)])
def test_random_layouts(layout, chunk):
    rng = np.random.default_rng(hash((layout, chunk)) % 2**32)
    n = 70_003
    v = layouts(rng, n)[layout] + 0.0
    data = enc(v, chunk, 1000)
    nrec = n
    masks = (None, random_mask(nrec, 0.3, rng), random_mask(nrec, 0.001, rng), O.mask_from_rows([], nrec))
    preds = random_preds(v, rng)
    n_chunks = O.Decoder(data).n_chunks
    check_query_suite(data, preds, masks=masks, chunk_ids=(None, int(rng.integers(n_chunks)), n_chunks + 3))


@pytest.mark.parametrize("order", ["narrow_first", "wide_first"])
def test_mixed_chunk_widths(order):
    # chunks of 10, 14, 21 and 31 bits in one column: the scan kernel is built
    # for the most common width and runs the others through its general path
    rng = np.random.default_rng(7 if order == "narrow_first" else 8)
    parts = [np.round(rng.uniform(0, 1, 12_000), 3), np.round(rng.uniform(0, 16, 8_192), 3),
             np.round(rng.uniform(-1000, 1000, 30_000), 3), np.round(rng.uniform(-1e6, 1e6, 9_000), 3)]
    if order == "wide_first":
        parts = parts[::-1]
    v = np.concatenate(parts) + 0.0
    data = enc(v, ("record_count", 4096), 1000)
    masks = (None, random_mask(len(v), 0.3, rng), random_mask(len(v), 0.01, rng))
    n_chunks = O.Decoder(data).n_chunks
    check_query_suite(data, random_preds(v, rng, k=6), masks=masks,
                      chunk_ids=(None, 0, int(rng.integers(n_chunks)), n_chunks - 1))


@pytest.mark.parametrize("chunk", [("record_count", 65536), ("record_count", 1000), ("byte_size", 30000)])
def test_open_from_pinned_host_memory(chunk):
    # a pinned file is repacked by the device straight from host memory; the
    # result equals opening the same bytes from pageable memory
    import torch
    rng = np.random.default_rng(5)
    v = np.concatenate([np.round(rng.uniform(-1000, 1000, 50_003), 3), np.round(rng.uniform(0, 1, 7_000), 3)]) + 0.0
    data = bytes(enc(v, chunk, 1000))
    for offset in (0, 3, 8):  # the caller's buffer at several alignments
        pinned = torch.zeros(len(data) + offset, dtype=torch.uint8).pin_memory()
        pinned[offset:] = torch.frombuffer(bytearray(data), dtype=torch.uint8)
        a = E.Decoder(pinned[offset:])
        b = E.Decoder(data)
        assert same_f64(a.materialize().cpu().numpy(), b.materialize().cpu().numpy())
        p = E.Predicate.range(E.RangeValue.inclusive(-10.0), E.RangeValue.exclusive(600.0))
        ma, sa, mna, mxa, na = a.filter_agg(p)
        mb, sb, mnb, mxb, nb = b.filter_agg(p)
        assert np.array_equal(mask_np(ma), mask_np(mb)) and (sa, mna, mxa, na) == (sb, mnb, mxb, nb)


@pytest.mark.parametrize("scale", [1, 10, 100, 10000])
def test_scales(scale):
    rng = np.random.default_rng(scale)
    v = np.round(rng.normal(50, 20, 20_000) * scale) / scale + 0.0
    data = enc(v, ("record_count", 4096), scale)
    check_query_suite(data, random_preds(v, rng), masks=(None, random_mask(len(v), 0.5, rng)))


@pytest.mark.parametrize("precision", [0, 1, 2, 3])
def test_controlled_precision_materialize(precision):
    rng = np.random.default_rng(precision)
    v = np.round(rng.uniform(-1000, 1000, 30_000), 3) + 0.0
    data = enc(v, ("record_count", 10_000), 1000)
    check_query_suite(data, [], masks=(None, random_mask(len(v), 0.2, rng)), precision=precision)


def test_errors_match_oracle():
    v = np.round(np.random.default_rng(1).uniform(-1, 1, 5000), 3)
    data = bytearray(enc(v, ("record_count", 1000), 1000))
    # wrong field type byte -> ConversionError
    bad = bytearray(data); bad[4] = 1
    with pytest.raises(E.ConversionError):
        E.Decoder(bytes(bad))
    # truncated file -> IO
    with pytest.raises(E.IOError_):
        E.Decoder(bytes(data[:20]))
    # second chunk's header claims more bits than its bytes hold -> UnexpectedEndOfChunk
    d = O.Decoder(bytes(data))
    phys, size, _, _ = d.chunk_info(1)
    bad = bytearray(data); bad[phys + 12] = 40
    g = E.Decoder(bytes(bad))
    with pytest.raises(E.UnexpectedEndOfChunk):
        g.sum()
    with pytest.raises(O.OracleError) as ei:
        O.Decoder(bytes(bad)).sum()
    assert ei.value.code == E.UnexpectedEndOfChunk.code
    # reading only chunk 0 does not touch the bad chunk
    assert g.sum(chunk_id=0) == O.Decoder(bytes(bad)).sum(chunk_id=0)


def test_empty_column():
    data = enc(np.zeros(0), ("record_count", 100), 1000)
    check_query_suite(data, [E.Predicate.eq(1.0)], masks=(None,))


def test_alternating_query_kinds_on_one_column():
    """On a column whose totals are exact for any query, queries without an
    input bitmask leave their totals for the host (two alternating totals
    blocks) and the others fold on the device: any sequence of them gives the
    oracle's results."""
    rng = np.random.default_rng(21)
    v = np.round(rng.uniform(-1000, 1000, 300_000), 3)
    data = enc(v, ("record_count", 65536), 1000)
    d, o = E.Decoder(data), O.Decoder(data)
    n = d.n_records
    mask = random_mask(n, 0.3, rng)
    p = E.Predicate.range(E.RangeValue.inclusive(-100.0), E.RangeValue.exclusive(250.0))
    op = O.rng(O.BOUND_INCLUSIVE, -100.0, O.BOUND_EXCLUSIVE, 250.0)
    for rep in range(3):
        assert d.sum() == o.sum()
        assert d.max(mask) == o.max(mask)
        assert d.min() == o.min()
        assert d.sum(chunk_id=2) == o.sum(chunk_id=2)
        assert same_f64(mask_np(d.filter(p))[: (n + 63) // 64], o.filter(op))
        _, s_, mn_, mx_, cnt_ = d.filter_agg(p, mask, want_mask=True)
        ms, ss, smn, smx = o.filter_agg(op, mask)
        assert (s_, mn_, mx_) == (ss, smn, smx)
        _, s2, mn2, mx2, cnt2 = d.filter_agg(p, want_mask=False)
        _, s3, mn3, mx3 = o.filter_agg(op)
        assert (s2, mn2, mx2) == (s3, mn3, mx3)
        assert d.sum(mask) == o.sum(mask)
