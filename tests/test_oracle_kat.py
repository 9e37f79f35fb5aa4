"""Pins the C oracle to the known-answer vectors held by lemolatoon/ebi's own tests (CPU only)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.kat import KAT, CODECS, chunk_option, oracle_pred, round_at


@pytest.mark.parametrize("case", KAT["bit_reads"], ids=lambda c: c["src"])
def test_bit_reader_doctests(case):
    got = O.read_bits(bytes(case["buf"]), case["reads"])
    for g, e, chk in zip(got, case["expect"], case["check"]):
        if chk:
            assert g == e


def test_gorilla_known_prefix():
    k = KAT["gorilla_prefix"]
    stream = O.encode_chunk(k["values"], "gorilla")
    assert list(stream[: len(k["prefix_bytes"])]) == k["prefix_bytes"]
    assert O.decode_chunk(stream, "gorilla").tolist() == k["values"]


def test_buff_precision_table():
    bp = KAT["buff_precision"]
    for scale, prec in bp["scale_to_precision"]:
        assert O.buff_precision(scale) == prec


@pytest.mark.parametrize("codec", CODECS)
@pytest.mark.parametrize("idx", range(len(KAT["filter_cases"])))
def test_filter_cases(codec, idx):
    case = KAT["filter_cases"][idx]
    scale = KAT["filter_buff_scale"] if codec == "buff" else 1
    kind, val = chunk_option(case["chunk"])
    f = O.encode(case["values"], codec, kind, val, scale)
    d = O.Decoder(f)
    n = d.n_records
    mask = O.mask_from_rows(case["bitmask"], n) if "bitmask" in case else None
    pred = oracle_pred(case["pred"])
    got = O.rows_from_mask(d.filter(pred, mask, case.get("chunk_id")), n)
    assert got == case["expect"], case["src"]
    # filter_materialize returns the values of the same rows (query.rs:128-196)
    fm = d.filter_materialize(pred, mask, case.get("chunk_id"))
    want = np.asarray(case["values"])[case["expect"]]
    if codec == "buff":
        np.testing.assert_array_equal(round_at(fm, scale), round_at(want, scale))
    else:
        np.testing.assert_array_equal(fm, want)


@pytest.mark.parametrize("codec", CODECS)
@pytest.mark.parametrize("idx", range(len(KAT["agg_cases"])))
def test_agg_cases(codec, idx):
    case = KAT["agg_cases"][idx]
    scale = KAT["agg_buff_scale"] if codec == "buff" else 1
    kind, val = chunk_option(case["chunk"])
    d = O.Decoder(O.encode(case["values"], codec, kind, val, scale))
    mask = O.mask_from_rows(case["bitmask"], d.n_records) if "bitmask" in case else None
    got = getattr(d, case["op"])(mask)
    if case["op"] == "sum":
        eps = 0.5 * len(case["values"]) if codec == "buff" else 1e-3   # aggregation.rs:72-82
        assert abs(got - case["expect"]) < eps
    else:
        s = scale if codec == "buff" else 1
        assert round_at(got, s) == round_at(case["expect"], s)
