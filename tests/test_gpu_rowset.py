"""Row-id sets (the reference's RoaringBitmap) <-> dense device bitmasks."""
import numpy as np
import pytest

import ebi_gb300 as E
from oracle import oracle as O
from tests.parity import mask_np

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n_records,density", [(1, 1.0), (63, 0.5), (64, 0.3), (100_000, 0.01), (1_000_003, 0.4),
                                               (300_000, 0.0)])
def test_round_trip(n_records, density):
    rng = np.random.default_rng(n_records)
    rows = np.nonzero(rng.random(n_records) < density)[0].astype(np.uint32)
    shuffled = rng.permutation(np.concatenate([rows, rows[: len(rows) // 3]]))  # any order, duplicates
    extra = np.array([n_records, n_records + 5, 2**32 - 1], dtype=np.uint64).astype(np.uint32)  # dropped
    m = E.mask_from_rows(np.concatenate([shuffled, extra]), n_records)
    assert np.array_equal(mask_np(m)[: (n_records + 63) // 64], O.mask_from_rows(rows.tolist(), n_records))
    back = E.rows_from_mask(m, n_records).cpu().numpy().view(np.uint32)
    assert np.array_equal(back, rows)


def test_filter_result_as_rows():
    rng = np.random.default_rng(3)
    v = np.round(rng.uniform(-1000, 1000, 200_000), 3)
    d = E.Decoder(E.encode(v, "buff", ("record_count", 65536), 1000))
    m = d.filter(E.Predicate.range(E.RangeValue.inclusive(-10.0), E.RangeValue.inclusive(10.0)))
    rows = E.rows_from_mask(m, d.n_records).cpu().numpy().view(np.uint32)
    want = O.rows_from_mask(O.Decoder(d_data := E.encode(v, "buff", ("record_count", 65536), 1000)).filter(
        O.rng(O.BOUND_INCLUSIVE, -10.0, O.BOUND_INCLUSIVE, 10.0)), d.n_records)
    assert rows.tolist() == want
