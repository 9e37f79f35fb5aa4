"""A bounded wait that runs out, on the GPU, without hanging or faulting it.

The kernels that stage data with bulk copies (the pipelined BUFF scan, used
for chunks wider than 32 bits, and the Gorilla chunk pass) wait for their
copies on mbarriers with a limit (ebi_column_set_copy_wait).  With the limit
at zero each of those waits is a single look, which comes before the copy has
landed: the query must fail with CudaError (EBI_E_CUDA, the reference's error
kinds are in decoder/error.rs:6-21), the kernel must still wait out its copies
in flight before it exits, and the same column must then answer queries
exactly as the oracle does.  The failure is made on the host (a limit), not by
a fault: nothing here traps, faults or hangs the GPU."""
import numpy as np
import pytest

import ebi_gb300 as E
from oracle import oracle as O
from tests.parity import mask_np, same_scalar, sum_ok

pytestmark = pytest.mark.gpu


def column(kind):
    rng = np.random.default_rng(41)
    if kind == "buff_wide":
        # 6 decimals at scale 10^6: 21 fraction bits and a 2e6 range, about 42-bit chunks
        v = np.round(rng.uniform(-1e6, 1e6, 200_000), 6) + 0.0
        data = E.encode(v, "buff", ("record_count", 65536), 1_000_000)
        a, b = -2e5, 3e5
    else:
        v = np.round(30 + np.cumsum(rng.normal(0, 0.5, 100_000)), 2) + 0.0
        data = E.encode(v, "gorilla", ("record_count", 8192))
        a, b = 10.0, 50.0
    pred = E.Predicate.range(E.RangeValue.inclusive(a), E.RangeValue.inclusive(b))
    return data, pred, O.rng(O.BOUND_INCLUSIVE, a, O.BOUND_INCLUSIVE, b)


@pytest.mark.parametrize("kind", ["buff_wide", "gorilla"])
def test_copy_wait_runs_out_then_the_column_answers(kind):
    data, pred, opred = column(kind)
    d = E.Decoder(data)
    o = O.Decoder(data)
    om, os_, omn, omx = o.filter_agg(opred)
    sel = o.filter_materialize(opred)
    exact = kind == "buff_wide"
    for _ in range(2):
        d.set_copy_wait(0)
        with pytest.raises(E.CudaError):
            d.filter_agg(pred)
        d.set_copy_wait(None)
        m, s, mn, mx, n = d.filter_agg(pred)
        assert np.array_equal(mask_np(m)[: len(om)], om)
        assert n == len(sel)
        assert sum_ok(s, os_, exact, sel)
        assert same_scalar(mn, omn) and same_scalar(mx, omx)
        assert sum_ok(d.sum(), o.sum(), exact, o.materialize())
    d.close()
