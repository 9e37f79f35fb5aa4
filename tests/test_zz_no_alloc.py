"""ebi_materialize_static (the materialize that allocates nothing) against
ebi_materialize and against the oracle's Decoder::materialize on the same
bytes, through the C ABI, two calls in a row; on a freshly opened column
its calls leave the column's device memory unchanged (no query scratch is
allocated).  Collected last; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest
import torch

import ebi_gb300 as E
from ebi_gb300 import _native
from oracle import oracle as O
from tests.parity import random_mask, same_f64

pytestmark = pytest.mark.gpu

STATIC_TILES = 16384


def static_materialize(d: E.Decoder, mask, chunk_id, cap):
    """(status, values) of ebi_materialize_static through the raw C ABI."""
    lib = _native.lib()
    keep = None
    mp = C.c_void_p(0)
    if mask is not None:
        keep = torch.from_numpy(np.ascontiguousarray(mask, dtype=np.uint64).view(np.int64)).to(d.device)
        mp = C.c_void_p(keep.data_ptr())
    out = torch.full((max(cap, 1),), np.nan, dtype=torch.float64, device=d.device)
    n = C.c_uint64(0)
    rc = lib.ebi_materialize_static(d._h, mp, -1 if chunk_id is None else chunk_id, C.c_void_p(out.data_ptr()),
                                    cap, C.byref(n), d._sp())
    torch.cuda.synchronize()
    return rc, out[: n.value].cpu().numpy()


def columns():
    rng = np.random.default_rng(21)
    n = 150_000
    walk = np.round(30 + np.cumsum(rng.normal(0, 0.5, n)), 2) + 0.0
    steps = np.repeat(np.round(rng.normal(0, 5, n // 40 + 1), 1), 40)[:n] + 0.0
    return [
        ("buff", np.round(rng.uniform(-1000, 1000, n), 3) + 0.0, ("record_count", 65536), 1000),
        ("rle", steps, ("record_count", 8192), 1),
        ("gorilla", walk, ("record_count", 8192), 1),
        ("chimp128", walk, ("record_count", 8192), 1),
        ("uncompressed", walk, ("record_count", 5000), 1),
    ]


@pytest.mark.parametrize("codec,values,chunk,scale", columns(), ids=lambda x: x if isinstance(x, str) else None)
def test_static_matches_materialize_twice(codec, values, chunk, scale):
    data = E.encode(values, codec, chunk, scale)
    d = E.Decoder(data)
    o = O.Decoder(data)
    rng = np.random.default_rng(5)
    n = d.n_records
    masks = (None, random_mask(n, 0.2, rng), O.mask_from_rows([], n))
    # a fresh column: the static calls come first and allocate nothing on the device
    held = d.device_bytes
    for mask in masks:
        for cid in (None, 1):
            want = o.materialize(mask, cid)
            for _ in range(2):  # two calls in a row reuse the same fixed scratch
                rc, got = static_materialize(d, mask, cid, n)
                assert rc == 0, _native.lib().ebi_last_error()
                assert same_f64(got, want), (codec, cid)
    assert d.device_bytes == held
    # the allocating entry point agrees (and its first use does allocate the column's scratch)
    for mask in masks:
        for cid in (None, 1):
            rc, got = static_materialize(d, mask, cid, n)
            assert rc == 0 and same_f64(got, d.materialize(mask, cid).cpu().numpy()), (codec, cid)
    if codec != "buff":
        assert d.device_bytes > held
    d.close()


@pytest.mark.skipif(torch.cuda.device_count() < 2, reason="needs a second GPU")
def test_static_rejects_another_current_device():
    d = E.Decoder(E.encode(np.arange(100.0), "gorilla", ("record_count", 32)), device="cuda:0")
    with torch.cuda.device(1):
        rc, _ = static_materialize(d, None, None, 100)
    assert rc == E.InvalidArgument.code and b"device" in _native.lib().ebi_last_error()
    d.close()


def test_static_rejects_more_tiles_than_its_scratch():
    v = np.arange(STATIC_TILES + 1, dtype=np.float64)
    d = E.Decoder(E.encode(v, "rle", ("record_count", 1)))  # one tile per chunk
    assert d.n_chunks == STATIC_TILES + 1
    rc, _ = static_materialize(d, None, None, len(v))
    assert rc == E.InvalidArgument.code
    assert b"fixed scratch" in _native.lib().ebi_last_error()
    # a query covering one chunk fits
    rc, got = static_materialize(d, None, 7, len(v))
    assert rc == 0 and same_f64(got, np.array([7.0]))
    d.close()


def test_static_reports_a_short_output_buffer():
    v = np.round(np.random.default_rng(2).normal(0, 1, 20_000), 3) + 0.0
    d = E.Decoder(E.encode(v, "gorilla", ("record_count", 8192)))
    lib = _native.lib()
    out = torch.empty(100, dtype=torch.float64, device=d.device)
    n = C.c_uint64(0)
    rc = lib.ebi_materialize_static(d._h, C.c_void_p(0), -1, C.c_void_p(out.data_ptr()), 100, C.byref(n), d._sp())
    assert rc == E.InvalidArgument.code and n.value == len(v)
    d.close()
