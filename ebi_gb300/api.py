"""Python mirror of ebi's public Decoder / Encoder API over the GB300 engine.

Names, argument meaning and error behaviour follow the reference:
  ebi/src/api/decoder.rs   Decoder::{new, materialize, filter, filter_materialize, sum, min, max,
                           with_precision}, ChunkId
  ebi/src/decoder/query.rs Predicate::{Eq, Ne, Range}, Range, RangeValue::{Inclusive, Exclusive, None}
  ebi/src/decoder/error.rs DecoderError::{IO, ConversionError, UnexpectedEndOfChunk,
                           PreconditionsNotMet, CudaError}
Every call goes through the C ABI of include/ebi_gpu.h; device buffers are torch tensors.
A bitmask is an int64 tensor of ceil(n_records / 64) words (bit r % 64 of word r // 64 = row r).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _native

UNCOMPRESSED, RLE, BUFF, GORILLA, CHIMP, CHIMP128, ELF_ON_CHIMP, ELF = range(8)
SCHEMES = {"uncompressed": UNCOMPRESSED, "rle": RLE, "buff": BUFF, "gorilla": GORILLA,
           "chimp": CHIMP, "chimp128": CHIMP128, "elf_on_chimp": ELF_ON_CHIMP, "elf": ELF}
CHUNK_KINDS = {"full": 0, "record_count": 1, "byte_size": 2}


# ---- errors (decoder/error.rs) -----------------------------------------------------------
class DecoderError(RuntimeError):
    code = -1

    def __init__(self, msg: str, code: Optional[int] = None):
        super().__init__(msg)
        if code is not None:
            self.code = code


class IOError_(DecoderError): code = 1
class ConversionError(DecoderError): code = 2
class UnexpectedEndOfChunk(DecoderError): code = 3
class PreconditionsNotMet(DecoderError): code = 4
class CudaError(DecoderError): code = 5
class CorruptChunk(DecoderError): code = 6
class InvalidArgument(DecoderError): code = 7
class OutOfMemory(DecoderError): code = 8
class Unsupported(DecoderError): code = 9


_ERRORS = {c.code: c for c in (IOError_, ConversionError, UnexpectedEndOfChunk, PreconditionsNotMet, CudaError,
                               CorruptChunk, InvalidArgument, OutOfMemory, Unsupported)}


def _check(code: int, what: str):
    if code != 0:
        msg = _native.lib().ebi_last_error().decode(errors="replace")
        raise _ERRORS.get(code, DecoderError)(f"{what}: {msg}", code)


# ---- predicates (decoder/query.rs:352-446) --------------------------------------------------
@dataclass(frozen=True)
class RangeValue:
    kind: int  # 0 None, 1 Inclusive, 2 Exclusive
    value: float = 0.0

    @staticmethod
    def inclusive(v: float) -> "RangeValue": return RangeValue(1, float(v))
    @staticmethod
    def exclusive(v: float) -> "RangeValue": return RangeValue(2, float(v))

    def eval_start(self, x):
        return x >= self.value if self.kind == 1 else x > self.value if self.kind == 2 else True

    def eval_end(self, x):
        return x <= self.value if self.kind == 1 else x < self.value if self.kind == 2 else True


RangeValue.NONE = RangeValue(0, 0.0)


@dataclass(frozen=True)
class Range:
    start: RangeValue
    end: RangeValue

    def eval(self, x) -> bool:  # RangeImpl::eval (query.rs:396-409)
        return self.start.eval_start(x) and self.end.eval_end(x)


@dataclass(frozen=True)
class Predicate:
    kind: int                 # 0 Eq, 1 Ne, 2 Range
    value: float = 0.0
    rng: Optional[Range] = None

    @staticmethod
    def eq(v: float) -> "Predicate": return Predicate(0, float(v))
    @staticmethod
    def ne(v: float) -> "Predicate": return Predicate(1, float(v))

    @staticmethod
    def range_(start: RangeValue, end: RangeValue) -> "Predicate":
        return Predicate(2, 0.0, Range(start, end))

    def eval(self, x) -> bool:  # PredicateImpl::eval (query.rs:431-437)
        if self.kind == 0:
            return x == self.value
        if self.kind == 1:
            return x != self.value
        return self.rng.eval(x)

    def to_c(self) -> _native.Predicate:
        if self.kind == 2:
            r = self.rng
            return _native.Predicate(2, r.start.kind, r.end.kind, 0, 0.0, r.start.value, r.end.value)
        return _native.Predicate(self.kind, 0, 0, 0, self.value, 0.0, 0.0)


# Predicate.range(start, end) reads like the reference's Predicate::Range(Range::new(start, end)).
Predicate.range = staticmethod(Predicate.range_)


@dataclass(frozen=True)
class ChunkId:
    index: int


def _cid(chunk_id) -> int:
    if chunk_id is None:
        return -1
    return int(chunk_id.index if isinstance(chunk_id, ChunkId) else chunk_id)


# ---- encoder (api/encoder.rs) ------------------------------------------------------------------
def encode(values, scheme, chunk_option=("record_count", 8192), scale: int = 1) -> bytes:
    """Encoder::new(input, output, chunk_option, config).encode(); returns the EBI1 bytes."""
    v = np.ascontiguousarray(values, dtype=np.float64)
    kind, val = chunk_option if isinstance(chunk_option, tuple) else (chunk_option, 0)
    out = C.POINTER(C.c_uint8)()
    n = C.c_uint64()
    L = _native.lib()
    sch = SCHEMES[scheme] if isinstance(scheme, str) else int(scheme)
    _check(L.ebi_encode(v.ctypes.data_as(C.POINTER(C.c_double)), len(v), sch, CHUNK_KINDS[kind], int(val),
                        int(scale), C.byref(out), C.byref(n)), "Encoder::encode")
    try:
        return C.string_at(out, n.value)
    finally:
        L.ebi_free(out)


# ---- decoder (api/decoder.rs) --------------------------------------------------------------------
def _torch():
    import torch
    return torch


class Decoder:
    """Decoder::new over an in-memory EBI1 file (bytes, or a host uint8 tensor;
    Decoder.from_file reads a path); the column stays resident on the GPU."""

    def __init__(self, data, device: str = "cuda:0", stream=None, _path=None):
        torch = _torch()
        self.device = torch.device(device)
        self._stream = stream
        L = _native.lib()
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            if _path is not None:  # Decoder::new(DecoderInput::from_file(path))
                _check(L.ebi_column_open_file(os.fsencode(_path), self._sp(), C.byref(h)), "Decoder::new")
                self._h = h
                return
            if isinstance(data, torch.Tensor):  # host uint8 tensor (pinned for async copies)
                assert data.dtype == torch.uint8 and not data.is_cuda
                ptr, n = C.cast(data.data_ptr(), C.c_char_p), data.numel()
                self._keep = data
            else:
                buf = bytes(data)
                ptr, n = buf, len(buf)
            _check(L.ebi_column_open(ptr, n, self._sp(), C.byref(h)), "Decoder::new")
        self._h = h

    @classmethod
    def from_file(cls, path, device: str = "cuda:0", stream=None):
        """Decoder::new(DecoderInput::from_file(path)): the file is read into
        pinned host memory and moved to HBM (BUFF planes in one device pass)."""
        return cls(None, device=device, stream=stream, _path=path)

    def _sp(self):
        torch = _torch()
        s = self._stream if self._stream is not None else torch.cuda.current_stream(self.device)
        return C.c_void_p(s.cuda_stream)

    def close(self):
        if getattr(self, "_h", None):
            _native.lib().ebi_column_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- metadata --
    @property
    def n_records(self) -> int: return _native.lib().ebi_column_num_records(self._h)
    @property
    def n_chunks(self) -> int: return _native.lib().ebi_column_num_chunks(self._h)
    @property
    def scheme(self) -> int: return _native.lib().ebi_column_scheme(self._h)
    def set_copy_wait(self, cycles=None):
        """Limit (SM clocks) of the column's kernels' waits for their bulk copies; None: the default.
        A query whose copy has not landed by then raises CudaError; the column stays usable."""
        _check(_native.lib().ebi_column_set_copy_wait(self._h, -1 if cycles is None else int(cycles)),
               "Decoder::set_copy_wait")

    @property
    def device_bytes(self) -> int:
        """Device memory the column holds (resident file, tables, query scratch once allocated)."""
        return _native.lib().ebi_column_device_bytes(self._h)
    @property
    def mask_words(self) -> int: return max((self.n_records + 63) // 64, 1)

    def chunk_info(self, i):
        a, b, c, d = (C.c_uint64() for _ in range(4))
        _check(_native.lib().ebi_column_chunk_info(self._h, i, C.byref(a), C.byref(b), C.byref(c), C.byref(d)),
               "chunk_info")
        return a.value, b.value, c.value, d.value

    def set_timing(self, enable: bool = True):
        _check(_native.lib().ebi_column_set_timing(self._h, int(enable)), "set_timing")

    def segmented_execution_times(self) -> dict:
        """Device time of the last query by segment (Decoder::segmented_execution_times)."""
        t = _native.SegmentTimes()
        _check(_native.lib().ebi_column_last_times(self._h, C.byref(t)), "segmented_execution_times")
        return {"scan_ms": t.scan_ms, "finalize_ms": t.finalize_ms, "total_ms": t.total_ms, "kernels": t.kernels}

    def with_precision(self, precision: int):
        _check(_native.lib().ebi_column_set_precision(self._h, int(precision)), "Decoder::with_precision")

    # -- buffers --
    def _mask_in(self, bitmask):
        if bitmask is None:
            return None, None
        torch = _torch()
        if isinstance(bitmask, torch.Tensor):
            t = bitmask.to(self.device, dtype=torch.int64).contiguous()
        else:
            t = torch.from_numpy(np.ascontiguousarray(bitmask, dtype=np.uint64).view(np.int64)).to(self.device)
        assert t.numel() >= self.mask_words, "bitmask shorter than ceil(n_records / 64) words"
        return C.c_void_p(t.data_ptr()), t

    def new_mask(self):
        torch = _torch()
        return torch.empty(self.mask_words, dtype=torch.int64, device=self.device)

    # -- queries --
    def materialize(self, bitmask=None, chunk_id=None, out=None):
        torch = _torch()
        mp, keep = self._mask_in(bitmask)
        call = lambda o, n: _native.lib().ebi_materialize(self._h, mp, _cid(chunk_id), C.c_void_p(o.data_ptr()),
                                                          o.numel(), C.byref(n), self._sp())
        return self._materialize(call, out, "Decoder::materialize")

    def _materialize(self, call, out, what):
        torch = _torch()
        grow = out is None
        if out is None:
            out = torch.empty(max(self.n_records, 1), dtype=torch.float64, device=self.device)
        n = C.c_uint64()
        rc = call(out, n)
        if rc == InvalidArgument.code and grow and n.value > out.numel():
            # the chunks decode to more values than the footer counts: retry at the size reported
            out = torch.empty(n.value, dtype=torch.float64, device=self.device)
            rc = call(out, n)
        _check(rc, what)
        return out[: n.value]

    def filter(self, predicate: Predicate, bitmask=None, chunk_id=None, out=None):
        mp, keep = self._mask_in(bitmask)
        out = self.new_mask() if out is None else out
        p = predicate.to_c()
        _check(_native.lib().ebi_filter(self._h, C.byref(p), mp, _cid(chunk_id), C.c_void_p(out.data_ptr()),
                                        self._sp()), "Decoder::filter")
        return out

    def filter_materialize(self, predicate: Predicate, bitmask=None, chunk_id=None, out=None):
        torch = _torch()
        mp, keep = self._mask_in(bitmask)
        p = predicate.to_c()
        call = lambda o, n: _native.lib().ebi_filter_materialize(self._h, C.byref(p), mp, _cid(chunk_id),
                                                                 C.c_void_p(o.data_ptr()), o.numel(), C.byref(n),
                                                                 self._sp())
        return self._materialize(call, out, "Decoder::filter_materialize")

    def _agg(self, fn, bitmask, chunk_id, what):
        mp, keep = self._mask_in(bitmask)
        r = C.c_double()
        _check(fn(self._h, mp, _cid(chunk_id), C.byref(r), self._sp()), what)
        return r.value

    def sum(self, bitmask=None, chunk_id=None) -> float:
        return self._agg(_native.lib().ebi_sum, bitmask, chunk_id, "Decoder::sum")

    def min(self, bitmask=None, chunk_id=None) -> float:
        return self._agg(_native.lib().ebi_min, bitmask, chunk_id, "Decoder::min")

    def max(self, bitmask=None, chunk_id=None) -> float:
        return self._agg(_native.lib().ebi_max, bitmask, chunk_id, "Decoder::max")

    def filter_agg(self, predicate: Predicate, bitmask=None, chunk_id=None, out=None, want_mask=True,
                   aggregates=("sum", "min", "max")):
        """Decoder::filter then Decoder::{sum, min, max} over its result, one pass.

        Only the aggregates named in `aggregates` are computed; the others come back as None."""
        mp, keep = self._mask_in(bitmask)
        if want_mask and out is None:
            out = self.new_mask()
        p = predicate.to_c()
        s, a, b, n = C.c_double(), C.c_double(), C.c_double(), C.c_uint64()
        ref = lambda x, name: C.byref(x) if name in aggregates else None
        _check(_native.lib().ebi_filter_agg(self._h, C.byref(p), mp, _cid(chunk_id),
                                            C.c_void_p(out.data_ptr()) if want_mask else None,
                                            ref(s, "sum"), ref(a, "min"), ref(b, "max"), C.byref(n), self._sp()),
               "Decoder::filter_agg")
        val = lambda x, name: x.value if name in aggregates else None
        return out, val(s, "sum"), val(a, "min"), val(b, "max"), n.value


# ---- multi-column aggregation (api/decoder.rs:755-917, decoder/expr.rs) ----------
class Op:
    """Op (decoder/expr.rs:11-29): one IEEE f64 operation."""
    Add, Sub, Mul, Div = 2, 3, 4, 5


class Expr:
    """Expr (decoder/expr.rs:31-40): Expr.Index(i) is the decoders[i] column,
    Expr.Literal(x) a constant, Expr.Binary(op, lhs, rhs) lhs OP rhs.  The
    arithmetic operators build Binary nodes: (Expr.Index(0) * (1.0 - Expr.Index(1)))."""

    __slots__ = ("kind", "index", "value", "op", "lhs", "rhs")

    def __init__(self, kind, index=0, value=0.0, op=None, lhs=None, rhs=None):
        self.kind, self.index, self.value, self.op, self.lhs, self.rhs = kind, index, value, op, lhs, rhs

    @staticmethod
    def Index(i: int) -> "Expr": return Expr("index", index=int(i))
    @staticmethod
    def Literal(x: float) -> "Expr": return Expr("literal", value=float(x))
    @staticmethod
    def Binary(op: int, lhs: "Expr", rhs: "Expr") -> "Expr": return Expr("binary", op=int(op), lhs=lhs, rhs=rhs)

    @staticmethod
    def _wrap(x) -> "Expr": return x if isinstance(x, Expr) else Expr.Literal(x)
    def __add__(self, o): return Expr.Binary(Op.Add, self, Expr._wrap(o))
    def __radd__(self, o): return Expr.Binary(Op.Add, Expr._wrap(o), self)
    def __sub__(self, o): return Expr.Binary(Op.Sub, self, Expr._wrap(o))
    def __rsub__(self, o): return Expr.Binary(Op.Sub, Expr._wrap(o), self)
    def __mul__(self, o): return Expr.Binary(Op.Mul, self, Expr._wrap(o))
    def __rmul__(self, o): return Expr.Binary(Op.Mul, Expr._wrap(o), self)
    def __truediv__(self, o): return Expr.Binary(Op.Div, self, Expr._wrap(o))
    def __rtruediv__(self, o): return Expr.Binary(Op.Div, Expr._wrap(o), self)

    def max_chunk_reader_index(self):
        """Expr::max_chunk_reader_index (expr.rs:43-58)."""
        if self.kind == "literal":
            return None
        if self.kind == "index":
            return self.index
        ids = [i for i in (self.lhs.max_chunk_reader_index(), self.rhs.max_chunk_reader_index()) if i is not None]
        return max(ids) if ids else None

    def postfix(self):
        """[(EBI_EXPR_* kind, index, literal), ...] in postfix order."""
        if self.kind == "index":
            return [(0, self.index, 0.0)]
        if self.kind == "literal":
            return [(1, 0, self.value)]
        return self.lhs.postfix() + self.rhs.postfix() + [(self.op, 0, 0.0)]

    def __repr__(self):
        if self.kind == "index":
            return f"Index({self.index})"
        if self.kind == "literal":
            return f"Literal({self.value!r})"
        return f"({self.lhs!r} {'+-*/'[self.op - 2]} {self.rhs!r})"


class AggregationKind:
    """AggregationKind (api/decoder.rs:755-761)."""
    NONE, MAX, MIN, SUM = 0, 1, 2, 3


class Aggregation:
    """Aggregation { kind, expr } (api/decoder.rs:840-917) over resident
    columns: compute() returns a float (Max / Min / Sum) or, for
    AggregationKind.NONE, the device tensor of the values (the reference's
    AggregationResult::Array)."""

    def __init__(self, kind: int, expr: Expr):
        self.kind, self.expr = int(kind), expr

    @classmethod
    def new(cls, kind, expr): return cls(kind, expr)
    @classmethod
    def sum(cls, expr): return cls(AggregationKind.SUM, expr)
    @classmethod
    def min(cls, expr): return cls(AggregationKind.MIN, expr)
    @classmethod
    def max(cls, expr): return cls(AggregationKind.MAX, expr)
    @classmethod
    def none(cls, expr): return cls(AggregationKind.NONE, expr)

    def compute(self, decoders, bitmask=None):
        """Aggregation::compute (api/decoder.rs:858-879)."""
        return Aggregation.compute_multiple([self], decoders, bitmask)[0]

    @staticmethod
    def compute_multiple(aggregations, decoders, bitmask=None):
        """Aggregation::compute_multiple (api/decoder.rs:881-916)."""
        torch = _torch()
        if not decoders:
            raise InvalidArgument("Aggregation::compute: no decoders", InvalidArgument.code)
        d0 = decoders[0]
        hs = (C.c_void_p * len(decoders))(*[d._h for d in decoders])
        mask_ptr, keep = None, None
        if bitmask is not None:
            words = max(max(d.mask_words for d in decoders), 1)
            if isinstance(bitmask, torch.Tensor):
                keep = bitmask.to(d0.device, dtype=torch.int64).contiguous()
            else:
                keep = torch.from_numpy(np.ascontiguousarray(bitmask, dtype=np.uint64).view(np.int64)).to(d0.device)
            if keep.numel() < words:
                keep = torch.cat([keep, keep.new_zeros(words - keep.numel())])
            mask_ptr = C.c_void_p(keep.data_ptr())
        n = len(aggregations)
        arr = (_native.Aggregation * max(n, 1))()
        node_bufs, outs = [], []
        for i, g in enumerate(aggregations):
            pf = g.expr.postfix()
            nodes = (_native.ExprNode * len(pf))(*[_native.ExprNode(k, ix, float(x)) for k, ix, x in pf])
            node_bufs.append(nodes)
            arr[i].kind = g.kind
            arr[i].n_nodes = len(pf)
            arr[i].nodes = nodes
            out = None
            if g.kind == AggregationKind.NONE:
                cap = max(d.n_records for d in decoders)
                out = torch.empty(max(cap, 1), dtype=torch.float64, device=d0.device)
                arr[i].d_array = C.c_void_p(out.data_ptr())
                arr[i].array_cap = cap
            outs.append(out)
        with torch.cuda.device(d0.device):
            rc = _native.lib().ebi_aggregate(hs, len(decoders), arr, n, mask_ptr, d0._sp())
            if rc == InvalidArgument.code and any(
                    g.kind == AggregationKind.NONE and arr[i].n_array > arr[i].array_cap
                    for i, g in enumerate(aggregations)):
                for i, g in enumerate(aggregations):  # decoded chunks held more values than their row counts
                    if g.kind == AggregationKind.NONE:
                        outs[i] = torch.empty(max(arr[i].n_array, 1), dtype=torch.float64, device=d0.device)
                        arr[i].d_array = C.c_void_p(outs[i].data_ptr())
                        arr[i].array_cap = arr[i].n_array
                rc = _native.lib().ebi_aggregate(hs, len(decoders), arr, n, mask_ptr, d0._sp())
            _check(rc, "Aggregation::compute_multiple")
        return [outs[i][: arr[i].n_array] if g.kind == AggregationKind.NONE else arr[i].scalar
                for i, g in enumerate(aggregations)]


_AGG_BITS = {"sum": 1, "min": 2, "max": 4}


class Batch:
    """A fixed list of filter + aggregate queries over open Decoders (columns may
    repeat and mix codecs), run as one persistent mixed-codec launch captured in
    a CUDA graph (ebi_batch_* of the C ABI; no counterpart in the reference).

    queries: sequence of (decoder, predicate) or (decoder, predicate, aggregates)."""

    def __init__(self, queries, stream=None, want_masks=False):
        torch = _torch()
        if not queries:
            raise InvalidArgument("a batch needs at least one query")
        self.decoders = [q[0] for q in queries]
        self.device = self.decoders[0].device
        self._stream = stream
        n = len(queries)
        arr = (_native.BatchQuery * n)()
        self.masks = []
        for i, q in enumerate(queries):
            d, p = q[0], q[1]
            aggs = q[2] if len(q) > 2 else ("sum", "min", "max")
            m = d.new_mask() if want_masks else None
            self.masks.append(m)
            arr[i].col = d._h
            arr[i].pred = p.to_c()
            arr[i].aggregates = sum(_AGG_BITS[a] for a in aggs)
            arr[i].d_out_mask = m.data_ptr() if m is not None else None
        self._aggs = [q[2] if len(q) > 2 else ("sum", "min", "max") for q in queries]
        h = C.c_void_p()
        _check(_native.lib().ebi_batch_create(arr, n, self._sp(), C.byref(h)), "Batch::new")
        self._h = h
        self._n = n
        self._res = (_native.BatchResult * n)()

    def _sp(self):
        torch = _torch()
        s = self._stream if self._stream is not None else torch.cuda.current_stream(self.device)
        return C.c_void_p(s.cuda_stream)

    def run(self, predicates=None):
        """Runs every query; returns [(sum, min, max, count)] (None for aggregates not asked for)."""
        preds = None
        if predicates is not None:
            assert len(predicates) == self._n
            preds = (_native.Predicate * self._n)(*[p.to_c() for p in predicates])
        rc = _native.lib().ebi_batch_run(self._h, preds, self._res, self._sp())
        out = []
        for i in range(self._n):
            r = self._res[i]
            a = self._aggs[i]
            out.append((r.sum if "sum" in a else None, r.min if "min" in a else None,
                        r.max if "max" in a else None, r.count))
        _check(rc, "Batch::run")
        return out

    def statuses(self):
        return [self._res[i].status for i in range(self._n)]

    def info(self) -> dict:
        """The launch chosen by the first run: shape, tiling per column-size bucket
        (< 262,144 rows, < 4,194,304, larger) and the timed candidates."""
        inf = _native.BatchInfo()
        _check(_native.lib().ebi_batch_get_info(self._h, C.byref(inf)), "Batch::info")
        return {"queries": inf.queries, "items": inf.items, "chunks": inf.chunks, "shape": inf.shape,
                "ctas_per_sm": inf.ctas_per_sm, "order": ["cost", "query"][inf.order] if inf.shape >= 0 else None,
                "shape_ms": list(inf.shape_ms), "buff_tiles": list(inf.buff_tiles),
                "value_chunks": list(inf.value_chunks), "gorilla_chunks": list(inf.gorilla_chunks),
                "trials": self.trials(), "from_cache": bool(inf.from_cache), "best_ms": inf.best_ms}

    _KNOBS = ("shape", "buff_tiles", "value_chunks", "gorilla_chunks")

    def trials(self) -> list:
        """The first run's timed candidates, in the order timed."""
        buf = (_native.BatchTrial * 256)()
        n = C.c_uint32()
        _check(_native.lib().ebi_batch_get_trials(self._h, buf, 256, C.byref(n)), "Batch::trials")
        out = []
        for t in buf[: n.value]:
            if t.knob == 0:
                what = {"ctas_per_sm": t.value // 2, "order": ["cost", "query"][t.value % 2]}
            else:
                what = {"bucket": t.bucket, "value": t.value}
            out.append(dict(knob=self._KNOBS[t.knob], ms=round(t.ms, 4), kept=bool(t.kept), **what))
        return out

    @staticmethod
    def set_tuning_cache(path):
        """Process-wide JSON tuning cache (None turns it off): batches of a column
        shape found there skip the first run's timing."""
        _check(_native.lib().ebi_batch_set_tuning_cache(None if path is None else str(path).encode()),
               "Batch::set_tuning_cache")

    def close(self):
        if getattr(self, "_h", None):
            _native.lib().ebi_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _requests(reqs):
    """[(column ids, predicate, aggregates)] -> ebi_request array."""
    arr = (_native.Request * len(reqs))()
    for i, (cols, p, aggs) in enumerate(reqs):
        if not 1 <= len(cols) <= 8:
            raise InvalidArgument("a request reads 1..8 columns")
        arr[i].n_columns = len(cols)
        for k, c in enumerate(cols):
            arr[i].columns[k] = int(c)
        arr[i].pred = p.to_c()
        arr[i].aggregates = sum(_AGG_BITS[a] for a in aggs)
    return arr


def _responses(arr):
    return [{"sum": r.sum, "min": r.min, "max": r.max, "count": r.count, "status": r.status,
             "submit_ns": r.submit_ns, "launch_ns": r.launch_ns, "done_ns": r.done_ns} for r in arr]


class Server:
    """Continuous-batching request loop over resident columns (ebi_server_* of
    the C ABI; no counterpart in the reference).  Requests are
    (column ids, predicate, aggregates) over 1..8 of the server's decoders."""

    def __init__(self, decoders, slots=4, max_queries=1024, max_chunks=1 << 20, max_items=1 << 21, device=None,
                 buff_tiles=0, value_chunks=0, gorilla_chunks=0):
        """buff_tiles / value_chunks / gorilla_chunks: work-item tiling (BUFF tiles, RLE / Uncompressed
        chunks, Gorilla chunks per item; 0 keeps the default: 8, 8, 16)."""
        self.decoders = list(decoders)
        dev = self.decoders[0].device if device is None else _torch().device(device)
        cfg = _native.ServerConfig(dev.index or 0, slots, max_queries, max_chunks, max_items, buff_tiles,
                                   value_chunks, gorilla_chunks, 0)
        cols = (C.c_void_p * len(self.decoders))(*[d._h.value for d in self.decoders])
        h = C.c_void_p()
        _check(_native.lib().ebi_server_create(cols, len(self.decoders), C.byref(cfg), C.byref(h)), "Server::new")
        self._h = h

    def submit(self, cols, predicate, aggregates=("sum", "min", "max")) -> int:
        arr = _requests([(cols, predicate, aggregates)])
        t = C.c_uint64()
        _check(_native.lib().ebi_server_submit(self._h, arr, C.byref(t)), "Server::submit")
        return t.value

    def poll(self, max_n=1024):
        buf = (_native.Response * max_n)()
        n = C.c_uint32()
        _check(_native.lib().ebi_server_poll(self._h, buf, max_n, C.byref(n)), "Server::poll")
        return [dict(ticket=buf[i].ticket, **_responses([buf[i]])[0]) for i in range(n.value)]

    def replay(self, requests, arrival_ns=None):
        """Open-loop load (native): request i is submitted arrival_ns[i] after the start."""
        arr = _requests(requests)
        out = (_native.Response * len(requests))()
        arrivals = None
        if arrival_ns is not None:
            arrivals = (C.c_uint64 * len(requests))(*[int(t) for t in arrival_ns])
        _check(_native.lib().ebi_server_replay(self._h, arr, arrivals, len(requests), out), "Server::replay")
        return _responses(out)

    def stats(self) -> dict:
        st = _native.ServerStats()
        _check(_native.lib().ebi_server_get_stats(self._h, C.byref(st)), "Server::stats")
        return {"batches": st.batches, "requests": st.requests, "max_in_flight": st.max_in_flight,
                "pending": st.pending, "items": st.items, "build_ms": round(st.build_ns / 1e6, 3)}

    def close(self):
        if getattr(self, "_h", None):
            _native.lib().ebi_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_plain(decoders, requests, stream=None):
    """The requests answered one at a time with per-column filter_agg calls (no batching)."""
    torch = _torch()
    cols = (C.c_void_p * len(decoders))(*[d._h.value for d in decoders])
    arr = _requests(requests)
    out = (_native.Response * len(requests))()
    s = stream if stream is not None else torch.cuda.current_stream(decoders[0].device)
    _check(_native.lib().ebi_run_plain(cols, len(decoders), arr, len(requests), out, C.c_void_p(s.cuda_stream)),
           "run_plain")
    return _responses(out)


def mask_from_rows(rows, n_records: int, device="cuda:0"):
    """Dense device bitmask of a u32 row-id set (RoaringBitmap::iter order or any order)."""
    torch = _torch()
    dev = torch.device(device)
    r = torch.as_tensor(np.ascontiguousarray(rows, dtype=np.uint32).view(np.int32), device=dev)
    m = torch.empty(max((n_records + 63) // 64, 1), dtype=torch.int64, device=dev)
    s = torch.cuda.current_stream(dev)
    _check(_native.lib().ebi_mask_from_rows(C.c_void_p(r.data_ptr()), r.numel(), n_records, C.c_void_p(m.data_ptr()),
                                            C.c_void_p(s.cuda_stream)), "mask_from_rows")
    return m


def rows_from_mask(mask, n_records: int):
    """Ascending u32 row ids of a device bitmask (as RoaringBitmap::iter yields them)."""
    torch = _torch()
    dev = mask.device
    s = torch.cuda.current_stream(dev)
    n = C.c_uint64()
    cap = 1 << 16
    while True:
        out = torch.empty(cap, dtype=torch.int32, device=dev)
        rc = _native.lib().ebi_rows_from_mask(C.c_void_p(mask.data_ptr()), n_records, C.c_void_p(out.data_ptr()), cap,
                                               C.byref(n), C.c_void_p(s.cuda_stream))
        if rc == InvalidArgument.code and n.value > cap:
            cap = n.value
            continue
        _check(rc, "rows_from_mask")
        return out[: n.value]


def kernel_launches() -> int:
    return _native.lib().ebi_kernel_launches()
