"""ctypes binding of the C oracle (oracle/ebi_oracle.c).

TEST INFRASTRUCTURE ONLY: the CPU restatement of lemolatoon/ebi's decode-and-query
path that checks the GPU engine and serves as bench.py's CPU baseline.  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module; the product never does.

Bitmasks are numpy uint64 arrays of ceil(n_records / 64) little-endian words
(bit r % 64 of word r // 64 is row r).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
LIB_PATH = BUILD_DIR / "libebi_oracle.so"
SOURCES = [HERE / "ebi_oracle.c"]

UNCOMPRESSED, RLE, BUFF, GORILLA, CHIMP, CHIMP128, ELF_ON_CHIMP, ELF = range(8)
SCHEMES = {"uncompressed": UNCOMPRESSED, "rle": RLE, "buff": BUFF, "gorilla": GORILLA,
           "chimp": CHIMP, "chimp128": CHIMP128, "elf_on_chimp": ELF_ON_CHIMP, "elf": ELF}
CHUNK_FULL, CHUNK_RECORD_COUNT, CHUNK_BYTE_SIZE = range(3)
PRED_EQ, PRED_NE, PRED_RANGE = range(3)
BOUND_NONE, BOUND_INCLUSIVE, BOUND_EXCLUSIVE = range(3)

STATUS = {0: "OK", 1: "IO", 2: "ConversionError", 3: "UnexpectedEndOfChunk",
          4: "PreconditionsNotMet", 6: "Corrupt", 7: "Invalid", 8: "OutOfMemory"}


class OracleError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what}: {STATUS.get(code, code)}")
        self.code = code


class Pred(C.Structure):
    _fields_ = [("kind", C.c_int32), ("start_kind", C.c_int32), ("end_kind", C.c_int32),
                ("reserved", C.c_int32), ("value", C.c_double), ("start", C.c_double),
                ("end", C.c_double)]


def eq(v): return Pred(PRED_EQ, 0, 0, 0, float(v), 0.0, 0.0)
def ne(v): return Pred(PRED_NE, 0, 0, 0, float(v), 0.0, 0.0)


class ExprNode(C.Structure):
    """ora_expr_node: one postfix node of an Expr (kind EXPR_*, column index, literal)."""
    _fields_ = [("kind", C.c_int32), ("index", C.c_uint32), ("literal", C.c_double)]


EXPR_INDEX, EXPR_LITERAL, EXPR_ADD, EXPR_SUB, EXPR_MUL, EXPR_DIV = range(6)
AGGR_NONE, AGGR_MAX, AGGR_MIN, AGGR_SUM = range(4)


def rng(start_kind=BOUND_NONE, start=0.0, end_kind=BOUND_NONE, end=0.0):
    return Pred(PRED_RANGE, start_kind, end_kind, 0, 0.0, float(start), float(end))


def build(force: bool = False) -> Path:
    """Compiles the oracle with gcc into oracle/_build (a C file, no reference build)."""
    BUILD_DIR.mkdir(exist_ok=True)
    newest = max(p.stat().st_mtime for p in SOURCES + [HERE / "ebi_oracle.h"])
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < newest:
        tmp = LIB_PATH.with_suffix(f".{os.getpid()}.tmp")
        subprocess.run(["gcc", "-O3", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(tmp),
                        *map(str, SOURCES), "-lpthread", "-lm"], check=True)
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(str(build()))
        u64p = C.POINTER(C.c_uint64)
        dp = C.POINTER(C.c_double)
        L.ora_encode.argtypes = [dp, C.c_uint64, C.c_int, C.c_int, C.c_uint64, C.c_uint64,
                                 C.POINTER(C.POINTER(C.c_uint8)), u64p]
        L.ora_encode_chunk.argtypes = [dp, C.c_uint64, C.c_int, C.c_uint64,
                                       C.POINTER(C.POINTER(C.c_uint8)), u64p]
        L.ora_free.argtypes = [C.c_void_p]
        L.ora_open.argtypes = [C.c_char_p, C.c_uint64, C.POINTER(C.c_void_p)]
        L.ora_close.argtypes = [C.c_void_p]
        L.ora_num_records.argtypes = [C.c_void_p]
        L.ora_num_records.restype = C.c_uint64
        L.ora_num_chunks.argtypes = [C.c_void_p]
        L.ora_num_chunks.restype = C.c_uint64
        L.ora_scheme.argtypes = [C.c_void_p]
        L.ora_chunk_info.argtypes = [C.c_void_p, C.c_uint64, u64p, u64p, u64p, u64p]
        L.ora_set_precision.argtypes = [C.c_void_p, C.c_int32]
        L.ora_materialize.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, dp, C.c_uint64, u64p, C.c_int]
        L.ora_filter.argtypes = [C.c_void_p, C.POINTER(Pred), C.c_void_p, C.c_int64, C.c_void_p, C.c_int]
        L.ora_filter_materialize.argtypes = [C.c_void_p, C.POINTER(Pred), C.c_void_p, C.c_int64, dp,
                                             C.c_uint64, u64p, C.c_int]
        for fn in (L.ora_sum, L.ora_min, L.ora_max):
            fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, dp, C.c_int]
        L.ora_filter_agg.argtypes = [C.c_void_p, C.POINTER(Pred), C.c_void_p, C.c_int64, C.c_void_p,
                                     dp, dp, dp, C.c_int]
        L.ora_read_bits.argtypes = [C.c_char_p, C.c_uint64, u64p, C.c_int, u64p]
        L.ora_decode_chunk.argtypes = [C.c_char_p, C.c_uint64, C.c_int, C.c_uint64, dp, C.c_uint64, u64p]
        L.ora_buff_fixed.argtypes = [C.c_double, C.c_int32]
        L.ora_buff_fixed.restype = C.c_int64
        L.ora_buff_precision.argtypes = [C.c_uint64]
        L.ora_buff_precision.restype = C.c_int32
        L.ora_aggregate.argtypes = [C.POINTER(C.c_void_p), C.c_uint32, C.c_int, C.POINTER(ExprNode), C.c_uint32,
                                    C.c_void_p, dp, dp, C.c_uint64, u64p]
        _lib = L
    return _lib


def _check(code, what):
    if code != 0:
        raise OracleError(code, what)


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _mask_ptr(mask):
    if mask is None:
        return None
    mask = np.ascontiguousarray(mask, dtype=np.uint64)
    return mask.ctypes.data_as(C.c_void_p), mask


def encode(values, scheme, chunk_kind=CHUNK_RECORD_COUNT, chunk_value=8192, scale=1) -> bytes:
    """Encoder::new(..).encode() on an in-memory f64 column; returns EBI1 bytes."""
    v = np.ascontiguousarray(values, dtype=np.float64)
    out = C.POINTER(C.c_uint8)()
    n = C.c_uint64()
    sch = SCHEMES[scheme] if isinstance(scheme, str) else scheme
    _check(lib().ora_encode(_dptr(v), len(v), sch, chunk_kind, chunk_value, scale,
                            C.byref(out), C.byref(n)), "encode")
    try:
        return C.string_at(out, n.value)
    finally:
        lib().ora_free(out)


def encode_chunk(values, scheme, scale=1) -> bytes:
    v = np.ascontiguousarray(values, dtype=np.float64)
    out = C.POINTER(C.c_uint8)()
    n = C.c_uint64()
    sch = SCHEMES[scheme] if isinstance(scheme, str) else scheme
    _check(lib().ora_encode_chunk(_dptr(v), len(v), sch, scale, C.byref(out), C.byref(n)), "encode_chunk")
    try:
        return C.string_at(out, n.value)
    finally:
        lib().ora_free(out)


def decode_chunk(chunk: bytes, scheme, n_rows=0, cap=None):
    sch = SCHEMES[scheme] if isinstance(scheme, str) else scheme
    cap = cap if cap is not None else max(8 * len(chunk) + 64, n_rows + 1)
    out = np.empty(cap, dtype=np.float64)
    n = C.c_uint64()
    _check(lib().ora_decode_chunk(chunk, len(chunk), sch, n_rows, _dptr(out), cap, C.byref(n)), "decode_chunk")
    return out[: n.value].copy()


def read_bits(buf: bytes, reads):
    """Runs a sequence of read_bits(n) calls; None marks a read that found too few bits."""
    pos = C.c_uint64(0)
    res = []
    for n in reads:
        v = C.c_uint64()
        ok = lib().ora_read_bits(buf, len(buf), C.byref(pos), n, C.byref(v))
        res.append(v.value if ok else None)
    return res


def buff_fixed(v, frac): return lib().ora_buff_fixed(float(v), int(frac))
def buff_precision(scale): return lib().ora_buff_precision(int(scale))


class Decoder:
    """Mirror of api::decoder::Decoder over an in-memory EBI1 file."""

    def __init__(self, data: bytes, threads: int = 1):
        self._data = bytes(data)
        self.threads = threads
        h = C.c_void_p()
        _check(lib().ora_open(self._data, len(self._data), C.byref(h)), "Decoder::new")
        self._h = h

    def close(self):
        if self._h:
            lib().ora_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def n_records(self): return lib().ora_num_records(self._h)
    @property
    def n_chunks(self): return lib().ora_num_chunks(self._h)
    @property
    def scheme(self): return lib().ora_scheme(self._h)

    def chunk_info(self, i):
        a, b, c, d = (C.c_uint64() for _ in range(4))
        _check(lib().ora_chunk_info(self._h, i, C.byref(a), C.byref(b), C.byref(c), C.byref(d)), "chunk_info")
        return a.value, b.value, c.value, d.value

    def with_precision(self, p: int):
        lib().ora_set_precision(self._h, p)

    def _mask(self, mask):
        if mask is None:
            return None, None
        m = np.ascontiguousarray(mask, dtype=np.uint64)
        assert len(m) >= (self.n_records + 63) // 64
        return m.ctypes.data_as(C.c_void_p), m

    def materialize(self, bitmask=None, chunk_id=None):
        mp, keep = self._mask(bitmask)
        cap = max(self.n_records, 1) * 2 + 16
        out = np.empty(cap, dtype=np.float64)
        n = C.c_uint64()
        _check(lib().ora_materialize(self._h, mp, -1 if chunk_id is None else chunk_id, _dptr(out), cap,
                                     C.byref(n), self.threads), "materialize")
        return out[: n.value].copy()

    def filter(self, pred, bitmask=None, chunk_id=None):
        mp, keep = self._mask(bitmask)
        out = np.zeros(max((self.n_records + 63) // 64, 1), dtype=np.uint64)
        _check(lib().ora_filter(self._h, C.byref(pred), mp, -1 if chunk_id is None else chunk_id,
                                out.ctypes.data_as(C.c_void_p), self.threads), "filter")
        return out

    def filter_materialize(self, pred, bitmask=None, chunk_id=None):
        mp, keep = self._mask(bitmask)
        cap = max(self.n_records, 1) * 2 + 16
        out = np.empty(cap, dtype=np.float64)
        n = C.c_uint64()
        _check(lib().ora_filter_materialize(self._h, C.byref(pred), mp, -1 if chunk_id is None else chunk_id,
                                            _dptr(out), cap, C.byref(n), self.threads), "filter_materialize")
        return out[: n.value].copy()

    def _agg(self, fn, bitmask, chunk_id, what):
        mp, keep = self._mask(bitmask)
        out = C.c_double()
        _check(fn(self._h, mp, -1 if chunk_id is None else chunk_id, C.byref(out), self.threads), what)
        return out.value

    def sum(self, bitmask=None, chunk_id=None): return self._agg(lib().ora_sum, bitmask, chunk_id, "sum")
    def min(self, bitmask=None, chunk_id=None): return self._agg(lib().ora_min, bitmask, chunk_id, "min")
    def max(self, bitmask=None, chunk_id=None): return self._agg(lib().ora_max, bitmask, chunk_id, "max")

    def filter_agg(self, pred, bitmask=None, chunk_id=None, want_mask=True):
        mp, keep = self._mask(bitmask)
        out = np.zeros(max((self.n_records + 63) // 64, 1), dtype=np.uint64) if want_mask else None
        s, a, b = C.c_double(), C.c_double(), C.c_double()
        _check(lib().ora_filter_agg(self._h, C.byref(pred), mp, -1 if chunk_id is None else chunk_id,
                                    out.ctypes.data_as(C.c_void_p) if out is not None else None,
                                    C.byref(s), C.byref(a), C.byref(b), self.threads), "filter_agg")
        return out, s.value, a.value, b.value


def mask_from_rows(rows, n_records):
    m = np.zeros(max((n_records + 63) // 64, 1), dtype=np.uint64)
    for r in rows:
        m[r >> 6] |= np.uint64(1) << np.uint64(r & 63)
    return m


def rows_from_mask(mask, n_records=None):
    bits = np.unpackbits(np.ascontiguousarray(mask, dtype=np.uint64).view(np.uint8), bitorder="little")
    rows = np.nonzero(bits)[0]
    if n_records is not None:
        rows = rows[rows < n_records]
    return rows.tolist()


def aggregate(decoders, kind, postfix, bitmask=None):
    """Aggregation::new(kind, expr).compute(decoders, bitmask) over oracle
    Decoders; postfix = [(EXPR_*, index, literal), ...].  Returns a float, or
    the concatenated values (numpy) for AGGR_NONE."""
    hs = (C.c_void_p * len(decoders))(*[d._h.value if isinstance(d._h, C.c_void_p) else d._h for d in decoders])
    nodes = (ExprNode * max(len(postfix), 1))(*[ExprNode(k, i, float(x)) for k, i, x in postfix])
    keep = None
    mp = None
    if bitmask is not None:
        keep = np.ascontiguousarray(bitmask, dtype=np.uint64)
        mp = keep.ctypes.data_as(C.c_void_p)
    out = C.c_double()
    n = C.c_uint64()
    if kind != AGGR_NONE:
        _check(lib().ora_aggregate(hs, len(decoders), kind, nodes, len(postfix), mp, C.byref(out), None, 0,
                                   C.byref(n)), "Aggregation::compute")
        return out.value
    cap = 0
    while True:
        arr = np.empty(max(cap, 1), dtype=np.float64)
        rc = lib().ora_aggregate(hs, len(decoders), kind, nodes, len(postfix), mp, C.byref(out), _dptr(arr), cap,
                                 C.byref(n))
        if rc == 7 and n.value > cap:
            cap = n.value
            continue
        _check(rc, "Aggregation::compute")
        return arr[: n.value]
