"""Writes tests/golden/kat.json: the known-answer vectors held by lemolatoon/ebi's own tests.

The reference is a Rust workspace and no Rust toolchain exists where this
project is built, so its tests cannot be run to dump fixtures.  Instead the
fixed (non-random) cases of its test suite are transcribed here, each with the
reference file:line it comes from.  Its randomised tests draw from an unseeded
RNG (`StdRng::from_entropy()`, ebi/tests/common/mod.rs:34) and hold no
vectors; tests/test_gpu_values.py and tests/test_gpu_buff.py restate their pattern with a seeded RNG.

Run:  python tests/golden/make_golden.py      (rewrites kat.json next to this file)
"""
from __future__ import annotations

import json
from pathlib import Path

# --- io/bit_read.rs doctests: sequences of read_bits(n); None = too few bits -----------
BIT_READS = [
    # read_bit / read_bits(7) / read_bit -> None (io/bit_read.rs:198-210)
    {"src": "ebi/src/io/bit_read.rs:198-210", "buf": [0b10101010], "reads": [1, 7, 1],
     "expect": [1, None, None], "check": [True, False, True]},
    # read_bits(4), read_bits(12), read_bits(4) -> None (io/bit_read.rs:278-292)
    {"src": "ebi/src/io/bit_read.rs:278-292", "buf": [0b10110000, 0b11110000], "reads": [4, 12, 4],
     "expect": [0b1011, 0b0000_1111_0000, None], "check": [True, True, True]},
    # read_byte, read_bit, unaligned read_byte, read_byte -> None (io/bit_read.rs:234-250)
    {"src": "ebi/src/io/bit_read.rs:234-250", "buf": [0xAA, 0b0101_1111, 0b1100_0011], "reads": [8, 1, 8, 8],
     "expect": [0xAA, 0, 0b1011_1111, None], "check": [True, True, True, True]},
    # skip_bits(4) read 3, skip 5 read 3, skip 9 read_byte (io/bit_read.rs:164-178)
    {"src": "ebi/src/io/bit_read.rs:164-178", "buf": [0b1010_1010, 0b1111_0010, 0b1111_1111, 0b0011_1100],
     "reads": [4, 3, 5, 3, 9, 8], "expect": [None, 0b101, None, 0b001, None, 0b0011_1100],
     "check": [False, True, False, True, False, True]},
    # read 4 -> 0b1011; 5 more -> None (does not advance); 4 more -> 0 (io/bit_read.rs:342-355)
    {"src": "ebi/src/io/bit_read.rs:342-355", "buf": [0b10110000], "reads": [4, 5, 4],
     "expect": [0b1011, None, 0b0000], "check": [True, True, True]},
]

# --- Gorilla [12.0, 24.0] (decoder/chunk_reader/gorilla.rs:161-207) --------------------
# The test lists `_encoded` but never asserts it; its first 80 bits are ebi's
# stream (12.0 raw, '11', leading 01011, sig-1 000000, payload '1', and the
# '11' that opens the end marker); the bytes after that follow upstream tsz's
# end marker, not ebi's NaN marker (compressor/gorilla.rs:27-30).
GORILLA_PREFIX = {"src": "ebi/src/decoder/chunk_reader/gorilla.rs:173-192",
                  "values": [12.0, 24.0],
                  "prefix_bytes": [0x40, 0x28, 0, 0, 0, 0, 0, 0, 0b11010110, 0b00000111]}

# --- Fixed filter cases (ebi/tests/query.rs:285-757), run for every codec --------------
# chunk: ["record_count", k] | ["byte_size", n];  pred: ["range", [kind, v], [kind, v]] with
# kind in {"incl", "excl", "none"} | ["eq", v] | ["ne", v];  expect: sorted row ids.
S = [1.0] * 5 + [2.0] * 15 + [10.5, 10.6, 10.7, 10.9, 10.9] + [100.0] * 5 + [10.0] * 5
V1 = [-300.3, -5.6, -3.8, -699.7, 2.1, 9.9, 100.1]
V2 = [3.3, 5.6, 3.8, 6.7, 2.1, 9.9, 10.1]
V3 = [3.3, 5.6, 3.8, 6.7, 2.1, 9.9, 10.1, 3.8]
T6 = [14.22, 5.57, 6.61, 9.25, 2.72, 8.23, 13.2, -0.68, 12.95, 13.85, 12.21, 10.36, 2.33,
      8.5, 18.13, 19.54, 16.42, 19.12, 11.68, 1.78, 7.73, -2.19, 17.43, 21.88, 3.01,
      10.76, 25.08, 4.01, 8.84, 23.35, -4.32, 12.5, 5.72, -7.0, 14.02, -1.23, 19.57,
      6.73, 8.4, 11.27, 15.61, -3.01, -15.35, 14.38, -3.09, 19.94, 23.16, 10.28, 1.46,
      9.2, 20.33, 8.93, 2.18, 1.54, -0.48, -4.13, 16.71, 3.71, 9.09, -10.67, 13.75,
      14.24, 10.93, 8.0, 23.34, 8.92, 1.81, 5.89, 13.97, -7.69, 18.02, 4.85, 4.21, 17.07,
      -0.65, 11.39, 10.36, 17.98, 4.27, 2.95, 18.71, 0.72, 1.85, -5.6, 6.43, 12.12,
      -2.33, -0.91, 14.51, 5.36, 5.49, 5.11, 10.65, 0.39, -1.55, 10.05, -2.89, 21.09,
      -3.97, 7.83, 22.17, 20.66, 7.24, 15.89, 1.96, 13.53, 10.87, 9.67, 12.27, 12.62,
      3.52, 24.96, 13.25, 25.06]
T6_EXPECT = [0, 1, 2, 3, 4, 5, 6, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 22, 23, 24,
             25, 26, 27, 28, 29, 31, 32, 34, 36, 37, 38, 39, 40, 43, 45, 46, 47, 48, 49, 50, 51,
             52, 53, 56, 57, 58, 60, 61, 62, 63, 64, 65, 66, 67, 68, 70, 71, 72, 73, 75, 76, 77,
             78, 79, 80, 81, 82, 84, 85, 88, 89, 90, 91, 92, 93, 95, 97, 99, 100, 101, 102, 103,
             104, 105, 106, 107, 108, 109, 110, 111, 112, 113]
F41 = ([41.4] * 15 + [41.5] * 15) * 2

FILTER_CASES = [
    {"src": "ebi/tests/query.rs:285-299", "values": V1, "chunk": ["record_count", 5],
     "pred": ["range", ["incl", -3.8], ["none", 0]], "expect": [2, 4, 5, 6]},
    {"src": "ebi/tests/query.rs:301-317", "values": V1, "chunk": ["record_count", 5],
     "pred": ["range", ["incl", -3.8], ["incl", 9.9]], "expect": [2, 4, 5]},
    {"src": "ebi/tests/query.rs:319-335", "values": V2, "chunk": ["record_count", 5],
     "pred": ["range", ["excl", 3.8], ["incl", 9.9]], "expect": [1, 3, 5]},
    {"src": "ebi/tests/query.rs:337-353", "values": V2, "chunk": ["record_count", 5],
     "pred": ["range", ["incl", 3.8], ["excl", 9.9]], "expect": [1, 2, 3]},
    {"src": "ebi/tests/query.rs:355-371", "values": V2, "chunk": ["record_count", 5],
     "pred": ["range", ["excl", 3.8], ["excl", 9.9]], "expect": [1, 3]},
    {"src": "ebi/tests/query.rs:373-387", "values": [3.3, 52.6, 3.8, 6.7, 2.1, 9.9, 100.1],
     "chunk": ["record_count", 5], "pred": ["range", ["excl", 3.8], ["none", 0]], "expect": [1, 3, 5, 6]},
    {"src": "ebi/tests/query.rs:389-403", "values": V2, "chunk": ["record_count", 5],
     "pred": ["range", ["incl", 3.8], ["none", 0]], "expect": [1, 2, 3, 5, 6]},
    {"src": "ebi/tests/query.rs:405-419", "values": V2, "chunk": ["record_count", 5],
     "pred": ["range", ["none", 0], ["excl", 9.9]], "expect": [0, 1, 2, 3, 4]},
    {"src": "ebi/tests/query.rs:421-435", "values": V2, "chunk": ["record_count", 5],
     "pred": ["range", ["none", 0], ["none", 0]], "bitmask": [0, 1, 3, 4, 6], "expect": [0, 1, 3, 4, 6]},
    {"src": "ebi/tests/query.rs:437-456", "values": [9.9, 10.1], "chunk": ["record_count", 5],
     "pred": ["range", ["incl", -1000.0], ["incl", 10000000.0]], "expect": [0, 1]},
    {"src": "ebi/tests/query.rs:458-480", "values": S, "chunk": ["record_count", 35],
     "pred": ["range", ["incl", 10.7], ["none", 0]], "expect": list(range(22, 30))},
    {"src": "ebi/tests/query.rs:482-504", "values": S, "chunk": ["record_count", 35],
     "pred": ["range", ["none", 0], ["excl", 10.7]], "expect": list(range(0, 22)) + list(range(30, 35))},
    {"src": "ebi/tests/query.rs:509-522", "values": [322.3, 5204029348.6, 3.8, -6.7, 2.1, 99.9, 1000220.1, 3.8],
     "chunk": ["record_count", 5], "pred": ["eq", 3.8], "expect": [2, 7]},
    {"src": "ebi/tests/query.rs:524-537", "values": [3.7, 522.6, 3.8, 6099.7, -22390.1, 908.9, -10.1, 3.8],
     "chunk": ["record_count", 5], "pred": ["ne", 3.8], "expect": [0, 1, 3, 4, 5, 6]},
    {"src": "ebi/tests/query.rs:539-560", "values": S, "chunk": ["record_count", 35],
     "pred": ["eq", 10.5], "expect": [20]},
    {"src": "ebi/tests/query.rs:562-583", "values": S, "chunk": ["record_count", 35],
     "pred": ["ne", 10.5], "expect": list(range(0, 20)) + list(range(21, 35))},
    {"src": "ebi/tests/query.rs:585-602", "values": [-7072.1] * 32 + [-7071.2], "chunk": ["record_count", 35],
     "pred": ["ne", -7071.2], "expect": list(range(0, 32))},
    {"src": "ebi/tests/query.rs:604-624", "values": F41, "chunk": ["record_count", 33],
     "pred": ["range", ["incl", 41.4], ["none", 0]], "expect": list(range(0, 60))},
    {"src": "ebi/tests/query.rs:626-645", "values": [5714.14, 5710.09, 5718.45, 5712.45, 5714.98, 5715.13,
                                                     5717.12, 5714.03, 5712.14, 5714.21, 5716.51],
     "chunk": ["byte_size", 5274], "pred": ["range", ["incl", 5715.88], ["none", 0]],
     "bitmask": [0, 3, 5, 8, 9, 10], "expect": [10]},
    {"src": "ebi/tests/query.rs:647-680", "values": T6, "chunk": ["record_count", 50],
     "pred": ["range", ["incl", 0.37], ["none", 0]], "expect": T6_EXPECT},
    {"src": "ebi/tests/query.rs:685-700", "values": V3, "chunk": ["record_count", 5],
     "pred": ["range", ["excl", 3.8], ["none", 0]], "bitmask": [0, 2, 3, 4, 6, 7], "expect": [3, 6]},
    {"src": "ebi/tests/query.rs:702-716", "values": [3.3, 5.6, 3.8, 3.3, 2.1, 9.9, 10.1, 3.8],
     "chunk": ["record_count", 5], "pred": ["ne", 3.3], "bitmask": [0, 2, 3, 4, 6, 7], "expect": [2, 4, 6, 7]},
    {"src": "ebi/tests/query.rs:718-736", "values": V3, "chunk": ["record_count", 3],
     "pred": ["range", ["incl", 3.8], ["excl", 9.9]], "chunk_id": 2, "expect": [7]},
    {"src": "ebi/tests/query.rs:738-757", "values": V3, "chunk": ["record_count", 3],
     "pred": ["range", ["excl", 3.8], ["incl", 9.9]], "chunk_id": 1, "bitmask": [0, 2, 3, 5, 7],
     "expect": [3, 5]},
]
# BUFF runs these with scale 100 (ebi/tests/query.rs:1318-1336); the other codecs take no scale.
FILTER_BUFF_SCALE = 100

# --- Fixed aggregation cases (ebi/tests/aggregation.rs:202-241, 313-322, 360-369) -----------
AGG_CASES = [
    {"src": "ebi/tests/aggregation.rs:202-211", "op": "sum", "values": [0.0, 2.0, 3.0, 4.0, 5.0],
     "chunk": ["record_count", 8], "expect": 14.0},
    {"src": "ebi/tests/aggregation.rs:212-221", "op": "sum", "values": [11.0, 12.0],
     "chunk": ["record_count", 8], "bitmask": [0], "expect": 11.0},
    {"src": "ebi/tests/aggregation.rs:222-231", "op": "sum", "values": [0.0, 2.0, 3.0, 4.0, 500.0],
     "chunk": ["record_count", 8], "expect": 509.0},
    {"src": "ebi/tests/aggregation.rs:232-241", "op": "sum", "values": [-1.0, 2.0, 3.0, 4.0, 5.0],
     "chunk": ["record_count", 8], "expect": 13.0},
    {"src": "ebi/tests/aggregation.rs:313-322", "op": "max", "values": [-1.0, 2.0, 3.0, 4.0, 5.0],
     "chunk": ["record_count", 8], "expect": 5.0},
    {"src": "ebi/tests/aggregation.rs:360-369", "op": "min", "values": [-1.0, 2.0, 3.0, 4.0, 5.0],
     "chunk": ["record_count", 8], "expect": -1.0},
]
# Tolerances of the reference (aggregation.rs:72-82): |sum - expect| < 1e-3, or 0.5 * n for
# BUFF; max/min equal after round_at(scale).  BUFF aggregation runs at scale 100
# (aggregation.rs:779-784).
AGG_BUFF_SCALE = 100

# BUFF precision table and scale -> precision (compression_common/buff.rs:36,
# compressor/buff.rs:131-135): scale 10^k selects PRECISION_MAP[k].
BUFF_PRECISION = {"src": "ebi/src/compression_common/buff.rs:36",
                  "precision_map": [0, 5, 8, 11, 15, 18, 21, 25, 28, 31, 35, 38, 50],
                  "scale_to_precision": [[1, 0], [10, 1], [100, 2], [1000, 3], [10000, 4]]}


# --- Aggregation / Expr (ebi/tests/aggregation.rs:471-754) -----------------------------
# Every column is encoded Uncompressed with RecordCount(3) (helper::decoder,
# ebi/tests/aggregation.rs:172-188).  expr: ["index", i] | ["lit", x] |
# [op, lhs, rhs] with op in add/sub/mul/div; kind: sum/min/max; bitmask: row ids.
_I = lambda i: ["index", i]
EXPR_CASES = [
    {"src": "ebi/tests/aggregation.rs:471-479", "columns": [[0.0, 2.0, 3.0, 4.0, 5.0]],
     "aggs": [{"kind": "sum", "expr": _I(0), "expect": 14.0}]},
    {"src": "ebi/tests/aggregation.rs:485-509", "columns": [[0.0, 2.0, -3.0, 4.0, 7.0], [1.0, 2.0, 3.0, 4.0, 5.0]],
     "aggs": [{"kind": "sum", "expr": ["add", ["mul", _I(0), _I(1)], _I(1)], "expect": 61.0}]},
    {"src": "ebi/tests/aggregation.rs:512-519", "columns": [[0.0, 2.0, 3.0, 4.0, 5.0]],
     "aggs": [{"kind": "sum", "expr": _I(0), "expect": 14.0}]},
    {"src": "ebi/tests/aggregation.rs:522-543", "columns": [[0.0, 2.0, -3.0, 4.0, 7.0], [1.0, 2.0, 3.0, 4.0, 5.0]],
     "aggs": [{"kind": "sum", "expr": ["add", ["mul", _I(0), _I(1)], _I(1)], "expect": 61.0}]},
    {"src": "ebi/tests/aggregation.rs:547-554", "columns": [[1.0, 5.0, 2.0, 4.0]],
     "aggs": [{"kind": "max", "expr": _I(0), "expect": 5.0}]},
    {"src": "ebi/tests/aggregation.rs:557-571", "columns": [[1.0, 2.0, 3.0], [2.0, 1.0, 4.0]],
     "aggs": [{"kind": "max", "expr": ["mul", _I(0), _I(1)], "expect": 12.0}]},
    {"src": "ebi/tests/aggregation.rs:575-582", "columns": [[1.0, 5.0, 2.0, 4.0]],
     "aggs": [{"kind": "min", "expr": _I(0), "expect": 1.0}]},
    {"src": "ebi/tests/aggregation.rs:585-599", "columns": [[3.0, 1.0, 4.0], [2.0, 2.0, 1.0]],
     "aggs": [{"kind": "min", "expr": ["sub", _I(0), _I(1)], "expect": -1.0}]},
    {"src": "ebi/tests/aggregation.rs:603-614", "columns": [[0.0, 0.8, 0.3], [1.0, 1.0, 20.0]], "bitmask": [0, 1],
     "aggs": [{"kind": "sum", "expr": _I(0), "expect": 0.8}]},
    {"src": "ebi/tests/aggregation.rs:617-633", "columns": [[1.0, 2.2, 5.0, 4.0]], "bitmask": [0, 2],
     "aggs": [{"kind": "sum", "expr": _I(0), "expect": 6.0}]},
    {"src": "ebi/tests/aggregation.rs:636-663", "columns": [[1.0, 2.0, 3.0], [10.0, 20.0, 30.0]],
     "aggs": [{"kind": "sum", "expr": _I(0), "expect": 6.0},
              {"kind": "sum", "expr": ["add", _I(0), _I(1)], "expect": 66.0}]},
    {"src": "ebi/tests/aggregation.rs:666-693", "columns": [[3.0, 8.0, 5.0], [2.0, 1.0, 7.0]],
     "aggs": [{"kind": "max", "expr": _I(1), "expect": 7.0},
              {"kind": "max", "expr": ["mul", _I(0), _I(1)], "expect": 35.0}]},
    {"src": "ebi/tests/aggregation.rs:696-723", "columns": [[6.0, 2.0, 9.0], [1.0, 2.0, 3.0]],
     "aggs": [{"kind": "min", "expr": _I(0), "expect": 2.0},
              {"kind": "min", "expr": ["sub", _I(0), _I(1)], "expect": 0.0}]},
    {"src": "ebi/tests/aggregation.rs:726-753", "columns": [[1.0, 0.0, 3.0, 4.0], [5.0, 6.0, 7.0, 8.0]],
     "bitmask": [0, 2],
     "aggs": [{"kind": "sum", "expr": _I(0), "expect": 4.0},
              {"kind": "max", "expr": ["add", _I(0), _I(1)], "expect": 10.0}]},
]
EXPR_CHUNK = ["record_count", 3]


def main():
    out = {
        "about": "Known-answer vectors transcribed from lemolatoon/ebi's own tests; see make_golden.py.",
        "bit_reads": BIT_READS,
        "gorilla_prefix": GORILLA_PREFIX,
        "filter_cases": FILTER_CASES,
        "filter_buff_scale": FILTER_BUFF_SCALE,
        "agg_cases": AGG_CASES,
        "agg_buff_scale": AGG_BUFF_SCALE,
        "buff_precision": BUFF_PRECISION,
        "expr_cases": EXPR_CASES,
        "expr_chunk": EXPR_CHUNK,
    }
    path = Path(__file__).resolve().parent / "kat.json"
    path.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {path}")


if __name__ == "__main__":
    main()
