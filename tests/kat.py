"""Loads the known-answer vectors of tests/golden/kat.json and turns them into oracle calls."""
import json
from pathlib import Path

from oracle import oracle as O

KAT = json.loads((Path(__file__).resolve().parent / "golden" / "kat.json").read_text())

BOUND = {"none": O.BOUND_NONE, "incl": O.BOUND_INCLUSIVE, "excl": O.BOUND_EXCLUSIVE}
CODECS = ["uncompressed", "rle", "gorilla", "chimp", "chimp128", "elf_on_chimp", "elf", "buff"]


def chunk_option(spec):
    kind, v = spec
    return ({"record_count": O.CHUNK_RECORD_COUNT, "byte_size": O.CHUNK_BYTE_SIZE,
             "full": O.CHUNK_FULL}[kind], int(v))


def pred_tuple(spec):
    """(kind, start_kind, start, end_kind, end, value) for a kat.json predicate."""
    if spec[0] == "eq":
        return (O.PRED_EQ, 0, 0.0, 0, 0.0, float(spec[1]))
    if spec[0] == "ne":
        return (O.PRED_NE, 0, 0.0, 0, 0.0, float(spec[1]))
    (sk, sv), (ek, ev) = spec[1], spec[2]
    return (O.PRED_RANGE, BOUND[sk], float(sv), BOUND[ek], float(ev), 0.0)


def oracle_pred(spec):
    k, sk, sv, ek, ev, v = pred_tuple(spec)
    return O.Pred(k, sk, ek, 0, v, sv, ev)


def round_at(x, scale):
    """round_at of ebi/tests/aggregation.rs:14-16 with Rust's half-away-from-zero rounding."""
    import numpy as np
    y = np.asarray(x, dtype=np.float64) * scale
    r = np.trunc(y)
    r = r + np.where(np.abs(y - r) >= 0.5, np.sign(y), 0.0)
    return r / scale
