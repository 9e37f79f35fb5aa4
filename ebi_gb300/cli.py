"""Command line of the engine in the shape of lemolatoon/ebi's experimenter
(experimenter/src/main.rs): the per-file commands compress, filter,
filter-materialize, materialize, max and sum, reading the same JSON configs
and writing the same OutputWrapper JSON (experimenter/src/lib.rs:177-189) to
<file dir>/../result/<file stem>/<command>/NNN.json, so the reference's
tools/plot.py reads the results.

    python -m ebi_gb300 --input 'data/*.ebi' filter --config filter.json [--in-memory true]

Configs (serde JSON of the reference types):
  compress            CompressionConfig {"chunk_option": "Full" | {"RecordCount": n} |
                      {"ByteSizeBestEffort": n}, "compressor_config": {"type": "BUFF",
                      "scale": 1000} | {"type": "Gorilla", "capacity": 8192} | ...};
                      the input is raw f64 (native endian), the output <input>.ebi
  filter, filter-materialize
                      {"predicate": {"type": "Range", "predicate": {"start": {"Inclusive": 10.0},
                      "end": "None"}} | {"type": "Eq", "predicate": 1.0} | {"type": "Ne", ...},
                       "chunk_id": null | n, "bitmask": null | [row ids]}
  materialize, max, sum
                      {"chunk_id": null | n, "bitmask": null | [row ids]}

Timing: elapsed_time_nanos is host wall time, as the experimenter measures
it.  With --in-memory true the column is opened from the file's bytes before
the clock starts, and the clock covers the query and its read-back.  Without
it the clock also covers the file's transfer into HBM (io_read_nanos) and the
write of a materialized output to <input>.materialized or
<input>.filter_materialized.  execution_times carries the engine's device time
of the query: the decode-and-compare kernel under the codec's segment
(xor_nanos for the XOR family, bit_packing_nanos for BUFF, decompression_nanos
for RLE and Uncompressed) and the chunk-ordered fold under sum_nanos.
"""
from __future__ import annotations

import argparse
import datetime as _dt
import glob as _glob
import json
import os
import struct
import sys
import time
from decimal import Decimal
from pathlib import Path

import numpy as np

from . import api as E

VERSION = "0.1.0"
SCHEME_NAMES = {0: "Uncompressed", 1: "RLE", 2: "BUFF", 3: "Gorilla", 4: "Chimp", 5: "Chimp128",
                6: "ElfOnChimp", 7: "Elf"}
SCHEME_IDS = {v: k for k, v in SCHEME_NAMES.items()}
DECODE_SEGMENT = {0: "decompression_nanos", 1: "decompression_nanos", 2: "bit_packing_nanos"}
SEGMENTS = ["io_read_nanos", "io_write_nanos", "xor_nanos", "delta_nanos", "quantization_nanos",
            "bit_packing_nanos", "compare_insert_nanos", "sum_nanos", "decompression_nanos"]
COMMAND_DIRS = {"compress": "compress", "filter": "filter", "filter-materialize": "filter_materialize",
                "materialize": "materialize", "max": "max", "sum": "sum"}


# ---- formats of the reference's result strings ------------------------------------------------------
def rust_f64(x: float) -> str:
    """f64's Display: the shortest digits that round-trip, never in exponent form."""
    if x != x:
        return "NaN"
    if x in (float("inf"), float("-inf")):
        return "inf" if x > 0 else "-inf"
    s = format(Decimal(repr(float(x))), "f")
    if "." in s:
        s = s.rstrip("0").rstrip(".")
    return s


def bitmap_string(rows: np.ndarray) -> str:
    """The Debug form of the RoaringBitmap a filter returns: the ids when fewer
    than 16, else the count and the range."""
    n = len(rows)
    if n < 16:
        return "RoaringBitmap<[" + ", ".join(str(int(r)) for r in rows) + "]>"
    return f"RoaringBitmap<{n} values between {int(rows[0])} and {int(rows[-1])}>"


# ---- EBI1 metadata (format.rs:143-258) ---------------------------------------------------------------
def file_info(data: bytes | None = None, path: str | None = None) -> dict:
    """Header and footer facts: scheme, chunk option, compressor config value, sizes."""
    if data is None:
        with open(path, "rb") as f:
            head = f.read(30)
            footer = struct.unpack_from("<Q", head, 16)[0]
            f.seek(footer)
            f0 = f.read(16)
            nrec, nch = struct.unpack("<QQ", f0)
            chunk_footers = f.read(16 * nch)
            cfg = f.read(9)
            size = os.path.getsize(path)
    else:
        head = data[:30]
        footer = struct.unpack_from("<Q", data, 16)[0]
        nrec, nch = struct.unpack_from("<QQ", data, footer)
        chunk_footers = data[footer + 16: footer + 16 + 16 * nch]
        cfg = data[footer + 16 + 16 * nch: footer + 16 + 16 * nch + 9]
        size = len(data)
    scheme, kind = head[5], head[6]
    value = struct.unpack_from("<Q", head, 8)[0]
    config_value = struct.unpack_from("<Q", cfg, 1)[0] if len(cfg) == 9 else 0
    first_chunk = struct.unpack_from("<Q", chunk_footers, 0)[0] if nch else footer
    return {"scheme": scheme, "chunk_kind": kind, "chunk_value": value, "config_value": config_value,
            "n_records": nrec, "n_chunks": nch, "file_size": size, "chunk_bytes": footer - first_chunk,
            "footer_offset": footer}


def compression_config(info: dict) -> dict:
    kind, value = info["chunk_kind"], info["chunk_value"]
    chunk = "Full" if kind == 0 else {"RecordCount": value} if kind == 1 else {"ByteSizeBestEffort": value}
    name = SCHEME_NAMES.get(info["scheme"], str(info["scheme"]))
    field = "scale" if name == "BUFF" else "capacity"
    return {"chunk_option": chunk, "compressor_config": {"type": name, field: info["config_value"]}}


# ---- configs ---------------------------------------------------------------------------------------
def predicate_from_json(p: dict) -> E.Predicate:
    t = p["type"]
    if t == "Eq":
        return E.Predicate.eq(float(p["predicate"]))
    if t == "Ne":
        return E.Predicate.ne(float(p["predicate"]))
    if t != "Range":
        raise ValueError(f"unknown predicate type {t!r}")

    def bound(b):
        if b == "None" or b is None:
            return E.RangeValue.NONE
        (k, v), = b.items()
        return E.RangeValue.inclusive(v) if k == "Inclusive" else E.RangeValue.exclusive(v)

    r = p["predicate"]
    return E.Predicate.range_(bound(r["start"]), bound(r["end"]))


def _mask(d: E.Decoder, rows):
    return None if rows is None else E.mask_from_rows(rows, d.n_records, device=d.device)


# ---- commands ------------------------------------------------------------------------------------
def _execution_times(d: E.Decoder, scheme: int, io_read_ns: int = 0) -> dict:
    t = d.segmented_execution_times() or {}
    out = {k: 0 for k in SEGMENTS}
    out[DECODE_SEGMENT.get(scheme, "xor_nanos")] = int(round(1e6 * t.get("scan_ms", 0.0)))
    out["sum_nanos"] = int(round(1e6 * t.get("finalize_ms", 0.0)))
    out["io_read_nanos"] = io_read_ns
    return out


def _query(d: E.Decoder, command: str, cfg: dict):
    """One query; returns the result string and, for the materializing
    commands, the host copy of the values."""
    mask = _mask(d, cfg.get("bitmask"))
    chunk_id = cfg.get("chunk_id")
    if command == "filter":
        out = d.filter(predicate_from_json(cfg["predicate"]), mask, chunk_id)
        return bitmap_string(E.rows_from_mask(out, d.n_records).cpu().numpy().view(np.uint32)), None
    if command in ("filter-materialize", "materialize"):
        if command == "materialize":
            vals = d.materialize(mask, chunk_id).cpu().numpy()
        else:
            vals = d.filter_materialize(predicate_from_json(cfg["predicate"]), mask, chunk_id).cpu().numpy()
        return f"bytes: {vals.nbytes}", vals
    if command == "max":
        return rust_f64(d.max(mask, chunk_id)), None
    if command == "sum":
        return rust_f64(d.sum(mask, chunk_id)), None
    raise ValueError(command)


OUTPUT_SUFFIX = {"materialize": ".materialized", "filter-materialize": ".filter_materialized"}


def run_query(command: str, path: str, cfg: dict, in_memory: bool):
    """In memory: the file's bytes are read and the column opened before the
    clock starts, which then covers the query and its read-back.  From the
    file: the clock covers the file's transfer into HBM, the query and the
    write of a materialized output (<input>.materialized), as the
    experimenter's file mode covers the chunk reads and the output write."""
    import torch

    if in_memory:
        data = Path(path).read_bytes()
        info = file_info(data=data)
        d = E.Decoder(data)
        d.set_timing(True)
        torch.cuda.synchronize(d.device)
        io = 0
        t0 = time.perf_counter_ns()
    else:
        info = file_info(path=path)
        t0 = time.perf_counter_ns()
        d = E.Decoder.from_file(path)
        d.set_timing(True)
        torch.cuda.synchronize(d.device)
        io = time.perf_counter_ns() - t0
    try:
        result, vals = _query(d, command, cfg)
        if vals is not None and not in_memory:
            vals.tofile(Path(path).with_suffix(OUTPUT_SUFFIX[command]))
            result = f"bytes: {os.path.getsize(Path(path).with_suffix(OUTPUT_SUFFIX[command]))}"
        elapsed = time.perf_counter_ns() - t0
        times = _execution_times(d, info["scheme"], io)
    finally:
        d.close()
    return compression_config(info), elapsed, times, result


def run_compress(path: str, cfg: dict, in_memory: bool):
    v = np.fromfile(path, dtype=np.float64)
    co = cfg["chunk_option"]
    if co == "Full":
        chunk = ("full", 0)
    else:
        (k, n), = co.items()
        chunk = ("record_count", n) if k == "RecordCount" else ("byte_size", n)
    cc = cfg["compressor_config"]
    scheme = SCHEME_IDS[cc["type"]]
    scale = int(cc.get("scale", 1))
    t0 = time.perf_counter_ns()
    data = bytearray(E.encode(v, scheme, chunk, scale))
    elapsed = time.perf_counter_ns() - t0
    info = file_info(data=bytes(data))
    if "capacity" in cc:  # the config's u64 (capacity) as the caller set it
        at = info["footer_offset"] + 16 + 16 * info["n_chunks"] + 1
        struct.pack_into("<Q", data, at, int(cc["capacity"]))
    out = Path(path).with_suffix(".ebi")
    out.write_bytes(bytes(data))
    info = file_info(data=bytes(data))
    stats = {"compression_elapsed_time_nano_secs": elapsed, "uncompressed_size": 8 * info["n_records"],
             "compressed_size": info["file_size"], "compressed_size_chunk_only": info["chunk_bytes"]}
    u = max(stats["uncompressed_size"], 1)
    stats["compression_ratio"] = stats["compressed_size"] / u
    stats["compression_ratio_chunk_only"] = stats["compressed_size_chunk_only"] / u
    times = {k: 0 for k in SEGMENTS}
    return cfg, elapsed, times, f"number_of_records: {info['n_records']}", stats


def process_file(path: str, command: str, config_path: str, in_memory: bool) -> Path:
    cfg = json.loads(Path(config_path).read_text())
    now = _dt.datetime.now(_dt.timezone.utc).isoformat().replace("+00:00", "Z")
    if command == "compress":
        comp, elapsed, times, result, specific = run_compress(path, cfg, in_memory)
    else:
        comp, elapsed, times, result = run_query(command, path, cfg, in_memory)
        specific = cfg
    output = {"in_memory": in_memory, "version": VERSION, "config_path": config_path, "compression_config": comp,
              "command_specific": specific, "elapsed_time_nanos": int(elapsed), "execution_times": times,
              "input_filename": path, "datetime": now, "result_string": result}
    p = Path(path).resolve()
    save_dir = p.parent.parent / "result" / p.stem / COMMAND_DIRS[command]
    save_dir.mkdir(parents=True, exist_ok=True)
    k = 0
    while (save_dir / f"{k:03d}.json").exists():
        k += 1
    out = save_dir / f"{k:03d}.json"
    out.write_text(json.dumps(output, indent=2))
    return out


def _bool(s: str) -> bool:
    if s.lower() in ("true", "1", "yes"):
        return True
    if s.lower() in ("false", "0", "no"):
        return False
    raise argparse.ArgumentTypeError(f"expected true or false, got {s!r}")


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m ebi_gb300", description=__doc__.split("\n\n")[0])
    ap.add_argument("-i", "--input", required=True, help="glob of input files")
    sub = ap.add_subparsers(dest="command", required=True)
    for name in COMMAND_DIRS:
        s = sub.add_parser(name)
        s.add_argument("-c", "--config", required=True)
        s.add_argument("-i", "--in-memory", type=_bool, default=False)
    a = ap.parse_args(argv)
    files = sorted(_glob.glob(a.input))
    failed = 0
    for i, f in enumerate(files):
        print(f"[{i:03d}/{len(files):03d}] Processing file: {f}")
        if os.path.isdir(f):
            print(f"Skipping directory: {f}", file=sys.stderr)
            continue
        try:
            out = process_file(f, a.command, a.config, a.in_memory)
            print(f"[{i + 1:03d}/{len(files):03d}] Finished processing file: {f} -> {out}")
        except Exception as e:  # report and go on with the next file, as the experimenter does
            failed += 1
            print(f"Failed to process file {f}: {e!r}", file=sys.stderr)
    return 1 if failed else 0
