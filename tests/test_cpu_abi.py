"""CPU-only checks of the engine's C ABI: the library loads, exports every
symbol include/ebi_gpu.h declares, and its host-side encoder writes the same
EBI1 bytes as the oracle's restatement of ebi's Encoder (no GPU needed)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import ebi_gb300 as E
from ebi_gb300 import _native
from oracle import oracle as O

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "ebi_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ebi_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(_native.LIB_PATH))
    names = declared_symbols()
    assert names, "no declarations parsed"
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(_native.EXPORTS) == names


def mixed_decimals(rng, n):
    """Decimals of 0-9 digits over magnitudes 1e-14..1e14 with powers of ten,
    zeros, infinities, subnormals and full-precision doubles mixed in."""
    digits = rng.integers(0, 10, n)
    mag = 10.0 ** rng.integers(-14, 15, n)
    v = np.round(rng.uniform(-1, 1, n) * mag * 10.0 ** digits) / 10.0 ** digits
    pick = rng.random(n)
    v = np.where(pick < 0.05, 10.0 ** rng.integers(-320, 300, n).astype(np.float64), v)
    v = np.where((pick >= 0.05) & (pick < 0.07), 0.0, v)
    v = np.where((pick >= 0.07) & (pick < 0.08), rng.normal(0, 1, n), v)
    v = np.where((pick >= 0.08) & (pick < 0.085), 5e-324 * rng.integers(1, 1 << 40, n), v)
    v = np.where((pick >= 0.085) & (pick < 0.087), np.inf * np.sign(rng.normal(size=n)), v)
    return v


def gen(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "walk":
        v = np.round(30 + np.cumsum(rng.normal(0, 0.5, n)), 2)
    elif kind == "uniform":
        v = np.round(rng.uniform(-1000, 1000, n), 3)
    elif kind == "steps":
        v = np.repeat(np.round(rng.normal(0, 5, n // 8 + 1), 1), 8)[:n]
    elif kind == "const":
        v = np.full(n, 3.25)
    elif kind == "decimals":
        v = mixed_decimals(rng, n)
    else:
        v = rng.normal(0, 1e6, n)
    return v + 0.0


@pytest.mark.parametrize("codec", ["uncompressed", "rle", "gorilla", "chimp", "chimp128", "elf_on_chimp", "elf", "buff"])
@pytest.mark.parametrize("kind", ["walk", "uniform", "steps", "const", "wide", "decimals"])
@pytest.mark.parametrize("chunk", [("record_count", 1000), ("record_count", 4097), ("byte_size", 3000), ("full", 0)])
def test_encoder_bytes_match_oracle(codec, kind, chunk):
    v = gen(kind, 5003, 11)
    scale = 1000 if codec == "buff" else 1
    if codec == "buff" and kind == "wide":
        scale = 10
    ck = {"record_count": O.CHUNK_RECORD_COUNT, "byte_size": O.CHUNK_BYTE_SIZE, "full": O.CHUNK_FULL}[chunk[0]]
    assert E.encode(v, codec, chunk, scale) == O.encode(v, codec, ck, chunk[1], scale)


def test_encoder_empty_column():
    assert E.encode(np.zeros(0), "gorilla") == O.encode(np.zeros(0), "gorilla")


def test_encoder_rejects_bad_arguments():
    with pytest.raises(E.InvalidArgument):
        E.encode(np.ones(4), 99)


@pytest.mark.parametrize("codec", ["uncompressed", "rle", "gorilla", "chimp", "chimp128", "elf_on_chimp", "elf", "buff"])
@pytest.mark.parametrize("chunk", [("record_count", 1000), ("byte_size", 3000), ("full", 0)])
def test_file_header_layout(codec, chunk):
    # FileHeader (format.rs:143-172), repr(C, packed(1)): magic [u8; 4], FileConfig
    # {field_type u8, compression_scheme u8, ChunkOption {kind u8, reserved u8,
    # value u64}}, footer_offset u64 (byte 16, encoder.rs:126-128), version [u16; 3]
    import struct
    v = gen("walk", 5003, 3)
    for data in (E.encode(v, codec, chunk, 1000 if codec == "buff" else 1),
                 O.encode(v, codec, {"record_count": 1, "byte_size": 2, "full": 0}[chunk[0]], chunk[1],
                          1000 if codec == "buff" else 1)):
        magic, ftype, scheme, kind, reserved, value, footer, v0, v1, v2 = struct.unpack_from("<4sBBBBQQHHH", data, 0)
        assert magic == b"EBI1" and ftype == 0 and reserved == 0
        assert scheme == E.SCHEMES[codec] and kind == {"full": 0, "record_count": 1, "byte_size": 2}[chunk[0]]
        assert value == (0 if chunk[0] == "full" else chunk[1])
        assert (v0, v1, v2) == (0, 1, 14)
        # FileFooter0 {number_of_records, number_of_chunks} at the footer offset
        nrec, nch = struct.unpack_from("<QQ", data, footer)
        assert nrec == len(v) and nch == O.Decoder(data).n_chunks
        # the chunks fill the bytes between the 30-byte header and the footer
        first_chunk, first_row = struct.unpack_from("<QQ", data, footer + 16)
        assert first_chunk == 30 and first_row == 0


def test_ctypes_structs_match_the_header(tmp_path):
    """Every ctypes mirror in ebi_gb300/_native.py has the size and field offsets
    of its C struct in include/ebi_gpu.h (compiled here with the host C compiler)."""
    import ctypes
    import shutil
    import subprocess
    from pathlib import Path

    from ebi_gb300 import _native as N

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    pairs = {"ebi_predicate": N.Predicate, "ebi_batch_query": N.BatchQuery, "ebi_batch_result": N.BatchResult,
             "ebi_batch_info": N.BatchInfo, "ebi_batch_trial": N.BatchTrial, "ebi_request": N.Request,
             "ebi_response": N.Response, "ebi_server_config": N.ServerConfig, "ebi_server_stats": N.ServerStats,
             "ebi_segment_times": N.SegmentTimes, "ebi_expr_node": N.ExprNode, "ebi_aggregation": N.Aggregation}
    lines = ['#include <stdio.h>', '#include "ebi_gpu.h"', "int main(void) {"]
    for cname, py in pairs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in py._fields_:
            lines.append(f'printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = Path(__file__).resolve().parent.parent / "include"
    subprocess.run([cc, "-std=c11", "-I", str(inc), str(src), "-o", str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        name, field, val = ln.split()
        got[(name, field)] = int(val)
    for cname, py in pairs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f in py._fields_:
            assert got[(cname, f[0])] == getattr(py, f[0]).offset, (cname, f[0])
