"""The warp-per-chunk XOR decode (ebi_gb300/csrc/xor_lanes.h) emulated lane by
lane on the host, against the sequential reader built from the same record
parser and against the oracle's decoder.

For Chimp, Chimp128, Elf and ElfOnChimp chunks, intact and corrupted (flipped
bits, truncated bytes, NaN values inside the data), and of every size from one
value to tens of thousands: the 32-lane algorithm (segment parse rounds, XOR
scan or Chimp128 ring composition, end-marker pass and value pass; also the
single-pass form, and 64-bit positions) returns the same status and the same
values, Elf flags and beta* as the reader's own loop (whose record parser is
not the branch-free one the lanes use for Chimp and Chimp128), and that
loop's values equal the oracle's decoder for the non-Elf codecs.
"""
import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
BUILD = HERE / "_build"
SRC = HERE / "xor_lanes_emu.cpp"
CSRC = ROOT / "ebi_gb300" / "csrc"

CODECS = ["chimp", "chimp128", "elf_on_chimp", "elf"]


def emu_lib():
    BUILD.mkdir(exist_ok=True)
    lib = BUILD / "libxor_lanes_emu.so"
    deps = [SRC, CSRC / "xor_lanes.h", CSRC / "xor_parse.cuh", CSRC / "elf_dev.cuh"]
    if not lib.exists() or lib.stat().st_mtime < max(p.stat().st_mtime for p in deps):
        tmp = lib.with_suffix(f".{os.getpid()}.tmp")
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", str(CSRC), "-o", str(tmp), str(SRC)],
                       check=True)
        os.replace(tmp, lib)
    L = C.CDLL(str(lib))
    L.emu_decode.restype = C.c_uint32
    L.emu_decode.argtypes = [C.c_int, C.c_int, C.c_char_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p,
                             C.c_uint64, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]
    return L


_LIB = None


def decode(which, codec, chunk):
    global _LIB
    if _LIB is None:
        _LIB = emu_lib()
    cap = 8 * len(chunk) + 64
    v = np.zeros(cap, dtype=np.uint64)
    m = np.zeros(cap, dtype=np.uint8)
    b = np.zeros(cap, dtype=np.int32)
    n = C.c_uint64()
    r = C.c_uint32()
    st = _LIB.emu_decode(which, O.SCHEMES[codec], chunk, len(chunk), v.ctypes.data, m.ctypes.data, b.ctypes.data,
                         cap, C.byref(n), C.byref(r))
    k = min(n.value, cap)
    return st, v[:k].copy(), m[:k].copy(), b[:k].copy(), r.value


def series(rng, kind, n):
    i = np.arange(n)
    if kind == "walk":
        return np.round(30 + np.cumsum(rng.normal(0, 0.5, n)), 2) + 0.0
    if kind == "sensor":
        return np.round(20 + 10 * np.sin(2 * np.pi * i / 1440) + rng.normal(0, 0.1, n), 4) + 0.0
    if kind == "few":  # repeats and copies from the ring
        return rng.choice([-2.5, 0.0, 1.0, 7.25, 1e300, 3.141592653589793], n)
    if kind == "uniform":
        return rng.uniform(-1e6, 1e6, n)
    if kind == "const":
        return np.full(n, 42.125)
    if kind == "nan_inside":
        v = np.round(rng.normal(10, 3, n), 2)
        v[n // 3] = np.nan
        return v
    raise ValueError(kind)


def check(codec, chunk, expect_n=None):
    s0, v0, m0, b0, _ = decode(0, codec, chunk)
    for which in (1, 2, 3):
        s, v, m, b, rounds = decode(which, codec, chunk)
        assert s == s0, (codec, which, s, s0)
        if s0 == 0:
            assert np.array_equal(v, v0), (codec, which, len(v), len(v0))
            assert np.array_equal(m, m0) and np.array_equal(b, b0), (codec, which)
    if s0 == 0 and codec in ("chimp", "chimp128"):
        want = O.decode_chunk(chunk, codec)
        assert np.array_equal(v0, want.view(np.uint64)), (codec, len(v0), len(want))
    if expect_n is not None and s0 == 0:
        assert len(v0) == expect_n
    return s0


@pytest.mark.parametrize("codec", CODECS)
@pytest.mark.parametrize("kind", ["walk", "sensor", "few", "uniform", "const", "nan_inside"])
def test_warp_split_equals_reader(codec, kind):
    rng = np.random.default_rng(abs(hash((codec, kind))) % 2**32)
    for n in (1, 2, 3, 5, 17, 31, 32, 33, 64, 100, 257, 1000, 8192, 30011):
        v = series(rng, kind, n)
        chunk = O.encode_chunk(v, codec)
        stop = int(np.argmax(np.isnan(v))) if np.isnan(v).any() else n
        check(codec, chunk, expect_n=stop)


@pytest.mark.parametrize("codec", CODECS)
def test_warp_split_corrupt_chunks(codec):
    rng = np.random.default_rng(abs(hash((codec, "corrupt"))) % 2**32)
    statuses = set()
    for trial in range(150):
        n = int(rng.choice([40, 300, 2000, 8192]))
        v = series(rng, ["walk", "sensor", "few"][trial % 3], n)
        chunk = bytearray(O.encode_chunk(v, codec))
        if trial % 5 == 4:
            chunk = chunk[: int(rng.integers(1, len(chunk)))]  # truncated
        else:
            for _ in range(1 + trial % 4):
                k = int(rng.integers(len(chunk)))
                chunk[k] ^= 1 << int(rng.integers(8))
        statuses.add(check(codec, bytes(chunk)))
    assert len(statuses) >= 2  # both intact-looking and failing chunks were exercised


def test_rounds_stay_few_on_bench_series():
    # the segment parse converges in a couple of rounds on the benchmark's sensor series
    rng = np.random.default_rng(3)
    for codec in CODECS:
        rounds = []
        for _ in range(8):
            v = series(rng, "sensor", 8192)
            s, _, _, _, r = decode(1, codec, O.encode_chunk(v, codec))
            assert s == 0
            rounds.append(r)
        assert max(rounds) <= 3, (codec, rounds)
