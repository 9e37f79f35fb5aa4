"""The value-codec fold's fixed-point arithmetic (finalize.cuh), compiled for
the host: a fold of f64 terms equals the exact rational sum of the terms, each
truncated toward zero to a multiple of 2^(T - 1172) (T the largest exponent
field), rounded to nearest even; the 192-bit shift equals floor division.
Subnormals, overflow, ties and cancellation included."""
import math
import random
import shutil
import struct
import subprocess
from fractions import Fraction
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent


def bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def from_bits(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    exe = tmp_path_factory.mktemp("fold") / "fold_host"
    subprocess.run([nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a", "-o", str(exe), str(HERE / "fold_host.cu"), "-I", str(HERE.parent / "include")],
                   check=True, capture_output=True)
    return exe


def expected(vals):
    tops = [0 if not (bits(x) & (2**63 - 1)) else max((bits(x) >> 52) & 0x7FF, 1) for x in vals]
    T = max(tops)
    unit = Fraction(2) ** (T - 1172)
    total = Fraction(0)
    for x in vals:
        q = math.floor(abs(Fraction(x)) / unit)
        total += (q if x >= 0 else -q) * unit
    try:
        return float(total), T
    except OverflowError:
        return (math.inf if total > 0 else -math.inf), T


def cases():
    rng = random.Random(5)
    out = [[0.0], [-0.0, 0.0], [5e-324, -5e-324, 1.0], [1.7976931348623157e308] * 3,
           [1.0, 2.0 ** -53], [1.0, 3 * 2.0 ** -53], [1.0, 2.0 ** -53, 2.0 ** -110]]
    for _ in range(1500):
        n = rng.randint(1, 8)
        k = rng.random()
        if k < 0.3:
            out.append([rng.uniform(-1e3, 1e3) for _ in range(n)])
        elif k < 0.5:
            base = rng.uniform(-1, 1) * 10.0 ** rng.randint(-300, 300)
            out.append([base * rng.uniform(0.5, 2) * rng.choice([1, -1]) for _ in range(n)])
        elif k < 0.65:
            out.append([from_bits(rng.getrandbits(52) | (rng.getrandbits(1) << 63)) for _ in range(n)])
        elif k < 0.8:
            x = rng.uniform(1, 2) * 2.0 ** rng.randint(-1000, 1000)
            out.append([x, -x * (1 - 2.0 ** -52), x * 2.0 ** -rng.randint(40, 120)])
        else:
            out.append([rng.uniform(-1, 1) * 2.0 ** rng.randint(-1074, 1023) for _ in range(n)])
    return out


def test_fold_matches_exact_rounding(harness):
    cs = cases()
    inp = "".join(f"s {len(v)} " + " ".join(f"{bits(x):x}" for x in v) + "\n" for v in cs)
    lines = subprocess.run([str(harness)], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    for v, line in zip(cs, lines):
        got, T = line.split()
        want, wT = expected(v)
        assert int(T) == wT, v
        g = from_bits(int(got, 16))
        assert g == want and math.copysign(1, g) == math.copysign(1, want) or (g == 0 and want == 0), (v, g, want)


def test_shift_is_floor_division(harness):
    rng = random.Random(7)
    inp, want = [], []
    for _ in range(1000):
        w = rng.getrandbits(192)
        n = rng.choice([0, 1, 63, 64, 65, 127, 128, 129, 191, 192, 500, rng.randint(0, 200)])
        sw = w - (1 << 192) if w >> 191 else w
        r = (sw >> n) % (1 << 192)
        inp.append(f"r {w & (2**64 - 1):x} {(w >> 64) & (2**64 - 1):x} {w >> 128:x} {n}\n")
        want.append(f"{r & (2**64 - 1):016x} {(r >> 64) & (2**64 - 1):016x} {r >> 128:016x}")
    out = subprocess.run([str(harness)], input="".join(inp), capture_output=True, text=True, check=True).stdout.split("\n")
    assert out[: len(want)] == want
