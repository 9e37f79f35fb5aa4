"""Elf and ElfOnChimp in the C oracle (CPU only).

lemolatoon/ebi's tests hold no Elf byte vectors: its Elf coverage is the
codec-generic filter / aggregation known-answer cases (tests/aggregation.rs,
tests/ml_query.rs list elf and elf_on_chimp), which test_oracle_kat.py runs
for these codecs too.  Here the oracle's Elf stream layout is pinned to two
vectors derived by hand from compressor/elf.rs, and its decoder to round
trips of its encoder over decimals of every digit count and magnitude
(lossless but for a quirk of the reference's power-of-ten test).
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from tests.test_cpu_abi import mixed_decimals


def bits_to_bytes(bits: str) -> bytes:
    bits = bits + "0" * (-len(bits) % 8)
    return bytes(int(bits[i:i + 8], 2) for i in range(0, len(bits), 8))


def test_elf_stream_of_one_value_kept_as_is():
    # 1.5 = 0x3FF8000000000000: beta* = 2, alpha = 1, erase = 52 - (F[1] + 0) = 48
    # bits, but the low 48 mantissa bits are already 0 (delta == 0): case '10'.
    # ElfXor first value: 7-bit trailing zeros (51), the 12 bits above bit 51.
    # close: '10', then NaN ^ 1.5 = 0x4000000000000000: lead 0, trail 62,
    # center 2 -> '10' + lead code 000 + center 0010, one payload bit, then a 0 bit.
    want = "10" + "0110011" + "001111111111" + "10" + "10" + "000" + "0010" + "0" + "0"
    assert O.encode_chunk([1.5], "elf") == bits_to_bytes(want)
    assert O.decode_chunk(bits_to_bytes(want), "elf").tolist() == [1.5]


def test_elf_stream_with_erased_bits_and_restore():
    # 3.14 = 0x40091EB851EB851F: sp 0, beta* 3, alpha 2, g = F[2] + 1 = 8, erase
    # 44 bits -> v' = 0x4009100000000000, case '11' + beta* (0b110011).
    # first value: trailing zeros 44 (0101100), then v' >> 45 in 19 bits.
    # second 3.14: same beta* -> '0'; same v' -> ElfXor '01'.
    # close: '10'; NaN ^ v' = 0x3FF1100000000000: lead 0, trail 44, center 20
    # -> '11' + 000 + 010100, then the 19 bits above the lowest set one, a 0 bit.
    want = ("110011" + "0101100" + format(0x4009100000000000 >> 45, "019b") + "0" + "01" + "10" + "11" + "000" +
            "010100" + format(0x3FF1100000000000 >> 45, "019b") + "0")
    assert O.encode_chunk([3.14, 3.14], "elf") == bits_to_bytes(want)
    assert O.decode_chunk(bits_to_bytes(want), "elf").tolist() == [3.14, 3.14]


def test_elf_on_chimp_stream_of_one_value():
    # '10' + 64 raw bits; close '10' + Chimp: NaN ^ 1.5 = 0x4000000000000000 has
    # 62 trailing zeros (> 6): '01' + lead code 000 + 6-bit significant (2) + 2 bits.
    want = "10" + format(0x3FF8000000000000, "064b") + "10" + "01" + "000" + "000010" + "01" + "0"
    assert O.encode_chunk([1.5], "elf_on_chimp") == bits_to_bytes(want)


def elf_columns():
    rng = np.random.default_rng(7)
    yield "decimals", mixed_decimals(rng, 20000)
    for d in range(0, 16):
        yield f"digits{d}", np.round(rng.normal(0, 100, 3000), d)
    yield "raw", rng.normal(0, 1, 3000)
    yield "powers", np.concatenate([10.0 ** np.arange(-323, 309), -(10.0 ** np.arange(-20, 20))])
    yield "near_powers", np.concatenate([np.nextafter(10.0 ** np.arange(-300, 300), 0),
                                         np.nextafter(10.0 ** np.arange(-300, 300), np.inf)])
    yield "large", np.round(rng.uniform(1e9, 1e15, 3000), 2)
    yield "tiny", np.round(rng.uniform(0, 1e-9, 3000), 15)
    yield "subnormal", 5e-324 * rng.integers(1, 1 << 50, 2000)
    yield "specials", np.array([0.0, -0.0, np.inf, -np.inf, 1.0, -1.0, 0.1, 1e-10, 1e9, 5e-324, 1.7976931348623157e308])
    yield "repeats", np.repeat(np.round(rng.normal(0, 10, 300), 3), 7)


def is_pow10(x: float) -> bool:
    a = abs(x)
    if not math.isfinite(a) or a == 0.0:
        return False
    k = math.floor(math.log10(a))
    return any(a == float(f"1e{j}") for j in (k - 1, k, k + 1))


@pytest.mark.parametrize("codec", ["elf", "elf_on_chimp"])
@pytest.mark.parametrize("name,values", list(elf_columns()), ids=lambda x: x if isinstance(x, str) else "")
def test_elf_round_trip(codec, name, values):
    """Lossless, except the reference's power-of-ten quirk: get_sp_and_10i_n_flag
    (compression_common/elf.rs:135-155) calls |x| an exact power of ten when
    log10(|x|) rounds to an integer, which outside [1e-10, 1e9) also holds for
    the doubles next to 10^k, and get_significant_count then starts its digit
    search from beta* = 0; such a value may come back as that power of ten."""
    v = np.asarray(values, dtype=np.float64)
    d = O.Decoder(O.encode(v, codec, O.CHUNK_RECORD_COUNT, 4096))
    out = d.materialize(None)
    assert len(out) == len(v)
    lossy = np.nonzero(out.view(np.uint64) != v.view(np.uint64))[0]
    for i in lossy:
        x, y = float(v[i]), float(out[i])
        assert is_pow10(y) and not is_pow10(x) and abs(y - x) <= 2 * math.ulp(x), (i, x, y)
    if name != "near_powers":
        assert len(lossy) <= len(v) // 50


@pytest.mark.parametrize("codec", ["elf", "elf_on_chimp"])
def test_elf_power_of_ten_flag_quirk(codec):
    # log10(9.999999999999999e-31) rounds to -30: the encoder flags the value
    # as a power of ten (beta* = 0) and the reader restores 10^-30.
    x = float(np.nextafter(1e-30, 0.0))
    assert math.log10(x) == -30.0
    out = O.decode_chunk(O.encode_chunk([0.78, x], codec), codec)
    assert out.tolist() == [0.78, 1e-30]


@pytest.mark.parametrize("codec", ["elf", "elf_on_chimp"])
def test_elf_nan_ends_the_chunk(codec):
    # the encoder writes NaN as the end marker's bits: the reader stops there
    v = np.array([1.25, 2.5, np.nan, 3.75])
    assert O.decode_chunk(O.encode_chunk(v, codec), codec).tolist() == [1.25, 2.5]


@pytest.mark.parametrize("codec", ["elf", "elf_on_chimp"])
def test_elf_truncated_chunk_is_unexpected_end(codec):
    stream = O.encode_chunk(np.round(np.linspace(0, 10, 50), 2), codec)
    with pytest.raises(O.OracleError) as e:
        O.decode_chunk(stream[: len(stream) // 2], codec)
    assert e.value.code == 3
