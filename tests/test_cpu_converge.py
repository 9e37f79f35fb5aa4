"""The XOR decoders' segment convergence (xor_dev.cuh converge_segments),
emulated on the host over the kernel's own record step (xor_parse.cuh compiled
for the host): on encoded Chimp, Chimp128, Elf and ElfOnChimp chunks, the
rounds end with every segment start on the reader's own record path, and the
segments' record counts add up to the records of the in-order parse."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import ebi_gb300 as E
from oracle import oracle as O

HERE = Path(__file__).resolve().parent
CODEC_ID = {"chimp": 4, "chimp128": 5, "elf_on_chimp": 6, "elf": 7}  # ebi_gpu.h scheme numbers


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("conv") / "converge_host"
    subprocess.run([cxx, "-O2", "-std=c++17", "-o", str(exe), str(HERE / "converge_host.cpp")],
                   check=True, capture_output=True)
    return exe


def series(kind, n, rng):
    i = np.arange(n)
    if kind == "sensor":
        return np.round(20 + 10 * np.sin(2 * np.pi * i / 1440) + rng.normal(0, 0.1, n), 4) + 0.0
    if kind == "walk":
        return np.round(30 + np.cumsum(rng.normal(0, 0.5, n)), 2) + 0.0
    return rng.choice([-2.5, 0.0, 1.0, 7.25, 1e300], n)  # repeats: ring copies


@pytest.mark.parametrize("codec", sorted(CODEC_ID))
@pytest.mark.parametrize("kind", ["sensor", "walk", "few"])
def test_rounds_reach_the_reader_path(harness, tmp_path, codec, kind):
    rng = np.random.default_rng(abs(hash((codec, kind))) % 2**32)
    data = bytes(E.encode(series(kind, 20_000, rng), codec, ("record_count", 8192)))
    d = O.Decoder(data)
    lines = []
    for c in range(d.n_chunks):
        phys, size, _, _ = d.chunk_info(c)
        p = tmp_path / f"c{c}.bin"
        p.write_bytes(data[phys:phys + size])
        for T in (256, 64):
            lines.append(f"{CODEC_ID[codec]} {T} {p}\n")
    out = subprocess.run([str(harness)], input="".join(lines), capture_output=True, text=True, check=True)
    rows = [list(map(int, ln.split())) for ln in out.stdout.strip().split("\n")]
    assert len(rows) == len(lines)
    for (records, total, off_path, rounds), ln in zip(rows, lines):
        assert off_path == 0 and total == records, (ln, records, total, off_path, rounds)
        assert records > 0
