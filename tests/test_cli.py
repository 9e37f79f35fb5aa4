"""The experimenter-shaped command line (ebi_gb300/cli.py): result strings,
serde config formats, EBI1 metadata and the output layout on the CPU; the
query commands on the GPU against the oracle."""
import json

import numpy as np
import pytest

import ebi_gb300 as E
from ebi_gb300 import cli
from oracle import oracle as O
from tests.kat import round_at


# ---- CPU ------------------------------------------------------------------------------------------
@pytest.mark.parametrize("x,want", [
    (1.0, "1"), (-0.0, "-0"), (0.0, "0"), (1.5, "1.5"), (0.1 + 0.2, "0.30000000000000004"),
    (1e21, "1000000000000000000000"), (1.5e-7, "0.00000015"), (-123.25, "-123.25"),
    (float("nan"), "NaN"), (float("inf"), "inf"), (float("-inf"), "-inf"),
    (2.0 ** 70, "1180591620717411300000"), (5e-324, "0." + "0" * 323 + "5"),
])
def test_rust_f64_display(x, want):
    assert cli.rust_f64(x) == want


def test_bitmap_string():
    assert cli.bitmap_string(np.array([], np.uint32)) == "RoaringBitmap<[]>"
    assert cli.bitmap_string(np.array([1, 5, 9], np.uint32)) == "RoaringBitmap<[1, 5, 9]>"
    assert cli.bitmap_string(np.arange(15, dtype=np.uint32)).startswith("RoaringBitmap<[0, 1,")
    assert cli.bitmap_string(np.arange(3, 103, dtype=np.uint32)) == "RoaringBitmap<100 values between 3 and 102>"


def test_predicate_json():
    p = cli.predicate_from_json({"type": "Range", "predicate": {"start": {"Inclusive": 1.5}, "end": "None"}})
    assert p == E.Predicate.range(E.RangeValue.inclusive(1.5), E.RangeValue.NONE)
    p = cli.predicate_from_json({"type": "Range", "predicate": {"start": "None", "end": {"Exclusive": -2}}})
    assert p == E.Predicate.range(E.RangeValue.NONE, E.RangeValue.exclusive(-2.0))
    assert cli.predicate_from_json({"type": "Eq", "predicate": 3}) == E.Predicate.eq(3.0)
    assert cli.predicate_from_json({"type": "Ne", "predicate": 0.5}) == E.Predicate.ne(0.5)
    with pytest.raises(ValueError):
        cli.predicate_from_json({"type": "Like", "predicate": 1})


@pytest.mark.parametrize("scheme,chunk,scale", [
    ("buff", ("record_count", 100), 1000), ("gorilla", ("full", 0), 1), ("rle", ("byte_size", 256), 1),
    ("elf", ("record_count", 64), 1),
])
def test_file_info_matches_oracle(tmp_path, scheme, chunk, scale):
    v = np.round(np.random.default_rng(3).normal(50, 10, 1000), 3)
    data = E.encode(v, scheme, chunk, scale)
    info = cli.file_info(data=data)
    p = tmp_path / "x.ebi"
    p.write_bytes(data)
    assert cli.file_info(path=str(p)) == info
    with O.Decoder(data) as d:
        assert info["n_records"] == d.n_records == 1000
        assert info["n_chunks"] == d.n_chunks
        assert info["scheme"] == d.scheme == E.SCHEMES[scheme]
        assert info["chunk_bytes"] == sum(d.chunk_info(i)[1] for i in range(d.n_chunks))
    cfg = cli.compression_config(info)
    want_chunk = {"full": "Full", "record_count": {"RecordCount": chunk[1]},
                  "byte_size": {"ByteSizeBestEffort": chunk[1]}}[chunk[0]]
    assert cfg["chunk_option"] == want_chunk
    assert cfg["compressor_config"] == ({"type": "BUFF", "scale": scale} if scheme == "buff" else
                                        {"type": cli.SCHEME_NAMES[E.SCHEMES[scheme]], "capacity": 8192})


def test_compress_command(tmp_path):
    data_dir = tmp_path / "data"
    data_dir.mkdir()
    v = np.round(np.random.default_rng(0).uniform(-100, 100, 5000), 2)
    v.tofile(data_dir / "a.bin")
    (data_dir / "b.bin").write_bytes(v[:777].tobytes())
    cfg = tmp_path / "buff.json"
    cfg.write_text(json.dumps({"chunk_option": {"RecordCount": 1024},
                               "compressor_config": {"type": "BUFF", "scale": 100}}))
    assert cli.main(["-i", str(data_dir / "*.bin"), "compress", "-c", str(cfg)]) == 0
    for stem, n in (("a", 5000), ("b", 777)):
        enc = (data_dir / f"{stem}.ebi").read_bytes()
        assert enc == E.encode(v[:n], "buff", ("record_count", 1024), 100)
        with O.Decoder(enc) as d:
            assert np.array_equal(round_at(d.materialize(), 100), v[:n])  # BUFF keeps 2 decimals
        out = json.loads((tmp_path / "result" / stem / "compress" / "000.json").read_text())
        assert out["result_string"] == f"number_of_records: {n}"
        assert out["compression_config"] == json.loads(cfg.read_text())
        st = out["command_specific"]
        assert st["uncompressed_size"] == 8 * n and st["compressed_size"] == len(enc)
        assert st["compression_ratio"] == len(enc) / (8 * n)
        assert set(out) == {"in_memory", "version", "config_path", "compression_config", "command_specific",
                            "elapsed_time_nanos", "execution_times", "input_filename", "datetime", "result_string"}
        assert set(out["execution_times"]) == set(cli.SEGMENTS)
    # a second run numbers its output 001
    assert cli.main(["-i", str(data_dir / "a.bin"), "compress", "-c", str(cfg)]) == 0
    assert (tmp_path / "result" / "a" / "compress" / "001.json").exists()


def test_compress_capacity_kept(tmp_path):
    v = np.arange(100, dtype=np.float64)
    v.tofile(tmp_path / "c.bin")
    cfg = tmp_path / "g.json"
    cfg.write_text(json.dumps({"chunk_option": "Full", "compressor_config": {"type": "Gorilla", "capacity": 4096}}))
    assert cli.main(["-i", str(tmp_path / "c.bin"), "compress", "-c", str(cfg)]) == 0
    info = cli.file_info(path=str(tmp_path / "c.ebi"))
    assert info["config_value"] == 4096 and info["scheme"] == E.SCHEMES["gorilla"]


def test_missing_input_is_reported(tmp_path, capsys):
    cfg = tmp_path / "g.json"
    cfg.write_text(json.dumps({"chunk_option": "Full", "compressor_config": {"type": "Gorilla", "capacity": 8}}))
    (tmp_path / "dir.bin").mkdir()
    assert cli.main(["-i", str(tmp_path / "*.bin"), "compress", "-c", str(cfg)]) == 0
    assert "Skipping directory" in capsys.readouterr().err


# ---- GPU ------------------------------------------------------------------------------------------
def _expected(data, command, cfg):
    with O.Decoder(data) as d:
        mask = O.mask_from_rows(cfg["bitmask"], d.n_records) if cfg.get("bitmask") is not None else None
        cid = cfg.get("chunk_id")
        pred = None
        if "predicate" in cfg:
            p = cfg["predicate"]
            if p["type"] == "Eq":
                pred = O.eq(p["predicate"])
            else:
                r = p["predicate"]

                def b(x):
                    if x == "None":
                        return O.BOUND_NONE, 0.0
                    (k, v), = x.items()
                    return (O.BOUND_INCLUSIVE if k == "Inclusive" else O.BOUND_EXCLUSIVE), float(v)

                (sk, sv), (ek, ev) = b(r["start"]), b(r["end"])
                pred = O.rng(sk, sv, ek, ev)
        if command == "filter":
            return cli.bitmap_string(np.asarray(O.rows_from_mask(d.filter(pred, mask, cid), d.n_records), np.uint32))
        if command == "filter-materialize":
            return f"bytes: {8 * len(d.filter_materialize(pred, mask, cid))}"
        if command == "materialize":
            return f"bytes: {8 * len(d.materialize(mask, cid))}"
        return cli.rust_f64(d.max(mask, cid) if command == "max" else d.sum(mask, cid))


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", ["buff", "gorilla", "chimp128", "rle", "elf"])
@pytest.mark.parametrize("in_memory", [True, False])
def test_query_commands(tmp_path, scheme, in_memory):
    rng = np.random.default_rng(11)
    v = np.round(rng.normal(20, 5, 20000), 2)
    if scheme == "rle":
        v = np.repeat(v[:400], 50)
    data = E.encode(v, scheme, ("record_count", 4096), 100)
    d_dir = tmp_path / "data"
    d_dir.mkdir()
    (d_dir / "col.ebi").write_bytes(data)
    rows = sorted(rng.choice(len(v), 3000, replace=False).tolist())
    cases = [
        ("filter", {"predicate": {"type": "Range", "predicate": {"start": {"Inclusive": 18.0},
                                                                  "end": {"Exclusive": 22.5}}},
                    "chunk_id": None, "bitmask": None}),
        ("filter", {"predicate": {"type": "Eq", "predicate": float(v[7])}, "chunk_id": 0, "bitmask": None}),
        ("filter-materialize", {"predicate": {"type": "Range", "predicate": {"start": "None",
                                                                              "end": {"Inclusive": 15.0}}},
                                "chunk_id": None, "bitmask": rows}),
        ("materialize", {"chunk_id": 2, "bitmask": None}),
        ("max", {"chunk_id": None, "bitmask": rows}),
        ("sum", {"chunk_id": None, "bitmask": None}),
    ]
    for k, (command, cfg) in enumerate(cases):
        cpath = tmp_path / f"cfg{k}.json"
        cpath.write_text(json.dumps(cfg))
        argv = ["-i", str(d_dir / "col.ebi"), command, "-c", str(cpath), "--in-memory", str(in_memory).lower()]
        assert cli.main(argv) == 0
        outs = sorted((tmp_path / "result" / "col" / cli.COMMAND_DIRS[command]).glob("*.json"))
        out = json.loads(outs[-1].read_text())
        want = _expected(data, command, cfg)
        if command == "sum" and scheme != "buff":
            got = float(out["result_string"])
            assert abs(got - float(want)) <= 1e-12 * abs(float(want)), (got, want)
        else:
            assert out["result_string"] == want, (command, cfg)
        assert out["in_memory"] is in_memory and out["command_specific"] == cfg
        assert out["compression_config"]["compressor_config"]["type"] == cli.SCHEME_NAMES[E.SCHEMES[scheme]]
        t = out["execution_times"]
        seg = cli.DECODE_SEGMENT.get(E.SCHEMES[scheme], "xor_nanos")
        assert t[seg] > 0 and out["elapsed_time_nanos"] > 0
        assert (t["io_read_nanos"] > 0) == (not in_memory)
        if command in cli.OUTPUT_SUFFIX and not in_memory:
            written = np.fromfile(d_dir / ("col" + cli.OUTPUT_SUFFIX[command]), dtype=np.float64)
            assert out["result_string"] == f"bytes: {written.nbytes}"


@pytest.mark.gpu
def test_decoder_from_file_equals_bytes(tmp_path):
    v = np.round(np.random.default_rng(5).uniform(0, 1000, 300_000), 3)
    for scheme in ("buff", "chimp", "uncompressed"):
        data = E.encode(v, scheme, ("record_count", 65536), 1000)
        p = tmp_path / f"{scheme}.ebi"
        p.write_bytes(data)
        a, b = E.Decoder(data), E.Decoder.from_file(str(p))
        try:
            assert (a.n_records, a.n_chunks, a.scheme) == (b.n_records, b.n_chunks, b.scheme)
            assert np.array_equal(a.materialize().cpu().numpy(), b.materialize().cpu().numpy())
            pred = E.Predicate.range(E.RangeValue.inclusive(100), E.RangeValue.exclusive(700))
            assert np.array_equal(a.filter(pred).cpu().numpy(), b.filter(pred).cpu().numpy())
            assert a.sum() == b.sum()
        finally:
            a.close()
            b.close()
    with pytest.raises(E.DecoderError):
        E.Decoder.from_file(str(tmp_path / "missing.ebi"))
