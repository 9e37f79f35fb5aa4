"""Aggregation / Expr over several columns (api/decoder.rs:755-917,
decoder/expr.rs): the oracle against the reference's fixed cases and a plain
Python model of the chunk loop (CPU); the engine against both (GPU)."""
import math

import numpy as np
import pytest

import ebi_gb300 as E
from oracle import oracle as O
from tests.kat import KAT
from tests.parity import same_f64, same_scalar, sum_ok

KIND = {"sum": O.AGGR_SUM, "min": O.AGGR_MIN, "max": O.AGGR_MAX, "none": O.AGGR_NONE}
OPS = {"add": E.Op.Add, "sub": E.Op.Sub, "mul": E.Op.Mul, "div": E.Op.Div}


def to_expr(j):
    if j[0] == "index":
        return E.Expr.Index(j[1])
    if j[0] == "lit":
        return E.Expr.Literal(j[1])
    return E.Expr.Binary(OPS[j[0]], to_expr(j[1]), to_expr(j[2]))


def oracle_decoders(columns, chunk=("record_count", 3), scheme=O.UNCOMPRESSED, scale=1):
    kinds = {"record_count": O.CHUNK_RECORD_COUNT, "byte_size": O.CHUNK_BYTE_SIZE, "full": O.CHUNK_FULL}
    return [O.Decoder(O.encode(np.asarray(c, float), scheme, kinds[chunk[0]], chunk[1], scale)) for c in columns]


# ---- a plain model of Aggregation::compute (no codec: values and chunk row counts) ----
def model(columns, chunk_rows, expr, kind, rows=None):
    """columns[j]: values; chunk_rows[j]: rows per chunk of column j."""
    sel = None if rows is None else set(rows)

    def chunk_vals(j, c):
        r0 = sum(chunk_rows[j][:c])
        return [columns[j][r] for r in range(r0, r0 + chunk_rows[j][c]) if sel is None or r in sel]

    def ev(e, c):
        if e.kind == "index":
            return chunk_vals(e.index, c)
        if e.kind == "literal":
            raise ValueError("precondition")
        lit_l, lit_r = e.lhs.kind == "literal", e.rhs.kind == "literal"
        f = {E.Op.Add: lambda a, b: a + b, E.Op.Sub: lambda a, b: a - b, E.Op.Mul: lambda a, b: a * b,
             E.Op.Div: lambda a, b: a / b if b != 0 else (math.copysign(math.inf, a) * math.copysign(1, b)
                                                          if a != 0 and a == a else math.nan)}[e.op]
        if lit_l and lit_r:
            raise ValueError("precondition")
        if lit_r:
            return [f(x, e.rhs.value) for x in ev(e.lhs, c)]
        if lit_l:
            return [f(e.lhs.value, x) for x in ev(e.rhs, c)]
        return [f(a, b) for a, b in zip(ev(e.lhs, c), ev(e.rhs, c))]

    out = [] if kind == O.AGGR_NONE else (0.0 if kind == O.AGGR_SUM else math.inf if kind == O.AGGR_MIN else -math.inf)
    for c in range(len(chunk_rows[0])):
        v = ev(expr, c)
        if kind == O.AGGR_NONE:
            out += v
        elif kind == O.AGGR_SUM:
            s = -0.0
            for x in v:
                s += x
            out += s
        else:
            for x in v:
                if x == x:
                    out = min(out, x) if kind == O.AGGR_MIN else max(out, x)
    return out


def chunk_rows_of(n, k):
    return [min(k, n - r) for r in range(0, n, k)]


# ---- CPU: the oracle --------------------------------------------------------------------
@pytest.mark.parametrize("idx", range(len(KAT["expr_cases"])))
def test_oracle_expr_kats(idx):
    case = KAT["expr_cases"][idx]
    ds = oracle_decoders(case["columns"], tuple(KAT["expr_chunk"]))
    n = max(len(c) for c in case["columns"])
    mask = O.mask_from_rows(case["bitmask"], n) if "bitmask" in case else None
    for agg in case["aggs"]:
        got = O.aggregate(ds, KIND[agg["kind"]], to_expr(agg["expr"]).postfix(), mask)
        assert got == agg["expect"], (case["src"], agg)


EXPRS = [
    E.Expr.Index(0) * E.Expr.Index(1),
    E.Expr.Index(0) * (1.0 - E.Expr.Index(1)),
    (E.Expr.Index(0) * (1.0 - E.Expr.Index(1))) * (1.0 + E.Expr.Index(2)),
    (E.Expr.Index(0) + E.Expr.Index(1)) * (E.Expr.Index(1) - E.Expr.Index(2)),
    2.0 / E.Expr.Index(2),
    E.Expr.Index(1) - E.Expr.Index(0) / 3.0,
]


@pytest.mark.parametrize("ei", range(len(EXPRS)))
@pytest.mark.parametrize("kind", [O.AGGR_SUM, O.AGGR_MIN, O.AGGR_MAX, O.AGGR_NONE])
def test_oracle_matches_model_misaligned_chunks(ei, kind):
    rng = np.random.default_rng(40 + ei)
    n = 300
    cols = [np.round(rng.normal(0, 3, n), 2).tolist() for _ in range(3)]
    cols[2][5] = 0.0  # a division by zero
    ks = [32, 25, 40]  # chunk sizes differ: chunk i of each column covers other rows
    ds = [O.Decoder(O.encode(np.asarray(c), O.UNCOMPRESSED, O.CHUNK_RECORD_COUNT, k)) for c, k in zip(cols, ks)]
    ds = [ds[2], ds[0], ds[1]]  # the first column has the fewest chunks (40 rows each)
    cols = [cols[2], cols[0], cols[1]]
    crs = [chunk_rows_of(n, 40), chunk_rows_of(n, 32), chunk_rows_of(n, 25)]
    rows = sorted(rng.choice(n, 120, replace=False).tolist())
    for mask_rows in (None, rows):
        mask = None if mask_rows is None else O.mask_from_rows(mask_rows, n)
        got = O.aggregate(ds, kind, EXPRS[ei].postfix(), mask)
        want = model(cols, crs, EXPRS[ei], kind, mask_rows)
        if kind == O.AGGR_NONE:
            assert same_f64(np.nan_to_num(got, nan=7.5), np.nan_to_num(np.asarray(want, float), nan=7.5))
        else:
            assert same_scalar(got, want) or (np.isnan(got) and np.isnan(want)), (got, want)


def test_oracle_expr_errors():
    ds = oracle_decoders([[1.0, 2.0, 3.0, 4.0], [5.0, 6.0, 7.0, 8.0]])
    lit = [(O.EXPR_LITERAL, 0, 1.0)]
    with pytest.raises(O.OracleError) as e:
        O.aggregate(ds, O.AGGR_SUM, lit)
    assert e.value.code == 4  # PreconditionsNotMet
    with pytest.raises(O.OracleError) as e:
        O.aggregate(ds, O.AGGR_SUM, (E.Expr.Index(0) + (E.Expr.Literal(1) * E.Expr.Literal(2))).postfix())
    assert e.value.code == 4
    with pytest.raises(O.OracleError) as e:
        O.aggregate(ds, O.AGGR_SUM, (E.Expr.Index(0) + E.Expr.Index(2)).postfix())
    assert e.value.code == 7  # index past the decoders: the reference panics
    with pytest.raises(O.OracleError) as e:
        O.aggregate(ds, O.AGGR_NONE, E.Expr.Index(0).postfix())
    assert e.value.code == 7  # todo!() in the reference
    short = oracle_decoders([[1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0], [1.0, 2.0]])
    with pytest.raises(O.OracleError) as e:
        O.aggregate(short, O.AGGR_SUM, (E.Expr.Index(0) * E.Expr.Index(1)).postfix())
    assert e.value.code == 7  # chunk_handles[i] out of range: the reference panics
    # more chunks in a later column: only the first column's chunk count is visited
    longer = oracle_decoders([[1.0, 2.0, 3.0], [1.0, 2.0, 3.0, 4.0, 5.0]])
    assert O.aggregate(longer, O.AGGR_SUM, (E.Expr.Index(0) * E.Expr.Index(1)).postfix()) == 14.0


# ---- GPU: the engine ------------------------------------------------------------------
def engine_decoders(columns, chunk=("record_count", 3), scheme="uncompressed", scale=1):
    return [E.Decoder(E.encode(np.asarray(c, float), scheme, chunk, scale)) for c in columns]


@pytest.mark.gpu
@pytest.mark.parametrize("idx", range(len(KAT["expr_cases"])))
def test_engine_expr_kats(idx):
    case = KAT["expr_cases"][idx]
    ds = engine_decoders(case["columns"], tuple(KAT["expr_chunk"]))
    n = max(len(c) for c in case["columns"])
    mask = O.mask_from_rows(case["bitmask"], n) if "bitmask" in case else None
    aggs = [E.Aggregation(KIND[a["kind"]], to_expr(a["expr"])) for a in case["aggs"]]
    got = E.Aggregation.compute_multiple(aggs, ds, mask)
    assert got == [a["expect"] for a in case["aggs"]], case["src"]
    for a, g in zip(aggs, got):  # Aggregation::compute gives the same
        assert a.compute(ds, mask) == g


def expr_sum_ok(g: float, o: float, vals) -> bool:
    """An expression sum: within 1e-12 of the reference's per-chunk sequential
    sums relative to the sum of magnitudes, and within 16 eps of the exact sum
    relative to it (each thread sums 8 or 16 values, compensated above that)."""
    vals = np.asarray(vals, dtype=np.float64)
    if not np.all(np.isfinite(vals)) or not math.isfinite(o):
        return same_scalar(g, o)
    mag = max(float(np.abs(vals).sum()), abs(o), 1e-300)
    exact = math.fsum(vals.tolist())
    return abs(g - o) <= 1e-12 * mag and abs(g - exact) <= 16 * np.finfo(float).eps * mag


def _check_engine(ds_e, ds_o, expr, kind, mask):
    got = E.Aggregation(kind, expr).compute(ds_e, mask)
    want = O.aggregate(ds_o, kind, expr.postfix(), mask)
    if kind == O.AGGR_NONE:
        g = got.cpu().numpy()
        assert g.shape == want.shape
        assert same_f64(np.where(np.isnan(g), 0.5, g), np.where(np.isnan(want), 0.5, want))
    elif kind == O.AGGR_SUM:
        vals = O.aggregate(ds_o, O.AGGR_NONE, expr.postfix(), mask)
        assert expr_sum_ok(got, want, vals), (got, want)
    else:
        assert same_scalar(got, want), (got, want)


CODEC_CASES = [("buff", 100), ("gorilla", 1), ("chimp", 1), ("chimp128", 1), ("rle", 1), ("uncompressed", 1),
               ("elf", 1), ("elf_on_chimp", 1)]


@pytest.mark.gpu
@pytest.mark.parametrize("scheme,scale", CODEC_CASES)
def test_engine_expr_parity(scheme, scale):
    rng = np.random.default_rng(7)
    n = 70_000
    cols = [np.round(rng.uniform(900, 105000, n), 2), np.round(rng.integers(0, 11, n) / 100.0, 2),
            np.round(rng.integers(0, 9, n) / 100.0, 2)]
    if scheme == "rle":
        cols = [np.repeat(c[: n // 40], 40) for c in cols]
    ds_o = [O.Decoder(O.encode(c, O.SCHEMES[scheme], O.CHUNK_RECORD_COUNT, 8192, scale)) for c in cols]
    ds_e = [E.Decoder(E.encode(c, scheme, ("record_count", 8192), scale)) for c in cols]
    rows = np.sort(rng.choice(n, n // 3, replace=False))
    for mask in (None, O.mask_from_rows(rows.tolist(), n)):
        for expr in EXPRS:
            for kind in (O.AGGR_SUM, O.AGGR_MIN, O.AGGR_MAX, O.AGGR_NONE):
                _check_engine(ds_e, ds_o, expr, kind, mask)


@pytest.mark.gpu
def test_engine_misaligned_chunks_and_mixed_codecs():
    rng = np.random.default_rng(9)
    n = 50_000
    cols = [np.round(rng.normal(10, 4, n), 2) for _ in range(3)]
    specs = [("buff", 5000, 100), ("gorilla", 3000, 1), ("chimp128", 4096, 1)]
    ds_o = [O.Decoder(O.encode(c, O.SCHEMES[s], O.CHUNK_RECORD_COUNT, k, sc)) for c, (s, k, sc) in zip(cols, specs)]
    ds_e = [E.Decoder(E.encode(c, s, ("record_count", k), sc)) for c, (s, k, sc) in zip(cols, specs)]
    rows = np.sort(rng.choice(n, 20_000, replace=False))
    for mask in (None, O.mask_from_rows(rows.tolist(), n)):
        for expr in EXPRS:
            for kind in (O.AGGR_SUM, O.AGGR_MIN, O.AGGR_MAX, O.AGGR_NONE):
                _check_engine(ds_e, ds_o, expr, kind, mask)
    # compute_multiple: Index aggregations first, then the expressions in one pass
    aggs = [E.Aggregation.sum(E.Expr.Index(0)), E.Aggregation.max(EXPRS[2]), E.Aggregation.sum(EXPRS[3]),
            E.Aggregation.min(E.Expr.Index(1)), E.Aggregation.none(EXPRS[0])]
    got = E.Aggregation.compute_multiple(aggs, ds_e)
    for a, g in zip(aggs, got):
        one = a.compute(ds_e)
        if a.kind == E.AggregationKind.NONE:
            assert same_f64(g.cpu().numpy(), one.cpu().numpy())
        else:
            assert same_scalar(g, one)


@pytest.mark.gpu
def test_engine_expr_errors():
    ds = engine_decoders([[1.0, 2.0, 3.0, 4.0], [5.0, 6.0, 7.0, 8.0]])
    with pytest.raises(E.PreconditionsNotMet):
        E.Aggregation.sum(E.Expr.Literal(1.0)).compute(ds)
    with pytest.raises(E.PreconditionsNotMet):
        E.Aggregation.sum(E.Expr.Index(0) + (E.Expr.Literal(1) * E.Expr.Literal(2))).compute(ds)
    with pytest.raises(E.InvalidArgument):
        E.Aggregation.sum(E.Expr.Index(0) + E.Expr.Index(2)).compute(ds)
    with pytest.raises(E.Unsupported):
        E.Aggregation.none(E.Expr.Index(0)).compute(ds)
    short = engine_decoders([[1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0], [1.0, 2.0]])
    with pytest.raises(E.InvalidArgument):
        E.Aggregation.sum(E.Expr.Index(0) * E.Expr.Index(1)).compute(short)
    longer = engine_decoders([[1.0, 2.0, 3.0], [1.0, 2.0, 3.0, 4.0, 5.0]])
    assert E.Aggregation.sum(E.Expr.Index(0) * E.Expr.Index(1)).compute(longer) == 14.0


@pytest.mark.gpu
def test_tpch_q6_and_q1_shapes():
    """experimenter/src/tpch.rs:190-461: Q6 filters l_discount, then l_quantity
    under that mask, then sums l_extendedprice * l_discount; Q1 runs five
    aggregations with compute_multiple."""
    rng = np.random.default_rng(6)
    n = 300_000
    price = np.round(rng.uniform(900, 105000, n), 2)
    disc = np.round(rng.integers(0, 11, n) / 100.0, 2)
    qty = rng.integers(1, 51, n).astype(float)
    tax = np.round(rng.integers(0, 9, n) / 100.0, 2)
    cols = [qty, price, disc, tax]
    ds_o = [O.Decoder(O.encode(c, O.BUFF, O.CHUNK_RECORD_COUNT, 65536, 100)) for c in cols]
    ds_e = [E.Decoder(E.encode(c, "buff", ("record_count", 65536), 100)) for c in cols]
    # Q6
    p0 = E.Predicate.range(E.RangeValue.inclusive(0.05), E.RangeValue.inclusive(0.07))
    p1 = E.Predicate.range(E.RangeValue.NONE, E.RangeValue.exclusive(24.0))
    m = ds_e[2].filter(p0)
    m = ds_e[0].filter(p1, m)
    o0 = ds_o[2].filter(O.rng(O.BOUND_INCLUSIVE, 0.05, O.BOUND_INCLUSIVE, 0.07))
    o1 = ds_o[0].filter(O.rng(O.BOUND_NONE, 0.0, O.BOUND_EXCLUSIVE, 24.0), o0)
    assert same_f64(m.cpu().numpy().view(np.uint64)[: len(o1)], o1)
    q6 = E.Expr.Index(1) * E.Expr.Index(2)
    got = E.Aggregation.sum(q6).compute(ds_e, m)
    want = O.aggregate(ds_o, O.AGGR_SUM, q6.postfix(), o1)
    assert expr_sum_ok(got, want, O.aggregate(ds_o, O.AGGR_NONE, q6.postfix(), o1))
    # Q1
    one = E.Expr.Literal(1.0)
    q1 = [E.Aggregation.sum(E.Expr.Index(0)), E.Aggregation.sum(E.Expr.Index(1)),
          E.Aggregation.sum(E.Expr.Index(1) * (one - E.Expr.Index(2))),
          E.Aggregation.sum((E.Expr.Index(1) * (one - E.Expr.Index(2))) * (one + E.Expr.Index(3))),
          E.Aggregation.sum(E.Expr.Index(2))]
    got = E.Aggregation.compute_multiple(q1, ds_e)
    for a, g in zip(q1, got):
        want = O.aggregate(ds_o, a.kind, a.expr.postfix())
        if a.expr.kind == "index":
            assert sum_ok(g, want, True), (a.expr, g, want)  # BUFF's exact integer sum
        else:
            assert expr_sum_ok(g, want, O.aggregate(ds_o, O.AGGR_NONE, a.expr.postfix())), (a.expr, g, want)


@pytest.mark.gpu
def test_buff_fused_and_general_paths_agree():
    """Aligned BUFF columns take the fused path; with a precision set (or an
    array result) they take the materializing one.  Both follow the oracle."""
    rng = np.random.default_rng(12)
    n = 100_000
    cols = [np.round(rng.uniform(-50, 50, n), 3) for _ in range(3)]
    ds_o = [O.Decoder(O.encode(c, O.BUFF, O.CHUNK_RECORD_COUNT, 10_000, 1000)) for c in cols]
    ds_e = [E.Decoder(E.encode(c, "buff", ("record_count", 10_000), 1000)) for c in cols]
    rows = np.sort(rng.choice(n, 7_000, replace=False))
    for mask in (None, O.mask_from_rows(rows.tolist(), n)):
        for expr in EXPRS:
            for kind in (O.AGGR_SUM, O.AGGR_MIN, O.AGGR_MAX):
                _check_engine(ds_e, ds_o, expr, kind, mask)
    for d in ds_e + ds_o:
        d.with_precision(1)
    for expr in EXPRS[:3]:
        for kind in (O.AGGR_SUM, O.AGGR_MAX):
            _check_engine(ds_e, ds_o, expr, kind, None)


@pytest.mark.gpu
def test_fused_pass_compiled_at_run_time_matches_interpreter(monkeypatch):
    """Exact fused passes run the walk compiled at run time with the programs
    written out (EBI_EXPR_JIT=require: a compile failure is an error); the
    same passes through the interpreter (EBI_EXPR_JIT=0) give bit-identical
    results, and both follow the oracle.  Rows not a multiple of the 256-row
    unit, masks (an empty one too), stacks, shifted literals, several
    aggregations per pass, chunks at and off a column's common width, bare
    Index aggregations folded into the pass."""
    rng = np.random.default_rng(14)
    n = 70_001
    price = np.round(rng.uniform(900, 105000, n), 2)
    disc = np.round(rng.integers(0, 11, n) / 100.0, 2)
    tax = np.round(rng.integers(0, 9, n) / 100.0, 2)
    # chunk-dependent magnitudes: the chunks of this column differ in width, so
    # the compiled pass decodes some at the common width and some generally
    neg = np.round(rng.uniform(-50, 50, n) * (1 + (np.arange(n) // 16_384) * 40), 2)
    cols = [price, disc, tax, neg]
    ds_o = [O.Decoder(O.encode(c, O.BUFF, O.CHUNK_RECORD_COUNT, 16_384, 100)) for c in cols]
    ds_e = [E.Decoder(E.encode(c, "buff", ("record_count", 16_384), 100)) for c in cols]
    one = E.Expr.Literal(1.0)
    i0, i1, i2, i3 = (E.Expr.Index(k) for k in range(4))
    aggs = [E.Aggregation.sum(i0 * (one - i1)), E.Aggregation.sum((i0 * (one - i1)) * (one + i2)),
            E.Aggregation.min(i3 * i1 - 0.25), E.Aggregation.max((i3 + i2) * (i1 - i3)),
            E.Aggregation.sum(i3 - i0), E.Aggregation.max(i0 * i1),
            # bare Index aggregations: folded into the compiled pass when it runs,
            # else their columns' own scans; the same bits either way
            E.Aggregation.sum(i3), E.Aggregation.min(i0)]
    rows = np.sort(rng.choice(n, 20_000, replace=False))
    for mask in (None, O.mask_from_rows(rows.tolist(), n), O.mask_from_rows([], n)):
        results = {}
        for mode in ("0", "require"):
            monkeypatch.setenv("EBI_EXPR_JIT", mode)
            results[mode] = E.Aggregation.compute_multiple(aggs, ds_e, mask)
            for a in aggs[:3]:
                _check_engine(ds_e, ds_o, a.expr, a.kind, mask)
        got, ref = results["require"], results["0"]
        assert np.array_equal(np.array(got, float).view(np.uint64), np.array(ref, float).view(np.uint64)), (got, ref)
        for a, g in zip(aggs, got):
            if a.expr.kind == "index":
                want = {O.AGGR_SUM: ds_o[a.expr.index].sum, O.AGGR_MIN: ds_o[a.expr.index].min,
                        O.AGGR_MAX: ds_o[a.expr.index].max}[a.kind](mask)
                assert same_scalar(g, want), (a.expr, g, want)  # BUFF's exact sums: bit for bit
                continue
            want = O.aggregate(ds_o, a.kind, a.expr.postfix(), mask)
            if a.kind == O.AGGR_SUM:
                assert expr_sum_ok(g, want, O.aggregate(ds_o, O.AGGR_NONE, a.expr.postfix(), mask)), (a.expr, g, want)
            else:
                assert same_scalar(g, want), (a.expr, g, want)


@pytest.mark.gpu
def test_buff_wide_values_take_the_f64_kernel():
    """Scale 10^6 on values near 10^6: 41-bit fixed-point integers, whose
    products pass 2^53, so the fused path evaluates in f64 (sums of single
    columns' linear terms stay exact on the integers)."""
    rng = np.random.default_rng(13)
    n = 60_000
    cols = [np.round(rng.uniform(-1e6, 1e6, n), 6) for _ in range(3)]
    ds_o = [O.Decoder(O.encode(c, O.BUFF, O.CHUNK_RECORD_COUNT, 16_384, 1_000_000)) for c in cols]
    ds_e = [E.Decoder(E.encode(c, "buff", ("record_count", 16_384), 1_000_000)) for c in cols]
    rows = np.sort(rng.choice(n, 9_000, replace=False))
    for mask in (None, O.mask_from_rows(rows.tolist(), n)):
        for expr in (E.Expr.Index(0) * E.Expr.Index(1), E.Expr.Index(0) + E.Expr.Index(2) - 0.5,
                     (E.Expr.Index(0) - E.Expr.Index(1)) * (E.Expr.Index(1) + E.Expr.Index(2))):
            for kind in (O.AGGR_SUM, O.AGGR_MIN, O.AGGR_MAX):
                _check_engine(ds_e, ds_o, expr, kind, mask)


@pytest.mark.gpu
def test_errors_in_a_column_reach_the_aggregation():
    """A chunk whose header claims more bits than its bytes hold: the fused pass
    sees its status and the general pass reports the reference's error."""
    rng = np.random.default_rng(31)
    v = np.round(rng.uniform(-1, 1, 5000), 3)
    data = bytearray(E.encode(v, "buff", ("record_count", 1000), 1000))
    d = O.Decoder(bytes(data))
    phys, _, _, _ = d.chunk_info(1)
    data[phys + 12] = 40
    other = E.encode(np.round(rng.uniform(0, 1, 5000), 2), "buff", ("record_count", 1000), 100)
    ds_e = [E.Decoder(bytes(data)), E.Decoder(other)]
    ds_o = [O.Decoder(bytes(data)), O.Decoder(other)]
    expr = E.Expr.Index(0) * E.Expr.Index(1)
    with pytest.raises(O.OracleError) as eo:
        O.aggregate(ds_o, O.AGGR_SUM, expr.postfix())
    with pytest.raises(E.DecoderError) as ee:
        E.Aggregation.sum(expr).compute(ds_e)
    assert ee.value.code == eo.value.code == E.UnexpectedEndOfChunk.code
    # a mask that misses the bad chunk's rows: neither side reads it
    mask = O.mask_from_rows(list(range(0, 900)), 5000)
    assert E.Aggregation.max(expr).compute(ds_e, mask) == O.aggregate(ds_o, O.AGGR_MAX, expr.postfix(), mask)


@pytest.mark.gpu
def test_empty_columns():
    ds_e = [E.Decoder(E.encode(np.zeros(0), "buff", ("record_count", 100), 1000)) for _ in range(2)]
    ds_o = [O.Decoder(E.encode(np.zeros(0), "buff", ("record_count", 100), 1000)) for _ in range(2)]
    expr = E.Expr.Index(0) + E.Expr.Index(1)
    for kind in (O.AGGR_SUM, O.AGGR_MIN, O.AGGR_MAX):
        assert same_scalar(E.Aggregation(kind, expr).compute(ds_e), O.aggregate(ds_o, kind, expr.postfix()))
    assert E.Aggregation.sum(E.Expr.Index(0)).compute(ds_e) == O.aggregate(ds_o, O.AGGR_SUM, E.Expr.Index(0).postfix())
    # AggregationResult::zero: a Literal is not even looked at without chunks
    assert E.Aggregation.sum(E.Expr.Literal(2.0)).compute(ds_e) == 0.0
