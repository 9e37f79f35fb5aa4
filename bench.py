"""Benchmark of the fused decode + range filter + sum/min/max path on one GB300.

Workload (the configuration the headline metric is quoted on): a BUFF column of
67,108,864 f64 values, uniform on [-1000, 1000] rounded to 3 decimals, in
65,536-value chunks (scale 1000).  One step is one fused filter+sum query
(Decoder::filter then Decoder::sum/min/max over its result, in one pass),
cycling through the 1 %, 10 % and 50 % selectivity ranges [-10, 10],
[-100, 100], [-500, 500].  The column is resident in HBM; L2 is flushed before
every step.  value = GB/s of decoded f64 (8 B x rows per query / device time),
the reference's throughput definition (uncompressed bytes / elapsed time).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload NAME]

--workload picks one of the other measured shapes instead of the headline
BUFF column: "gorilla" (1,048,576-value random walk, 8,192-value chunks,
filter 10 <= x <= 50 + sum/min/max), "chimp128" (16,777,216-value sensor
series, filter 15 <= x <= 25 + max), "elf" / "elf_on_chimp" (the same sensor
series and query through the Elf codecs) and "rle" (16,777,216-value step
series, filter over the middle 30 % of its values + max).

Under torchrun every rank runs the same workload on its own GPU (replicas: the
path has no cross-column exchange), and value sums the ranks' rows over the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "decode+filter+sum GB/s"
UNIT = "GB/s"
N_ROWS = 67_108_864
CHUNK = 65_536
SCALE = 1000
FALLBACK_HBM_GBS = 6800.0


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def replica_throughput(local_s: float, local_rows: int, dist=None, device=None):
    """Whole-job decoded GB/s of N replicas: every rank's rows over the slowest rank's time.

    Returns (slowest rank's device seconds, GB/s of 8-byte values).  Without a process group
    (one GPU) it is the local figure."""
    import torch

    t = local_s
    rows = local_rows
    if dist is not None and dist.is_initialized():
        tt = torch.tensor([local_s, float(local_rows)], dtype=torch.float64,
                          device=device if device is not None else "cpu")
        mx = tt.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        dist.all_reduce(tt, op=dist.ReduceOp.SUM)
        t = float(mx[0].item())
        rows = int(tt[1].item())
    return t, 8.0 * rows / t / 1e9


def workload_generators():
    """The seeded value generators (ebi_gb300/workloads.py), loaded from their file alone.

    Loading the file by path keeps the package (and so libebi_gpu.so) out of the
    reference arm's process: that arm runs only ebi's CPU path."""
    import importlib.util

    mod = sys.modules.get("_ebi_workloads")
    if mod is None:
        spec = importlib.util.spec_from_file_location("_ebi_workloads", ROOT / "ebi_gb300" / "workloads.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        sys.modules["_ebi_workloads"] = mod
    return mod


class Workload:
    """One measured shape: its column (EBI1 bytes) and the range queries a step cycles through."""

    def __init__(self, name, rows):
        W = workload_generators()

        self.name = name
        self.rows = rows
        if name == "buff":
            self.codec, self.chunk, self.scale = "buff", CHUNK, SCALE
            self.values = lambda: W.buff_uniform(self.rows)
            self.ranges = [(k, -a, a) for k, a in W.BUFF_RANGES.items()]
            self.aggregates = ("sum",)
            self.describe = ("BUFF 67,108,864 f64 U[-1000,1000] rounded to 3 dp, 65,536-row chunks, scale 1000; "
                             "fused filter (bitmask out) + sum at 1%/10%/50% selectivity")
        elif name == "gorilla":
            self.codec, self.chunk, self.scale = "gorilla", 8192, 1
            self.values = lambda: W.gorilla_walk(self.rows)
            self.ranges = [("10<=x<=50", 10.0, 50.0)]
            self.aggregates = ("sum", "min", "max")
            self.describe = ("Gorilla 1,048,576 f64 random walk x0=30, N(0,0.5) steps, 2 dp, 8,192-row chunks; "
                             "fused filter 10<=x<=50 (bitmask out) + sum/min/max")
        elif name == "chimp128":
            self.codec, self.chunk, self.scale = "chimp128", 8192, 1
            self.values = lambda: W.sensor(self.rows)
            self.ranges = [("15<=x<=25", 15.0, 25.0)]
            self.aggregates = ("max",)
            self.describe = ("Chimp128 16,777,216 f64 sensor series 20+10sin(2pi i/1440)+N(0,0.1), 4 dp, "
                             "8,192-row chunks; fused decode + filter 15<=x<=25 (bitmask out) + max")
        elif name in ("elf", "elf_on_chimp"):
            self.codec, self.chunk, self.scale = name, 8192, 1
            self.values = lambda: W.sensor(self.rows)
            self.ranges = [("15<=x<=25", 15.0, 25.0)]
            self.aggregates = ("max",)
            label = "Elf" if name == "elf" else "ElfOnChimp"
            self.describe = (f"{label} 16,777,216 f64 sensor series 20+10sin(2pi i/1440)+N(0,0.1), 4 dp, "
                             "8,192-row chunks; fused decode + decimal restore + filter 15<=x<=25 (bitmask out) + max")
        elif name == "rle":
            self.codec, self.chunk, self.scale = "rle", 8192, 1
            self.values = lambda: W.steps(self.rows)
            self.ranges = None  # the middle 30 % of the values, fixed once the column exists
            self.aggregates = ("max",)
            self.describe = ("RLE 16,777,216 f64 step series, Geometric(1/64) runs, 8,192-row chunks; "
                             "fused decode + filter over the middle 30% of values (bitmask out) + max")
        else:
            raise SystemExit(f"unknown workload {name}")

    def build(self, encoder="engine"):
        """The column's EBI1 bytes, written by the engine's host encoder or (encoder="oracle") by the
        oracle's; the two write identical bytes (tests/test_cpu_abi.py)."""
        t = time.perf_counter()
        v = self.values()
        if self.ranges is None:
            lo, hi = np.quantile(v, [0.35, 0.65])
            self.ranges = [(f"{lo:.1f}<=x<={hi:.1f}", float(lo), float(hi))]
        if encoder == "oracle":
            from oracle import oracle as O

            data = O.encode(v, self.codec, O.CHUNK_RECORD_COUNT, self.chunk, self.scale)
        else:
            import ebi_gb300 as E

            data = E.encode(v, self.codec, ("record_count", self.chunk), self.scale)
        log(f"workload {self.name}: {self.rows} rows, {len(data)} B EBI1 ({time.perf_counter() - t:.1f} s to generate)")
        return data

    def queries(self):
        import ebi_gb300 as E

        return [(k, E.Predicate.range(E.RangeValue.inclusive(a), E.RangeValue.inclusive(b))) for k, a, b in self.ranges]

    def oracle_preds(self):
        from oracle import oracle as O

        return [O.rng(O.BOUND_INCLUSIVE, a, O.BOUND_INCLUSIVE, b) for _, a, b in self.ranges]


DEFAULT_ROWS = {"buff": N_ROWS, "gorilla": 1_048_576, "chimp128": 16_777_216, "rle": 16_777_216,
                "elf": 16_777_216, "elf_on_chimp": 16_777_216}
KERNELS = {"buff": "buff_stream_kernel<2,6> (register-streaming decode + range filter + bitmask + sum)",
           "gorilla": "gorilla_kernel (three warps per chunk: parse, bitmask + min/max, sums)",
           "chimp128": "xor_converge_kernel + xor_kernel<Chimp128> (segment control parse, then extraction + ring "
                       "resolution + filter + bitmask + max)",
           "elf": "xor_converge_kernel + xor_kernel<Elf> (segment control parse, then extraction + decimal restore "
                  "+ filter + bitmask + max)",
           "elf_on_chimp": "xor_converge_kernel + xor_kernel<ElfOnChimp> (segment control parse, then extraction + "
                           "decimal restore + filter + bitmask + max)",
           "rle": "rle_kernel (run expansion + filter + bitmask + max)"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.perf_counter(), [x.strip() for x in line.split(",")]))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self, t0, t1):
        rows = [r for t, r in self.rows if t0 - 0.15 <= t <= t1 + 0.15] or [r for _, r in self.rows]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        pw = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "power_w_max": max(pw) if pw else None}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(workload="buff"):
    """DRAM bytes per launch of the workload's dominant kernel from the committed ncu summary, if any."""
    p = ROOT / "profiles" / f"{workload}_traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text()).get("dram_bytes_per_launch")
        except Exception:
            return None
    return None


def time_cpu_queries(d, preds, n, two_call=False, aggregates=("sum",)):
    """Seconds per query of n queries on the oracle Decoder d, cycling preds.

    two_call: the reference's own shape of a filtered aggregate, Decoder::filter followed by
    Decoder::sum / min / max(Some(&bitmask)), each call reading every chunk again
    (api/decoder.rs:242-281, 323-439); otherwise one fused pass per query."""
    ts = []
    for i in range(n):
        p = preds[i % len(preds)]
        t = time.perf_counter()
        if two_call:
            m = d.filter(p)
            for a in aggregates:
                getattr(d, a)(m)
        else:
            d.filter_agg(p)
        ts.append(time.perf_counter() - t)
    return ts


def cpu_figures(data: bytes, wl, threads: int, n_all: int = 9, n_one: int = 3):
    """The oracle port on the host cores, over the full column and the workload's own queries.

    Three figures, as decoded GB/s (8 B x rows / median seconds per query):
      value      fused filter+aggregate, chunk-parallel on `threads` host threads;
      threads_1  the same on one thread, the reference's execution model (single-threaded Decoder);
      two_call   filter, then the aggregates over its bitmask, each a separate chunk loop, on `threads`."""
    from oracle import oracle as O

    preds = wl.oracle_preds()
    dall = O.Decoder(data, threads=threads)
    n = dall.n_records
    dall.filter_agg(preds[0])  # first touch of the file's pages
    fused = time_cpu_queries(dall, preds, n_all)
    two = time_cpu_queries(dall, preds, max(n_one, len(preds)), two_call=True, aggregates=wl.aggregates)
    one = time_cpu_queries(O.Decoder(data, threads=1), preds, n_one) if n_one else []
    gbs = lambda ts: round(8.0 * n / statistics.median(ts) / 1e9, 3) if ts else None
    qs = ", ".join(k for k, _, _ in wl.ranges)
    return {"value": gbs(fused), "unit": UNIT, "cores": threads, "kind": "port",
            "mean_value": round(8.0 * n * len(fused) / sum(fused) / 1e9, 3),
            "threads_1": {"value": gbs(one), "cores": 1, "queries": len(one)},
            "two_call": {"value": gbs(two), "cores": threads, "queries": len(two),
                         "calls": f"filter, then {'/'.join(wl.aggregates)}(Some(&bitmask))"},
            "sample": f"median of {len(fused)} fused filter+aggregate queries ({qs} cycled) over the full {n}-row "
                      f"column, chunk-parallel C restatement of ebi's Decoder on {threads} host threads; threads_1: "
                      f"{len(one)} queries on one thread; two_call: {len(two)} queries as the reference's two calls"}


def same_bits(a, b):
    """Two f64 results with the same bits (NaN results compare equal)."""
    return np.float64(a).view(np.uint64) == np.float64(b).view(np.uint64) or (np.isnan(a) and np.isnan(b))


def value_config(name, dev, steps, warmup, flush, clean):
    """One of the other single-column configurations, measured as the headline is: each step one
    fused filter + aggregate query with L2 flushed before it; the median device time of the query
    and of its codec kernel (roofline over the compressed chunk bytes plus the bitmask), the last
    query against the oracle, and the oracle port on all host cores over the same queries."""
    import torch

    import ebi_gb300 as E
    from oracle import oracle as O

    wl = Workload(name, DEFAULT_ROWS[name])
    data = wl.build()
    dec = E.Decoder(data, device=str(dev))
    dec.set_timing(True)
    mask = dec.new_mask()
    qs = wl.queries()
    alg = sum(dec.chunk_info(c)[1] for c in range(dec.n_chunks)) + 8 * dec.mask_words
    scan, total = [], []
    for i in range(warmup + steps):
        flush.fill_(i & 0xFF)
        clean.sum()
        torch.cuda._sleep(1_000_000)
        dec.filter_agg(qs[i % len(qs)][1], out=mask, aggregates=wl.aggregates)
        t = dec.segmented_execution_times()
        if i >= warmup:
            scan.append(t["scan_ms"])
            total.append(t["total_ms"])
    _, p = qs[-1]
    _, s, mn, mx, cnt = dec.filter_agg(p, out=mask)
    o = O.Decoder(data, threads=os.cpu_count() or 1)
    om, os_, omn, omx = o.filter_agg(O.rng(1, p.rng.start.value, 1, p.rng.end.value))
    exact = wl.codec == "buff"
    same = (np.array_equal(mask.cpu().numpy().view(np.uint64)[: len(om)], om) and (mn, mx) == (omn, omx)
            and (s == os_ if exact else abs(s - os_) <= 1e-12 * max(abs(os_), 1e-300)))
    # the unfiltered aggregates (decode + sum / min / max, one call each, as the reference's Decoder)
    unfiltered = {}
    for a in wl.aggregates:
        ks_a = []
        for i in range(warmup + max(5, steps // 2)):
            flush.fill_(i & 0xFF)
            clean.sum()
            torch.cuda._sleep(1_000_000)
            got = getattr(dec, a)()
            if i >= warmup:
                ks_a.append(dec.segmented_execution_times()["total_ms"])
        want = getattr(o, a)()
        ok = same_bits(got, want) if a != "sum" else (got == want if exact else abs(got - want) <= 1e-12 * max(abs(want), 1e-300))
        unfiltered[a] = {"ms": round(statistics.median(ks_a), 4),
                         "decoded_gb_per_s": round(8.0 * wl.rows / (statistics.median(ks_a) / 1e3) / 1e9, 3),
                         "equal_to_oracle": bool(ok)}
    peak, _ = measured_peak()
    ks, ts = statistics.median(scan) / 1e3, statistics.median(total) / 1e3
    cpu = cpu_figures(data, wl, os.cpu_count() or 1, n_all=5, n_one=0)
    dec.close()
    return {"workload": wl.describe, "rows": wl.rows, "chunk_rows": wl.chunk, "column_bytes": len(data),
            "queries": [k for k, _, _ in wl.ranges], "value": round(8.0 * wl.rows / ts / 1e9, 3), "unit": UNIT,
            "ms_per_step": round(1e3 * ts, 4), "kernel": KERNELS[name], "kernel_ms": round(1e3 * ks, 4),
            "roofline": {"bound": "hbm", "algorithmic_bytes_per_launch": alg,
                         "achieved": round(alg / ks / 1e9, 1), "peak": peak, "frac": round(alg / ks / 1e9 / peak, 4)},
            "parity_check": {"bitmask_min_max_bit_exact_sum_within_tolerance": bool(same),
                             "sum_rel_diff": abs(s - os_) / max(abs(os_), 1e-300), "rows_selected": int(cnt)},
            "unfiltered": unfiltered,
            "cpu_baseline": {k: cpu[k] for k in ("value", "cores", "kind")}}


def materialize_config(dec, data, dev, steps, warmup, flush, clean):
    """C2's full materialize: every value of the headline column written out (8 B a row, the
    write-bound BUFF decode), median device time over L2-flushed steps, checked against the oracle."""
    import torch

    from oracle import oracle as O

    n = dec.n_records
    out = torch.empty(n, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    dec.set_timing(True)
    ts, ks = [], []
    for i in range(warmup + steps):
        flush.fill_(i & 0xFF)
        clean.sum()
        torch.cuda._sleep(1_000_000)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        dec.materialize(out=out)
        e1.record(stream)
        e1.synchronize()
        if i >= warmup:
            ts.append(e0.elapsed_time(e1) / 1e3)
            ks.append(dec.segmented_execution_times()["scan_ms"] / 1e3)
    t = statistics.median(ts)
    kt = statistics.median(ks)
    want = O.Decoder(data, threads=os.cpu_count() or 1).materialize()
    same = bool(np.array_equal(out.cpu().numpy().view(np.uint64), want.view(np.uint64)))
    col = sum(dec.chunk_info(c)[1] for c in range(dec.n_chunks))
    alg = col + 8 * n
    peak, _ = measured_peak()
    return {"workload": "C2 full materialize: every value of the headline column written to a device array",
            "rows": n, "value": round(8.0 * n / t / 1e9, 3), "unit": UNIT, "ms_per_step": round(1e3 * t, 4),
            "kernel": "buff_materialize_kernel<false> (32-bit deltas)", "kernel_ms": round(1e3 * kt, 4),
            "roofline": {"bound": "hbm", "algorithmic_bytes_per_launch": alg, "read_bytes": col, "write_bytes": 8 * n,
                         "achieved": round(alg / t / 1e9, 1), "peak": peak, "frac": round(alg / t / 1e9 / peak, 4),
                         "scope": "whole call (decode + write)",
                         "kernel_achieved": round(alg / kt / 1e9, 1), "kernel_frac": round(alg / kt / 1e9 / peak, 4)},
            "parity_check": {"values_bit_exact": same}}


def config_results(args, dec, data, dev, flush, clean):
    """The other configurations in one object of the headline line: C1, C3a, C3b (and the Elf
    codecs on C3a's series), C2's full materialize, C4 batched and C5 serving at full size."""
    import copy

    import torch

    props = torch.cuda.get_device_properties(dev)
    sampler = ClockSampler(f"GPU-{props.uuid}" if getattr(props, "uuid", None) else str(dev.index or 0))
    sampler.start()
    time.sleep(0.3)
    spans = {}

    def timed(key, fn):
        t0 = time.perf_counter()
        r = fn()
        spans[key] = (t0, time.perf_counter())
        return r

    res = {"C2_materialize": timed("C2_materialize", lambda: materialize_config(dec, data, dev, 10, 3, flush, clean))}
    for key, name in (("C1_gorilla", "gorilla"), ("C3a_chimp128", "chimp128"), ("C3b_rle", "rle"),
                      ("C3a_series_elf", "elf"), ("C3a_series_elf_on_chimp", "elf_on_chimp")):
        res[key] = timed(key, lambda: value_config(name, dev, 20, 3, flush, clean))
        log(f"config {key}: {res[key]['kernel_ms']} ms kernel")
    a = copy.copy(args)
    a.scale, a.steps, a.warmup = 1.0, 10, 3
    b = timed("C4_batched", lambda: batched_line(a))
    res["C4_batched"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "queries_per_s", "config", "roofline",
                                           "autotune", "parity_check")}
    a.steps = 40
    v = timed("C5_serving", lambda: serving_line(a))
    res["C5_serving"] = {k: v[k] for k in ("value", "unit", "plain_queries_per_s", "plain_statistic",
                                           "plain_queries_per_s_runs", "plain_queries_per_s_median", "speedup_vs_plain",
                                           "decoded_gb_per_s_saturated", "results_equal_alone_and_in_mix", "poisson",
                                           "config", "server_stats")}
    time.sleep(0.2)
    sampler.stop()
    for key, (t0, t1) in spans.items():
        res[key]["clocks"] = dict(sampler.summary(t0, t1), window="the whole configuration: column build and timed steps")
    return res


def run_reference(args):
    """Reference arm: ebi's CPU path (the C restatement; the Rust crate has no toolchain here).

    The column is the configuration's full column, written by the oracle's encoder (the same
    bytes the engine's encoder writes), and nothing of the engine is loaded in this process.
    Each step is one fused filter+aggregate query run chunk-parallel on every host thread;
    value uses the median step time.  The line also carries the one-thread figure (the
    reference's own execution model) and the reference's two-call filter-then-aggregate time."""
    rank, _, world = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    from oracle import oracle as O

    wl = Workload(args.workload, args.rows or DEFAULT_ROWS[args.workload])
    data = wl.build(encoder="oracle")
    d = O.Decoder(data, threads=threads)
    preds = wl.oracle_preds()
    for i in range(args.warmup):
        d.filter_agg(preds[i % len(preds)])
    ts = time_cpu_queries(d, preds, args.steps)
    med = statistics.median(ts)
    value = 8.0 * wl.rows / med / 1e9
    one = time_cpu_queries(O.Decoder(data, threads=1), preds, 3)
    two = time_cpu_queries(d, preds, max(3, len(preds)), two_call=True, aggregates=wl.aggregates)
    gbs = lambda t: round(8.0 * wl.rows / statistics.median(t) / 1e9, 3)
    sample = (f"per step one fused filter+aggregate ({', '.join(k for k, _, _ in wl.ranges)} cycled) over the "
              f"full {wl.rows}-row column ({d.n_chunks} chunks), chunk-parallel C restatement of ebi's CPU path "
              f"on {threads} host threads (ebi is Rust; no Rust toolchain exists on this image); median step")
    line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * med, 4),
            "mean_ms_per_step": round(1e3 * sum(ts) / len(ts), 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/u64 -> f64",
            "data": "synthetic (seeded numpy, the configuration's shape)",
            "config": {"workload": wl.describe, "rows": wl.rows, "chunk_rows": wl.chunk,
                       "column_bytes": len(data), "encoder": "oracle (byte-identical to the engine's)"},
            "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample,
                             "threads_1": {"value": gbs(one), "cores": 1, "queries": len(one)},
                             "two_call": {"value": gbs(two), "cores": threads, "queries": len(two),
                                          "calls": f"filter, then {'/'.join(wl.aggregates)}(Some(&bitmask))"}},
            "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


MIXED_CODECS = ("gorilla", "chimp128", "buff", "rle")


def mixed_column(rng, codec, n, seed):
    """One column of a mixed-codec configuration: the generator of its codec's measured shape."""
    import ebi_gb300 as E
    from ebi_gb300 import workloads as W

    if codec == "buff":
        v = W.round_dp(rng.uniform(-1000.0, 1000.0, n), 3)
        return E.encode(v, "buff", ("record_count", CHUNK), SCALE)
    if codec == "gorilla":
        v = W.gorilla_walk(n, seed=seed)
    elif codec == "chimp128":
        v = W.sensor(n, seed=seed)
    else:
        v = W.steps(n, seed=seed)
    return E.encode(v, codec, ("record_count", 8192))


def build_mixed(n_cols, lo, hi, seed, dev):
    """n_cols columns of log-uniform length in [lo, hi], codec drawn uniformly (seeded).
    Columns are generated and encoded on host threads (each from its own seeded generator),
    then opened on the device in order."""
    from concurrent.futures import ThreadPoolExecutor

    import ebi_gb300 as E

    rng = np.random.default_rng(seed)
    lens = np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi), n_cols))).astype(np.int64)
    codecs = rng.integers(0, len(MIXED_CODECS), n_cols)
    t = time.perf_counter()

    def make(i):
        codec = MIXED_CODECS[codecs[i]]
        return mixed_column(np.random.default_rng((seed, i)), codec, int(lens[i]), seed * 100003 + i)

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        datas = list(ex.map(make, range(n_cols)))
    decs, meta = [], []
    for i, data in enumerate(datas):
        decs.append(E.Decoder(data, device=str(dev)))
        meta.append((MIXED_CODECS[codecs[i]], int(lens[i]), len(data)))
    log(f"built {n_cols} columns, {int(lens.sum())} rows, {sum(m[2] for m in meta)} B in {time.perf_counter() - t:.1f} s")
    return decs, meta


def column_range(codec, rng):
    """A range predicate of about 10-50 % selectivity on a column of the codec's shape."""
    import ebi_gb300 as E

    if codec == "buff":
        a = float(rng.uniform(-900, 0)); b = a + float(rng.uniform(200, 1000))
    elif codec == "gorilla":
        a = float(rng.uniform(-200, 0)); b = a + float(rng.uniform(50, 400))
    elif codec == "chimp128":
        a = float(rng.uniform(10, 20)); b = a + float(rng.uniform(2, 10))
    else:
        a = float(rng.uniform(0, 60)); b = a + float(rng.uniform(20, 80))
    return E.Predicate.range(E.RangeValue.inclusive(a), E.RangeValue.inclusive(b))


def run_batched(args):
    print(json.dumps(batched_line(args)), flush=True)


def batched_line(args):
    """4,096 columns of log-uniform length 1K..4M, codec uniform over {Gorilla, Chimp128, BUFF, RLE};
    one step = filter+sum on every column as one batch (persistent mixed-codec launch, graph replay)."""
    import torch

    import ebi_gb300 as E

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    E.load_library()
    n_cols = max(1, int(round(4096 * args.scale)))
    decs, meta = build_mixed(n_cols, 1024, 4_194_304, 5, dev)
    rng = np.random.default_rng(55)
    preds = [column_range(m[0], rng) for m in meta]
    batch = E.Batch([(d, p, ("sum",)) for d, p in zip(decs, preds)])
    stream = torch.cuda.current_stream(dev)
    rows = sum(m[1] for m in meta)
    col_bytes = sum(m[2] for m in meta)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for i in range(max(args.warmup, 3)):
        batch.run()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = E.kernel_launches()
    ts = []
    for i in range(args.steps):
        flush.fill_(i & 0xFF)
        ev0.record(stream)
        batch.run()
        ev1.record(stream)
        ev1.synchronize()
        ts.append(ev0.elapsed_time(ev1) / 1e3)
    launches = E.kernel_launches() - launches0
    # parity spot check: the batch against single-column queries on a few columns
    got = batch.run()
    ok = True
    for k in list(range(0, n_cols, max(1, n_cols // 16)))[:16]:
        _, s_, _, _, n_ = decs[k].filter_agg(preds[k], aggregates=("sum",), want_mask=False)
        ok = ok and got[k][0] == s_ and got[k][3] == n_
    info = batch.info()
    t = statistics.median(ts)
    peak, peak_kind = measured_peak()
    by_codec = {c: sum(1 for m in meta if m[0] == c) for c in MIXED_CODECS}
    line = {"metric": "batched filter+sum GB/s (decoded)", "value": round(8.0 * rows / t / 1e9, 3), "unit": "GB/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(1e3 * t, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "mixed -> f64",
            "data": "synthetic (seeded numpy, the configuration's shape)",
            "config": {"workload": "batched: columns of log-uniform length 1K..4M f64, codec uniform over "
                                   "Gorilla/Chimp128/BUFF/RLE, filter+sum per column in one batch",
                       "columns": n_cols, "scale": args.scale, "rows": rows, "column_bytes": col_bytes,
                       "columns_by_codec": by_codec, "l2": "flushed before every step (256 MiB write)"},
            "queries_per_s": round(n_cols / t, 1),
            "roofline": {"bound": "hbm", "achieved": round(col_bytes / t / 1e9, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(col_bytes / t / 1e9 / peak, 4), "traffic": None,
                         "kernel": "batch_kernel + batch_finalize_kernel (graph replay)", "peak_source": peak_kind},
            "autotune": info, "gpu_launches": int(launches),
            "parity_check": {"sum_and_count_equal_single_column_queries": bool(ok)}}
    batch.close()
    for d in decs:
        d.close()
    return line


def run_serving(args):
    print(json.dumps(serving_line(args)), flush=True)


def serving_line(args):
    """512 resident columns of log-uniform length 256K..16M, mixed codecs; Poisson arrivals; each request a
    random range plus one of sum/min/max over 1..8 columns.  Continuous batching vs plain per-query launches."""
    import torch

    import ebi_gb300 as E

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    E.load_library()
    n_cols = max(8, int(round(512 * args.scale)))
    decs, meta = build_mixed(n_cols, 262_144, 16_777_216, 6, dev)
    rng = np.random.default_rng(66)

    def make_requests(n):
        reqs = []
        for _ in range(n):
            k = int(rng.integers(1, 9))
            ids = [int(x) for x in rng.choice(n_cols, size=k, replace=False)]
            p = column_range(meta[ids[0]][0], rng)
            reqs.append((ids, p, (("sum",), ("min",), ("max",))[int(rng.integers(3))]))
        return reqs

    # plain per-query launches (closed loop, one request at a time), after one query on every
    # column (first-use allocations out of the timing)
    E.run_plain(decs, [([i], column_range(meta[i][0], rng), ("sum",)) for i in range(n_cols)])
    plain_reqs = make_requests(max(20, args.steps))
    plain_rates, plain = [], None
    for _ in range(3):  # best of three: the host's other work can stretch single runs
        t0 = time.perf_counter()
        got = E.run_plain(decs, plain_reqs)
        plain_rates.append(len(plain_reqs) / (time.perf_counter() - t0))
        plain = plain if plain is not None else got
    plain_qps = max(plain_rates)
    plain_median_qps = 1e9 / float(np.median([r["done_ns"] - r["submit_ns"] for r in plain]))
    caps = {"slots": 4, "max_queries": 16384, "max_chunks": 1 << 23, "max_items": 1 << 23}
    srv = E.Server(decs, **caps)
    srv.replay(plain_reqs[:50])  # warm-up
    # saturated throughput: a full queue of 10,000 requests (the plain requests first, then more), all
    # submitted at once, so that several batches run back to back;
    # the plain requests' answers in the mix are compared bit for bit with their plain answers
    sat_reqs = plain_reqs + make_requests(max(0, 10_000 - len(plain_reqs)))
    t0 = time.perf_counter()
    mixed = srv.replay(sat_reqs)
    sat_s = time.perf_counter() - t0
    sat_qps = len(sat_reqs) / sat_s
    sat_rows = sum(meta[i][1] for ids, _, _ in sat_reqs for i in ids)
    mixed = mixed[: len(plain_reqs)]
    equal = all((a["count"] == b["count"]) and all(
        (a[f] == b[f]) or (np.isnan(a[f]) and np.isnan(b[f])) for f in ("sum", "min", "max"))
        for a, b in zip(plain, mixed))
    rates = []
    for lam in (2_000, 5_000, 10_000, 20_000, 50_000):
        n = int(min(4000, max(200, lam * 0.5)))
        reqs = make_requests(n)
        arr = np.cumsum(rng.exponential(1e9 / lam, n))
        t0 = time.perf_counter()
        res = srv.replay(reqs, arr)
        wall = time.perf_counter() - t0
        lat = np.array([(r["done_ns"] - r["submit_ns"]) / 1e6 for r in res])
        rates.append({"offered_per_s": lam, "requests": n, "achieved_per_s": round(n / wall, 1),
                      "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
                      "errors": int(sum(1 for r in res if r["status"]))})
    st = srv.stats()
    srv.close()
    line = {"metric": "serving queries/s (continuous batching) vs plain per-query launches", "value": round(sat_qps, 1),
            "unit": "queries/s", "n_gpus": 1, "steps": len(plain_reqs), "warmup": 50, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "mixed -> f64",
            "data": "synthetic (seeded numpy, the configuration's shape)",
            "config": {"workload": "serving: resident columns of log-uniform length 256K..16M f64, codecs uniform over "
                                   "Gorilla/Chimp128/BUFF/RLE; requests: random range + one of sum/min/max over 1..8 columns",
                       "columns": n_cols, "scale": args.scale, "rows": sum(m[1] for m in meta),
                       "column_bytes": sum(m[2] for m in meta), **caps,
                       "tiling": "server default: 8 BUFF tiles, 8 RLE chunks, 16 Gorilla chunks per work item"},
            "saturated_requests": len(sat_reqs), "plain_requests": len(plain_reqs),
            "plain_queries_per_s": round(plain_qps, 1),
            "plain_statistic": "requests / wall time, one at a time, best of three runs",
            "plain_queries_per_s_runs": [round(x, 1) for x in plain_rates],
            "plain_queries_per_s_median": round(plain_median_qps, 1), "speedup_vs_plain": round(sat_qps / plain_qps, 2),
            "decoded_gb_per_s_saturated": round(8.0 * sat_rows / sat_s / 1e9, 1),
            "results_equal_alone_and_in_mix": bool(equal), "poisson": rates, "server_stats": st}
    for d in decs:
        d.close()
    return line


TPCH_ROWS = 59_986_052       # lineitem rows at scale factor 10
TPCH_CHUNK = 16_777_216      # ChunkOption::RecordCount(128 MiB / 8), the experimenter's default chunking


def tpch_columns(n, seed=6):
    """lineitem-shaped columns (l_quantity, l_extendedprice, l_discount, l_tax) drawn like dbgen's:
    quantity 1..50, price = quantity x part price (900..2000 + cents), discount 0.00..0.10, tax 0.00..0.08."""
    rng = np.random.default_rng(seed)
    qty = rng.integers(1, 51, n).astype(np.float64)
    part = np.round(rng.uniform(900.0, 2000.0, n), 2)
    price = np.round(qty * part, 2)
    disc = rng.integers(0, 11, n) / 100.0
    tax = rng.integers(0, 9, n) / 100.0
    return [qty, price, disc, tax]


def tpch_queries(E):
    one = E.Expr.Literal(1.0)
    q1 = [E.Aggregation.sum(E.Expr.Index(0)), E.Aggregation.sum(E.Expr.Index(1)),
          E.Aggregation.sum(E.Expr.Index(1) * (one - E.Expr.Index(2))),
          E.Aggregation.sum((E.Expr.Index(1) * (one - E.Expr.Index(2))) * (one + E.Expr.Index(3))),
          E.Aggregation.sum(E.Expr.Index(2))]
    p_disc = E.Predicate.range(E.RangeValue.inclusive(0.05), E.RangeValue.inclusive(0.07))
    p_qty = E.Predicate.range(E.RangeValue.NONE, E.RangeValue.exclusive(24.0))
    q6 = E.Aggregation.sum(E.Expr.Index(1) * E.Expr.Index(2))
    return q1, p_disc, p_qty, q6


def tpch_oracle(datas, query, O, n, exact=False):
    """The query on the oracle (the restatement of ebi's Decoder / Aggregation loops), one thread.
    exact: each sum's exactly rounded value instead (fsum of the values the oracle's expression yields;
    the in-situ BUFF sums of single columns are exact integer sums already)."""
    import math

    ds = [O.Decoder(d) for d in datas]
    if exact:
        I = lambda i: (O.EXPR_INDEX, i, 0.0)
        L = lambda x: (O.EXPR_LITERAL, 0, x)
        if query == "tpch_q6":
            m = ds[2].filter(O.rng(O.BOUND_INCLUSIVE, 0.05, O.BOUND_INCLUSIVE, 0.07))
            m = ds[0].filter(O.rng(O.BOUND_NONE, 0.0, O.BOUND_EXCLUSIVE, 24.0), m)
            v = O.aggregate(ds, O.AGGR_NONE, [I(1), I(2), (O.EXPR_MUL, 0, 0.0)], m)
            return [math.fsum(v)], [float(np.abs(v).sum())]
        pfs = [[I(1), L(1.0), I(2), (O.EXPR_SUB, 0, 0.0), (O.EXPR_MUL, 0, 0.0)],
               [I(1), L(1.0), I(2), (O.EXPR_SUB, 0, 0.0), (O.EXPR_MUL, 0, 0.0), L(1.0), I(3), (O.EXPR_ADD, 0, 0.0),
                (O.EXPR_MUL, 0, 0.0)]]
        vals = [O.aggregate(ds, O.AGGR_NONE, pf) for pf in pfs]
        ex = [ds[0].sum(), ds[1].sum(), math.fsum(vals[0]), math.fsum(vals[1]), ds[2].sum()]
        mag = [abs(ex[0]), abs(ex[1]), float(np.abs(vals[0]).sum()), float(np.abs(vals[1]).sum()), abs(ex[4])]
        return ex, mag
    I = lambda i: (O.EXPR_INDEX, i, 0.0)
    L = lambda x: (O.EXPR_LITERAL, 0, x)
    if query == "tpch_q6":
        m = ds[2].filter(O.rng(O.BOUND_INCLUSIVE, 0.05, O.BOUND_INCLUSIVE, 0.07))
        m = ds[0].filter(O.rng(O.BOUND_NONE, 0.0, O.BOUND_EXCLUSIVE, 24.0), m)
        return [O.aggregate(ds, O.AGGR_SUM, [I(1), I(2), (O.EXPR_MUL, 0, 0.0)], m)]
    q1 = [[I(0)], [I(1)], [I(1), L(1.0), I(2), (O.EXPR_SUB, 0, 0.0), (O.EXPR_MUL, 0, 0.0)],
          [I(1), L(1.0), I(2), (O.EXPR_SUB, 0, 0.0), (O.EXPR_MUL, 0, 0.0), L(1.0), I(3), (O.EXPR_ADD, 0, 0.0),
           (O.EXPR_MUL, 0, 0.0)], [I(2)]]
    return [O.aggregate(ds, O.AGGR_SUM, pf) for pf in q1]


def run_tpch(args):
    """TPC-H Q1 / Q6 shapes over lineitem-shaped BUFF columns (experimenter/src/tpch.rs:190-461): Q6 filters
    l_discount, then l_quantity under that bitmask, then sums l_extendedprice * l_discount over it; Q1 runs
    five sums (two of expressions) with Aggregation::compute_multiple."""
    import torch

    import ebi_gb300 as E

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    E.load_library()
    n = args.rows or TPCH_ROWS
    cols = tpch_columns(n)
    datas = [E.encode(c, "buff", ("record_count", TPCH_CHUNK), 100) for c in cols]
    ds = [E.Decoder(d, device=str(dev)) for d in datas]
    q1, p_disc, p_qty, q6 = tpch_queries(E)
    col_bytes = [sum(d.chunk_info(c)[1] for c in range(d.n_chunks)) for d in ds]
    mask_bytes = 8 * ds[0].mask_words
    if args.workload == "tpch_q6":
        used = [0, 1, 2]
        # disc + mask out; qty + mask in + mask out; price + disc + mask in
        alg = col_bytes[2] + mask_bytes + col_bytes[0] + 2 * mask_bytes + col_bytes[1] + col_bytes[2] + mask_bytes

        def step():
            m = ds[2].filter(p_disc)
            m = ds[0].filter(p_qty, m)
            return [q6.compute(ds, m)]
    else:
        used = [0, 1, 2, 3]
        # three in-situ sums (qty, price, disc) and one fused pass over price, disc and tax
        alg = col_bytes[0] + col_bytes[1] + col_bytes[2] + (col_bytes[1] + col_bytes[2] + col_bytes[3])

        def step():
            return E.Aggregation.compute_multiple(q1, ds)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    clean = torch.zeros(32 << 20, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(max(args.warmup, 3)):
        step()
    steps = min(args.steps, 100)
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = E.kernel_launches()
    ts = []
    t0 = time.perf_counter()
    for i in range(steps):
        flush.fill_(i & 0xFF)
        clean.sum()
        torch.cuda._sleep(1_000_000)
        ev0.record(stream)
        got = step()
        ev1.record(stream)
        ev1.synchronize()
        ts.append(ev0.elapsed_time(ev1) / 1e3)
    t1 = time.perf_counter()
    sampler.stop()
    launches = E.kernel_launches() - launches0
    t = statistics.median(ts)
    rows_dec = n * len(used)
    peak, peak_kind = measured_peak()
    line = {"metric": "decode+filter+aggregate GB/s (decoded, all columns read)", "value": round(8.0 * rows_dec / t / 1e9, 3),
            "unit": "GB/s", "n_gpus": 1, "steps": steps, "warmup": max(args.warmup, 3), "ms_per_step": round(1e3 * t, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/i64 -> f64",
            "data": "synthetic lineitem-shaped columns (seeded numpy; dbgen's value ranges)",
            "config": {"workload": f"{args.workload}: TPC-H {'Q6' if args.workload == 'tpch_q6' else 'Q1'} shape over "
                                   f"{n} lineitem rows (scale factor {n / 5_998_405:.1f}), BUFF scale 100, "
                                   f"{TPCH_CHUNK}-row chunks", "rows": n, "column_bytes": col_bytes,
                       "l2": "flushed before every step (256 MiB write, then a 256 MiB read of another buffer)"},
            "roofline": {"bound": "hbm", "achieved": round(alg / t / 1e9, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(alg / t / 1e9 / peak, 4), "traffic": None, "scope": "whole step (every launch)",
                         "algorithmic_bytes_per_step": alg, "peak_source": peak_kind},
            "gpu_launches": int(launches), "clocks": sampler.summary(t0, t1), "result": got}
    if not args.no_cpu_baseline:
        from oracle import oracle as O

        m = min(n, 5_998_405)
        sample = [E.encode(c[:m], "buff", ("record_count", TPCH_CHUNK), 100) for c in cols]
        c0 = time.perf_counter()
        tpch_oracle(sample, args.workload, O, m)
        dt = time.perf_counter() - c0
        line["cpu_baseline"] = {"value": round(8.0 * m * len(used) / dt / 1e9, 3), "unit": "GB/s", "cores": 1,
                                "kind": "port", "sample": f"the same query over the first {m} rows (scale factor 1), "
                                                          "the C restatement of ebi's Decoder and Aggregation loops, one thread"}
    if not args.no_parity_check:
        from oracle import oracle as O

        # the reference sums each chunk sequentially in f64; over 16,777,216-row chunks its own rounding
        # error (at most (n - 1) u sum|x| per chunk) exceeds 1e-12, so the check is against both that
        # sequential oracle, within its error bound, and the exactly rounded sum
        want = tpch_oracle(datas, args.workload, O, n)
        exact, mag = tpch_oracle(datas, args.workload, O, n, exact=True)
        u = 2.0 ** -53
        bound = [(TPCH_CHUNK - 1) * u * m + 1e-12 * m for m in mag]
        line["parity_check"] = {
            "sequential_oracle": want, "exact": exact,
            "max_rel_diff_vs_sequential_oracle": max(abs(g - w) / max(abs(w), 1e-300) for g, w in zip(got, want)),
            "max_ulps_from_exact": max(abs(g - e) / max(math.ulp(e), 5e-324) for g, e in zip(got, exact)),
            "within_sequential_oracle_error_bound": bool(all(abs(g - w) <= b for g, w, b in zip(got, want, bound)))}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=6)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=12)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity-check", action="store_true")
    ap.add_argument("--rows", type=int, default=0, help="column length (profiling runs use smaller columns)")
    ap.add_argument("--workload", default="buff", choices=["buff", "gorilla", "chimp128", "rle", "elf", "elf_on_chimp",
                                                               "batched", "serving", "tpch_q6", "tpch_q1"])
    ap.add_argument("--scale", type=float, default=1.0,
                    help="batched / serving: fraction of the configuration's columns to build")
    ap.add_argument("--materialize", action="store_true",
                    help="BUFF workload: measure only the full materialize of the column (C2's second leg)")
    ap.add_argument("--no-configs", action="store_true",
                    help="headline only: skip the other configurations (C1, C2 materialize, C3a, C3b, C4, C5)")
    args = ap.parse_args()
    wl = None
    if args.workload in ("tpch_q6", "tpch_q1"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the TPC-H shapes are measured against the oracle in "
                                                                  "their own line (cpu_baseline)"}))
            return
        run_tpch(args)
        return
    if args.workload in ("batched", "serving"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "batched and serving shapes have no CPU reference path"}))
            return
        (run_batched if args.workload == "batched" else run_serving)(args)
        return
    args.warmup = max(args.warmup, 3)

    if args.impl == "reference":
        run_reference(args)
        return

    import torch

    import ebi_gb300 as E

    rank, local, world = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)

    E.load_library()
    wl = Workload(args.workload, args.rows or DEFAULT_ROWS[args.workload])
    args.rows = wl.rows
    data = wl.build()
    dec = E.Decoder(data, device=str(dev))
    dec.set_timing(True)
    n = dec.n_records
    mask = dec.new_mask()
    qs = wl.queries()
    nq = len(qs)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # 256 MiB > 129 MB L2
    clean = torch.zeros(32 << 20, dtype=torch.float64, device=dev)  # another 256 MiB, read after the write
    alg_bytes = sum(dec.chunk_info(c)[1] for c in range(dec.n_chunks)) + 8 * dec.mask_words
    if args.materialize:
        if rank == 0:
            print(json.dumps(materialize_config(dec, data, dev, args.steps, args.warmup, flush, clean)), flush=True)
        return

    def one_step(i):
        flush.fill_(i & 0xFF)  # evicts the column from L2 (not timed)
        clean.sum()  # reads another 256 MiB: the flush's dirty lines are written back before the query, not during it
        # ~0.5 ms of device spin (not timed): the device is still busy when the
        # host enqueues the query, so its events time device work, not the
        # host's launch latency
        if hasattr(torch.cuda, "_sleep"):
            torch.cuda._sleep(1_000_000)
        dec.filter_agg(qs[i % nq][1], out=mask, aggregates=wl.aggregates)
        return dec.segmented_execution_times()

    for i in range(args.warmup):
        one_step(i)
    props = torch.cuda.get_device_properties(dev)
    sampler = ClockSampler(f"GPU-{props.uuid}" if getattr(props, "uuid", None) else str(local))
    sampler.start()
    time.sleep(0.3)
    barrier()
    launches0 = E.kernel_launches()
    t0 = time.perf_counter()
    scan, total = [], []
    for i in range(args.steps):
        t = one_step(i)
        scan.append(t["scan_ms"])
        total.append(t["total_ms"])
    barrier()
    t1 = time.perf_counter()
    launches = E.kernel_launches() - launches0
    time.sleep(0.2)
    sampler.stop()
    clocks = sampler.summary(t0, t1)

    # value: the median step (BASELINE's "median of >= 20 reps"); the mean is reported beside it
    med_step_s = statistics.median(total) / 1e3
    dev_s, value = replica_throughput(med_step_s * args.steps, n * args.steps, dist, dev)
    _, mean_value = replica_throughput(sum(total) / 1e3, n * args.steps, dist, dev)

    # roofline of the dominant kernel (the fused BUFF filter+sum kernel)
    peak, peak_kind = measured_peak()
    scan_avg_s = statistics.mean(scan) / 1e3
    scan_med_s = statistics.median(scan) / 1e3
    achieved = alg_bytes / scan_avg_s / 1e9
    traffic = ncu_traffic(wl.name)

    # parity spot check of the last query against the oracle (outside the timed region)
    check = None
    if rank == 0 and not args.no_parity_check:
        from oracle import oracle as O
        name, p = qs[(args.steps - 1) % nq]
        _, s, mn, mx, cnt = dec.filter_agg(p, out=mask)
        o = O.Decoder(data, threads=os.cpu_count() or 1)
        om, os_, omn, omx = o.filter_agg(O.rng(1, p.rng.start.value, 1, p.rng.end.value))
        exact_sum = wl.codec == "buff"  # BUFF sums are exact; the others are compensated (1e-12 relative)
        sum_same = s == os_ if exact_sum else abs(s - os_) <= 1e-12 * max(abs(os_), 1e-300)
        same = np.array_equal(mask.cpu().numpy().view(np.uint64), om) and (mn, mx) == (omn, omx) and sum_same
        check = {"query": name, "bitmask_min_max_bit_exact_sum_within_tolerance": bool(same),
                 "sum_rel_diff": abs(s - os_) / max(abs(os_), 1e-300), "rows_selected": int(cnt)}

    # e2e: host file (pinned) -> open (H2D) -> fused query -> bitmask + scalars back to the host
    host_file = torch.frombuffer(bytearray(data), dtype=torch.uint8).pin_memory()
    host_mask = torch.empty(dec.mask_words, dtype=torch.int64).pin_memory()
    e2e_t = []
    for i in range(args.e2e_steps + 2 if args.e2e_steps > 0 else 0):
        torch.cuda.synchronize(dev)
        ts = time.perf_counter()
        d2 = E.Decoder(host_file, device=str(dev))
        m2 = d2.new_mask()
        _, s, mn, mx, cnt = d2.filter_agg(qs[i % nq][1], out=m2, aggregates=wl.aggregates)
        host_mask.copy_(m2, non_blocking=True)
        torch.cuda.synchronize(dev)
        d2.close()
        if i >= 2:
            e2e_t.append(time.perf_counter() - ts)
    e2e_s = statistics.median(e2e_t) if e2e_t else float("nan")
    e2e_val = 8.0 * n * world / e2e_s / 1e9 if e2e_t else None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_figures(data, wl, os.cpu_count() or 1)
    configs = None
    if world == 1 and wl.name == "buff" and not args.no_configs:
        configs = config_results(args, dec, data, dev, flush, clean)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * dev_s / args.steps, 5),
            "mean_value": round(mean_value, 3), "value_statistic": "median step (mean_value: mean step)",
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/u64 -> f64",
            "data": "synthetic (seeded numpy, the configuration's shape)",
            "config": {"workload": wl.describe, "queries": [k for k, _, _ in wl.ranges],
                       "rows": args.rows, "chunk_rows": wl.chunk, "column_bytes": len(data),
                       "l2": "flushed before every step (256 MiB write, then a 256 MiB read of another buffer so no dirty line is written back during the query)",
                       "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic,
                         "kernel": KERNELS[wl.name],
                         "algorithmic_bytes_per_launch": alg_bytes, "avg_launch_ms": round(1e3 * scan_avg_s, 5),
                         "median_launch_ms": round(1e3 * scan_med_s, 5),
                         "frac_at_median_launch": round(alg_bytes / scan_med_s / 1e9 / peak, 4),
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "fallback 6.8 TB/s"},
            "e2e": {"value": round(e2e_val, 3) if e2e_val else None, "unit": UNIT, "h2d_bytes_per_step": len(data),
                    "d2h_bytes_per_step": 8 * dec.mask_words + 48,
                    "ms_per_step": round(1e3 * e2e_s, 3) if e2e_t else None,
                    "path": "ebi_column_open (pinned host file -> HBM) + ebi_filter_agg + bitmask D2H + close"},
            "gpu_launches": int(launches),
            "clocks": clocks,
            "cpu_baseline": cpu,
            "parity_check": check,
            "wall_ms_per_step": round(1e3 * (t1 - t0) / args.steps, 4),
            "configs": configs,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
