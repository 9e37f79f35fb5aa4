"""ctypes binding of libebi_gpu.so (include/ebi_gpu.h).

The library is built in-tree by __graft_entry__.build() into ebi_gb300/_lib/.
There is no fallback: importing the engine without the library raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libebi_gpu.so"

# Every symbol include/ebi_gpu.h declares.
EXPORTS = [
    "ebi_column_open", "ebi_column_open_file", "ebi_column_close", "ebi_column_num_records", "ebi_column_num_chunks",
    "ebi_column_device_bytes", "ebi_column_set_copy_wait",
    "ebi_column_scheme", "ebi_column_chunk_info", "ebi_column_set_precision", "ebi_materialize",
    "ebi_filter", "ebi_filter_materialize", "ebi_sum", "ebi_min", "ebi_max", "ebi_filter_agg",
    "ebi_encode", "ebi_free", "ebi_last_error", "ebi_kernel_launches", "ebi_column_set_timing",
    "ebi_column_last_times", "ebi_materialize_static", "ebi_batch_create", "ebi_batch_run",
    "ebi_batch_get_info", "ebi_batch_get_trials", "ebi_batch_set_tuning_cache", "ebi_batch_destroy", "ebi_server_create", "ebi_server_submit", "ebi_server_poll",
    "ebi_server_replay", "ebi_server_get_stats", "ebi_server_destroy", "ebi_run_plain", "ebi_mask_from_rows",
    "ebi_rows_from_mask", "ebi_aggregate",
]


class Predicate(C.Structure):
    """ebi_predicate"""
    _fields_ = [("kind", C.c_int32), ("start_kind", C.c_int32), ("end_kind", C.c_int32),
                ("reserved", C.c_int32), ("value", C.c_double), ("start", C.c_double),
                ("end", C.c_double)]


class BatchQuery(C.Structure):
    """ebi_batch_query"""
    _fields_ = [("col", C.c_void_p), ("pred", Predicate), ("aggregates", C.c_uint32), ("reserved", C.c_uint32),
                ("d_out_mask", C.c_void_p)]


class BatchResult(C.Structure):
    """ebi_batch_result"""
    _fields_ = [("sum", C.c_double), ("min", C.c_double), ("max", C.c_double), ("count", C.c_uint64),
                ("status", C.c_int32), ("bad_chunk", C.c_uint32)]


class BatchInfo(C.Structure):
    """ebi_batch_info"""
    _fields_ = [("queries", C.c_uint64), ("items", C.c_uint64), ("chunks", C.c_uint64), ("shape", C.c_int32),
                ("ctas_per_sm", C.c_uint32), ("order", C.c_uint32), ("shape_ms", C.c_double * 4),
                ("buff_tiles", C.c_uint32 * 3), ("value_chunks", C.c_uint32 * 3), ("gorilla_chunks", C.c_uint32 * 3),
                ("trials", C.c_uint32), ("from_cache", C.c_uint32), ("best_ms", C.c_double)]


class BatchTrial(C.Structure):
    """ebi_batch_trial"""
    _fields_ = [("knob", C.c_uint32), ("bucket", C.c_uint32), ("value", C.c_uint32), ("kept", C.c_uint32),
                ("ms", C.c_double)]


class Request(C.Structure):
    """ebi_request"""
    _fields_ = [("n_columns", C.c_uint32), ("columns", C.c_uint32 * 8), ("pred", Predicate),
                ("aggregates", C.c_uint32), ("reserved", C.c_uint32)]


class Response(C.Structure):
    """ebi_response"""
    _fields_ = [("ticket", C.c_uint64), ("sum", C.c_double), ("min", C.c_double), ("max", C.c_double),
                ("count", C.c_uint64), ("status", C.c_int32), ("reserved", C.c_uint32),
                ("submit_ns", C.c_uint64), ("launch_ns", C.c_uint64), ("done_ns", C.c_uint64)]


class ServerConfig(C.Structure):
    """ebi_server_config"""
    _fields_ = [("device", C.c_int32), ("slots", C.c_uint32), ("max_queries_per_batch", C.c_uint64),
                ("max_chunks_per_batch", C.c_uint64), ("max_items_per_batch", C.c_uint64),
                ("buff_tiles_per_item", C.c_uint32), ("value_chunks_per_item", C.c_uint32),
                ("gorilla_chunks_per_item", C.c_uint32), ("reserved", C.c_uint32)]


class ServerStats(C.Structure):
    """ebi_server_stats"""
    _fields_ = [("batches", C.c_uint64), ("requests", C.c_uint64), ("max_in_flight", C.c_uint64),
                ("pending", C.c_uint64), ("items", C.c_uint64), ("build_ns", C.c_uint64)]


class SegmentTimes(C.Structure):
    """ebi_segment_times"""
    _fields_ = [("scan_ms", C.c_double), ("finalize_ms", C.c_double), ("total_ms", C.c_double),
                ("kernels", C.c_uint64)]


class ExprNode(C.Structure):
    """ebi_expr_node"""
    _fields_ = [("kind", C.c_int32), ("index", C.c_uint32), ("literal", C.c_double)]


class Aggregation(C.Structure):
    """ebi_aggregation"""
    _fields_ = [("kind", C.c_int32), ("n_nodes", C.c_uint32), ("nodes", C.POINTER(ExprNode)),
                ("d_array", C.c_void_p), ("array_cap", C.c_uint64), ("scalar", C.c_double), ("n_array", C.c_uint64)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() (no CPU fallback exists)")
    L = C.CDLL(str(LIB_PATH))
    vp, u64, i64, u64p, dp = C.c_void_p, C.c_uint64, C.c_int64, C.POINTER(C.c_uint64), C.POINTER(C.c_double)
    PP = C.POINTER(Predicate)
    L.ebi_column_open.argtypes = [C.c_char_p, u64, vp, C.POINTER(vp)]
    L.ebi_column_open_file.argtypes = [C.c_char_p, vp, C.POINTER(vp)]
    L.ebi_aggregate.argtypes = [C.POINTER(vp), C.c_uint32, C.POINTER(Aggregation), C.c_uint32, vp, vp]
    L.ebi_column_close.argtypes = [vp]
    L.ebi_column_set_copy_wait.argtypes = [vp, C.c_int64]
    for fn in (L.ebi_column_num_records, L.ebi_column_num_chunks, L.ebi_column_device_bytes):
        fn.argtypes = [vp]
        fn.restype = u64
    L.ebi_column_scheme.argtypes = [vp]
    L.ebi_column_chunk_info.argtypes = [vp, u64, u64p, u64p, u64p, u64p]
    L.ebi_column_set_precision.argtypes = [vp, C.c_int32]
    L.ebi_materialize.argtypes = [vp, vp, i64, vp, u64, u64p, vp]
    L.ebi_materialize_static.argtypes = [vp, vp, i64, vp, u64, u64p, vp]
    L.ebi_filter.argtypes = [vp, PP, vp, i64, vp, vp]
    L.ebi_filter_materialize.argtypes = [vp, PP, vp, i64, vp, u64, u64p, vp]
    for fn in (L.ebi_sum, L.ebi_min, L.ebi_max):
        fn.argtypes = [vp, vp, i64, dp, vp]
    L.ebi_filter_agg.argtypes = [vp, PP, vp, i64, vp, dp, dp, dp, u64p, vp]
    L.ebi_encode.argtypes = [dp, u64, C.c_int, C.c_int, u64, u64, C.POINTER(C.POINTER(C.c_uint8)), u64p]
    L.ebi_free.argtypes = [vp]
    L.ebi_last_error.restype = C.c_char_p
    L.ebi_kernel_launches.restype = u64
    L.ebi_column_set_timing.argtypes = [vp, C.c_int]
    L.ebi_column_last_times.argtypes = [vp, C.POINTER(SegmentTimes)]
    L.ebi_batch_create.argtypes = [C.POINTER(BatchQuery), u64, vp, C.POINTER(vp)]
    L.ebi_batch_run.argtypes = [vp, PP, C.POINTER(BatchResult), vp]
    L.ebi_batch_get_info.argtypes = [vp, C.POINTER(BatchInfo)]
    L.ebi_batch_get_trials.argtypes = [vp, C.POINTER(BatchTrial), C.c_uint32, C.POINTER(C.c_uint32)]
    L.ebi_batch_set_tuning_cache.argtypes = [C.c_char_p]
    L.ebi_batch_destroy.argtypes = [vp]
    RQ, RS = C.POINTER(Request), C.POINTER(Response)
    L.ebi_server_create.argtypes = [C.POINTER(vp), C.c_uint32, C.POINTER(ServerConfig), C.POINTER(vp)]
    L.ebi_server_submit.argtypes = [vp, RQ, u64p]
    L.ebi_server_poll.argtypes = [vp, RS, C.c_uint32, C.POINTER(C.c_uint32)]
    L.ebi_server_replay.argtypes = [vp, RQ, u64p, u64, RS]
    L.ebi_server_get_stats.argtypes = [vp, C.POINTER(ServerStats)]
    L.ebi_server_destroy.argtypes = [vp]
    L.ebi_mask_from_rows.argtypes = [vp, u64, u64, vp, vp]
    L.ebi_rows_from_mask.argtypes = [vp, u64, vp, u64, u64p, vp]
    L.ebi_run_plain.argtypes = [C.POINTER(vp), C.c_uint32, RQ, u64, RS, vp]
    _lib = L
    return L
