/*
 * ebi_gpu.h -- C ABI of the GB300 engine for lemolatoon/ebi's chunked
 * decode-and-query path (EBI1 files; Gorilla, Chimp, Chimp128, BUFF, RLE and
 * Uncompressed chunks).
 *
 * The entry points mirror ebi's public Decoder (ebi/src/api/decoder.rs) and
 * Encoder (ebi/src/api/encoder.rs); each declaration cites the reference item
 * it replaces.  A binding in the reference's own language is a thin `extern
 * "C"` block over these functions.
 *
 * Conventions
 *  - Every function returns an ebi_status; 0 is success.  The codes mirror
 *    DecoderError (ebi/src/decoder/error.rs:6-21).  When several chunks fail,
 *    the status of the first failing chunk in chunk order is returned, as the
 *    reference's sequential chunk loop would.
 *  - A column keeps the whole EBI1 file resident in device memory from
 *    ebi_column_open until ebi_column_close.
 *  - Bitmasks are dense arrays of ceil(n_records / 64) little-endian uint64
 *    words in DEVICE memory; bit (r % 64) of word (r / 64) is row r.  They
 *    stand for the reference's RoaringBitmap of global u32 row ids.  NULL
 *    means None.
 *  - chunk_id < 0 means None (all chunks); otherwise only that chunk is read,
 *    as Decoder::*(.., Some(ChunkId)) does.
 *  - Bulk outputs (bitmasks, materialized values) are DEVICE pointers;
 *    scalar outputs (sums, counts) are HOST pointers and the call waits for
 *    its stream before returning them.
 *  - `stream` is a cudaStream_t (NULL = the legacy default stream).  Calls on
 *    one column must not overlap: a column owns one set of query scratch.
 */
#ifndef EBI_GPU_H
#define EBI_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    EBI_OK = 0,
    EBI_E_IO = 1,             /* DecoderError::IO: the file is shorter than its own offsets say  */
    EBI_E_CONVERSION = 2,     /* DecoderError::ConversionError: bad field type / scheme / option */
    EBI_E_UNEXPECTED_END = 3, /* DecoderError::UnexpectedEndOfChunk                              */
    EBI_E_PRECONDITION = 4,   /* DecoderError::PreconditionsNotMet                               */
    EBI_E_CUDA = 5,           /* DecoderError::CudaError                                         */
    EBI_E_CORRUPT = 6,        /* a stream breaks an invariant the reference asserts in debug     */
    EBI_E_INVALID = 7,        /* bad argument (e.g. output buffer too small)                     */
    EBI_E_OOM = 8,            /* device or host allocation failed                                */
    EBI_E_UNSUPPORTED = 9     /* codec outside this engine (Sprintz, zstd, gzip, ...)            */
} ebi_status;

/* CompressionScheme (ebi/src/format.rs:185-199) */
enum { EBI_UNCOMPRESSED = 0, EBI_RLE = 1, EBI_BUFF = 2, EBI_GORILLA = 3, EBI_CHIMP = 4, EBI_CHIMP128 = 5,
       EBI_ELF_ON_CHIMP = 6, EBI_ELF = 7 };
/* ChunkOptionKind (ebi/src/format.rs:174-180) */
enum { EBI_CHUNK_FULL = 0, EBI_CHUNK_RECORD_COUNT = 1, EBI_CHUNK_BYTE_SIZE = 2 };
/* Predicate / RangeValue kinds (ebi/src/decoder/query.rs:352-428) */
enum { EBI_PRED_EQ = 0, EBI_PRED_NE = 1, EBI_PRED_RANGE = 2 };
enum { EBI_BOUND_NONE = 0, EBI_BOUND_INCLUSIVE = 1, EBI_BOUND_EXCLUSIVE = 2 };

/* Predicate = PredicateImpl<f64>::{Eq(v), Ne(v), Range{start, end}} (query.rs:422-437). */
typedef struct {
    int32_t kind;       /* EBI_PRED_*                          */
    int32_t start_kind; /* EBI_BOUND_* of Range::start         */
    int32_t end_kind;   /* EBI_BOUND_* of Range::end           */
    int32_t reserved;   /* 0                                   */
    double value;       /* operand of Eq / Ne                  */
    double start;       /* RangeValue payload of Range::start  */
    double end;         /* RangeValue payload of Range::end    */
} ebi_predicate;

typedef struct ebi_column ebi_column;

/* ---- open / inspect ------------------------------------------------------ */

/* Decoder::new (api/decoder.rs:136-156) over an in-memory EBI1 file: parses
 * the header and footer (FileReader::fetch_header/fetch_footer,
 * decoder.rs:131-220) and copies the file to device memory on `stream`.
 * `file` may be pageable or pinned host memory; it is not used after return. */
int ebi_column_open(const uint8_t* file, uint64_t len, void* stream, ebi_column** out);
/* Decoder::new(DecoderInput::from_file(path)) (api/decoder.rs:136-156,
 * DecoderInput::from_file :66-79): reads the EBI1 file at `path` into a
 * process-wide pinned staging buffer and opens it as ebi_column_open does
 * (BUFF planes go from that buffer to HBM in one device pass).  A file that
 * cannot be opened or read is EBI_E_IO.  Opens from several threads take
 * turns on the staging buffer. */
int ebi_column_open_file(const char* path, void* stream, ebi_column** out);
/* Drops the device copy (Decoder going out of scope). */
int ebi_column_close(ebi_column* col);

/* NativeFileFooter::{number_of_records, number_of_chunks} (format/native.rs:117-124) */
uint64_t ebi_column_num_records(const ebi_column* col);
uint64_t ebi_column_num_chunks(const ebi_column* col);
/* Device memory the column holds, in bytes: the resident file, its tables and
 * the query scratch it allocated on first use.  No counterpart in the
 * reference (its Decoder reads from host memory). */
uint64_t ebi_column_device_bytes(const ebi_column* col);
/* Limit, in SM clock cycles, of the bounded waits with which the column's
 * kernels wait for their bulk copies (shared-memory staging of BUFF tiles
 * whose chunks are wider than 32 bits or constant, and of Gorilla chunks):
 * a query whose copy has not landed by then fails with EBI_E_CUDA instead of
 * waiting on, and the column stays usable.  Negative restores the default
 * (about two seconds); 0 makes each such wait a single look.  A kernel still
 * waits out its copies in flight (full limit) before it exits.  No
 * counterpart in the reference (its reader has no device copies to wait
 * for); for failure-path tests and for callers that want a query to give up
 * early. */
int ebi_column_set_copy_wait(ebi_column* col, int64_t cycles);
/* NativeFileConfig::compression_scheme (format/native.rs:45-49) */
int ebi_column_scheme(const ebi_column* col);
/* GeneralChunkHandle::{physical_offset, chunk_size, logical_offset,
 * number_of_records} (decoder.rs:283-328) */
int ebi_column_chunk_info(const ebi_column* col, uint64_t chunk, uint64_t* physical_offset,
                          uint64_t* size, uint64_t* logical_offset, uint64_t* n_records);
/* Decoder::with_precision (api/decoder.rs:159-161): BUFF materialization keeps
 * only the byte planes needed for `precision` decimal digits
 * (buff/controlled_precision.rs:5-75).  precision < 0 restores full precision. */
int ebi_column_set_precision(ebi_column* col, int32_t precision);

/* ---- queries (Decoder methods, api/decoder.rs:202-439) -------------------- */

/* Decoder::materialize: decoded values of the rows in `mask` (all rows when
 * NULL), in row order, to d_out[0 .. *n_out).  When more than out_cap values
 * qualify it writes nothing past out_cap, sets *n_out to the number needed
 * and fails with EBI_E_INVALID, so the caller can retry with a larger buffer
 * (decoded chunks may hold more values than their footer's row count). */
int ebi_materialize(ebi_column* col, const uint64_t* d_mask, int64_t chunk_id, double* d_out,
                    uint64_t out_cap, uint64_t* n_out, void* stream);

/* ebi_materialize without any allocation (no reference counterpart: the
 * reference's Decoder allocates freely).  Same arguments, results and errors
 * as ebi_materialize, but its per-tile scratch lives in a fixed device array
 * of 16,384 tiles (tiles are 8,192-row slices of a BUFF chunk, or whole chunks
 * of the other codecs) instead of column memory allocated on first use; a
 * query covering more tiles fails with EBI_E_INVALID before touching the GPU.
 * It is for callers that must not allocate device memory, e.g. a serving
 * thread whose latency must not include the allocator, or a process whose
 * device memory is fully reserved by another allocator.  The first call on
 * each device looks up the array's address (cudaGetSymbolAddress, with that
 * device current); make that first call before any stream capture.  The array
 * is shared by every column on a device: calls that overlap in time (other
 * streams or host threads) race on it and must be serialised by the caller.
 * The column's device must be current (else EBI_E_INVALID). */
int ebi_materialize_static(ebi_column* col, const uint64_t* d_mask, int64_t chunk_id, double* d_out,
                           uint64_t out_cap, uint64_t* n_out, void* stream);

/* Decoder::filter: rows (of `mask` when given) whose value satisfies `pred`,
 * as a bitmask in d_out_mask (ceil(n_records/64) words, fully written). */
int ebi_filter(ebi_column* col, const ebi_predicate* pred, const uint64_t* d_mask, int64_t chunk_id,
               uint64_t* d_out_mask, void* stream);

/* Decoder::filter_materialize: the values of the rows ebi_filter selects. */
int ebi_filter_materialize(ebi_column* col, const ebi_predicate* pred, const uint64_t* d_mask,
                           int64_t chunk_id, double* d_out, uint64_t out_cap, uint64_t* n_out,
                           void* stream);

/* Decoder::sum / min / max over the rows of `mask` (all when NULL).  Sums of
 * BUFF chunks are exact integer sums rounded once, as the reference computes
 * them; sums of Gorilla/Chimp/Chimp128/RLE/Uncompressed chunks are
 * compensated (Neumaier) sums, within 1e-12 of the reference's sequential f64
 * sum relative to the sum of magnitudes, and within 2 ulps of the exact sum. */
int ebi_sum(ebi_column* col, const uint64_t* d_mask, int64_t chunk_id, double* out, void* stream);
int ebi_min(ebi_column* col, const uint64_t* d_mask, int64_t chunk_id, double* out, void* stream);
int ebi_max(ebi_column* col, const uint64_t* d_mask, int64_t chunk_id, double* out, void* stream);

/* Fused Decoder::filter followed by Decoder::{sum,min,max}(Some(&result)),
 * reading each chunk once.  Any output may be NULL.  n_selected receives the
 * number of rows in the filter result. */
int ebi_filter_agg(ebi_column* col, const ebi_predicate* pred, const uint64_t* d_mask,
                   int64_t chunk_id, uint64_t* d_out_mask, double* sum, double* min, double* max,
                   uint64_t* n_selected, void* stream);

/* ---- row sets ------------------------------------------------------------- */
/* The reference passes row sets as RoaringBitmap (ascending u32 row ids,
 * decoder/query.rs:199-238); the engine takes dense device bitmasks.  These
 * convert on the device, so a binding hands over RoaringBitmap::iter's ids:
 * ebi_mask_from_rows sets the bit of every id (any order, duplicates allowed;
 * ids >= n_records are dropped, as no chunk holds them) in a zeroed mask of
 * ceil(n_records / 64) words; ebi_rows_from_mask writes the set rows in
 * ascending order (RoaringBitmap::iter order) to d_rows[0 .. *n_out), or sets
 * *n_out to the number needed and fails with EBI_E_INVALID when cap is short. */
int ebi_mask_from_rows(const uint32_t* d_rows, uint64_t n_rows, uint64_t n_records, uint64_t* d_mask, void* stream);
int ebi_rows_from_mask(const uint64_t* d_mask, uint64_t n_records, uint32_t* d_rows, uint64_t cap, uint64_t* n_out,
                       void* stream);

/* ---- batched queries ------------------------------------------------------ */
/* No reference counterpart: the reference answers one Decoder call at a time
 * (its chunk loop, api/decoder.rs:243-281, is what a batch replaces).
 * A batch is a fixed list of filter + aggregate queries, each over one open
 * column (columns may repeat and mix codecs).  Running it executes every
 * query's chunks in one persistent mixed-codec launch followed by one fold
 * launch, captured once into a CUDA graph and replayed.  The first run tunes
 * the launch by timing graph replays: the persistent CTAs per SM and the work
 * items' order, then, for each codec family and column-size bucket in the
 * batch, how many 8,192-row BUFF tiles, RLE / Uncompressed chunks or Gorilla
 * chunks one work item covers; the fastest is kept (and, with a tuning cache
 * set, stored under the batch's column shape for later batches).  Results
 * equal the single-column calls (ebi_filter_agg) bit for bit whatever the
 * tiling.  Queries over the same column run together: a Chimp-family chunk
 * is decoded once for up to 32 of them and a Gorilla chunk group walked once
 * for up to 8.  The columns must stay open while the batch exists; runs of one
 * batch must not overlap. */
enum { EBI_AGG_SUM = 1, EBI_AGG_MIN = 2, EBI_AGG_MAX = 4 };
typedef struct {
    ebi_column* col;
    ebi_predicate pred;
    uint32_t aggregates;   /* EBI_AGG_* bits; the selected-row count is always kept */
    uint32_t reserved;
    uint64_t* d_out_mask;  /* device bitmask of the filter result, or NULL */
} ebi_batch_query;
typedef struct {
    double sum, min, max;
    uint64_t count;        /* rows selected */
    int32_t status;        /* ebi_status of this query (first failing chunk) */
    uint32_t bad_chunk;
} ebi_batch_result;
/* Column-size buckets of the tiling: 0: < 262,144 rows, 1: < 4,194,304, 2: larger. */
typedef struct {
    uint64_t queries, items, chunks;   /* items: work items of the chosen tiling (0 before the first run) */
    int32_t shape;         /* launch shape chosen by the first run (-1 before):
                              0: 2 CTAs/SM cost order, 1: 1 CTA/SM cost order, 2: 2 CTAs/SM query order, 3: 1 CTA/SM query order */
    uint32_t ctas_per_sm, order;
    double shape_ms[4];    /* device time of each candidate shape on the default tiling */
    uint32_t buff_tiles[3];      /* chosen BUFF tiles per item, per size bucket */
    uint32_t value_chunks[3];    /* chosen RLE / Uncompressed chunks per item */
    uint32_t gorilla_chunks[3];  /* chosen Gorilla chunks per item (one warp walks each) */
    uint32_t trials;       /* candidates timed by the first run (0: taken from the tuning cache) */
    uint32_t from_cache;   /* 1: the configuration came from the tuning cache */
    double best_ms;        /* device time of one run with the chosen configuration */
} ebi_batch_info;
/* One timed candidate of the first run.  knob 0: launch shape (value =
 * ctas_per_sm * 2 + order, bucket 0); 1: BUFF tiles per item; 2: RLE /
 * Uncompressed chunks per item; 3: Gorilla chunks per item (value = the count,
 * for the bucket).  kept: the candidate was the fastest so far and stayed. */
typedef struct {
    uint32_t knob, bucket, value, kept;
    double ms;
} ebi_batch_trial;
typedef struct ebi_batch ebi_batch;
int ebi_batch_create(const ebi_batch_query* queries, uint64_t n, void* stream, ebi_batch** out);
/* preds (n entries, may be NULL) replace the queries' predicates for this and
 * later runs; results (n entries, may be NULL) receive each query's result. */
int ebi_batch_run(ebi_batch* batch, const ebi_predicate* preds, ebi_batch_result* results, void* stream);
int ebi_batch_get_info(const ebi_batch* batch, ebi_batch_info* out);
/* Copies up to max of the first run's timed candidates, in the order timed. */
int ebi_batch_get_trials(const ebi_batch* batch, ebi_batch_trial* out, uint32_t max, uint32_t* n_out);
/* Process-wide tuning cache: a JSON file mapping a batch's column shape (the
 * SM count and the number of queries per codec and size bucket) to the chosen
 * configuration.  Batches whose first run finds their shape there skip the
 * timing; new choices are written back.  NULL (the default) turns it off. */
int ebi_batch_set_tuning_cache(const char* path);
int ebi_batch_destroy(ebi_batch* batch);

/* ---- serving loop ----------------------------------------------------------- */
/* No reference counterpart (the reference has no server).  A request is a
 * predicate and the aggregates wanted over 1..8 columns of the server; its
 * result combines the per-column filter_agg results in column order (sum of
 * sums, min of mins, max of maxes, total count) and equals that combination
 * computed one column at a time with ebi_filter_agg, bit for bit; aggregates
 * not asked for come back as NaN.
 *
 * A dispatcher thread keeps `slots` batches in flight, each on its own stream.
 * Whenever a slot is free it admits queued requests in arrival order while the
 * slot's capacity lasts (queries, per-chunk accumulators and work items: a
 * request's memory footprint), launches them as one mixed-codec batch, and
 * hands back each request's result with its submit / launch / completion
 * times.  Requests arriving while batches run go into the next free slot, so
 * batches overlap on the device.  The columns must stay open while the server
 * exists. */
typedef struct {
    uint32_t n_columns;     /* 1..8 */
    uint32_t columns[8];    /* indices into the server's column list */
    ebi_predicate pred;
    uint32_t aggregates;    /* EBI_AGG_* bits */
    uint32_t reserved;
} ebi_request;
typedef struct {
    uint64_t ticket;        /* from ebi_server_submit (ebi_run_plain: the request index) */
    double sum, min, max;
    uint64_t count;
    int32_t status;
    uint32_t reserved;
    uint64_t submit_ns, launch_ns, done_ns;  /* steady-clock times */
} ebi_response;
typedef struct {
    int32_t device;
    uint32_t slots;                  /* batches in flight (streams) */
    uint64_t max_queries_per_batch;  /* column queries per batch */
    uint64_t max_chunks_per_batch;   /* per-chunk accumulators per batch */
    uint64_t max_items_per_batch;    /* work items per batch */
    /* work-item tiling (0: the default) */
    uint32_t buff_tiles_per_item;     /* 8,192-row BUFF tiles per item (default 8, at most 16) */
    uint32_t value_chunks_per_item;   /* RLE / Uncompressed chunks per item (default 8, at most 16) */
    uint32_t gorilla_chunks_per_item; /* Gorilla chunks per item, one warp walks each (default 16, at most 64) */
    uint32_t reserved;
} ebi_server_config;
typedef struct {
    uint64_t batches, requests, max_in_flight, pending;
    uint64_t items;     /* work items launched */
    uint64_t build_ns;  /* dispatcher time spent building batches (host) */
} ebi_server_stats;
typedef struct ebi_server ebi_server;
int ebi_server_create(ebi_column* const* columns, uint32_t n_columns, const ebi_server_config* config,
                      ebi_server** out);
int ebi_server_submit(ebi_server* server, const ebi_request* req, uint64_t* ticket);
/* Moves up to `max` finished responses to out (any order); *n_out = how many. */
int ebi_server_poll(ebi_server* server, ebi_response* out, uint32_t max, uint32_t* n_out);
/* Open-loop load: submits reqs[i] at arrival_ns[i] nanoseconds after the call
 * starts (NULL: all at once) and waits for every response; out[i] answers reqs[i]. */
int ebi_server_replay(ebi_server* server, const ebi_request* reqs, const uint64_t* arrival_ns, uint64_t n,
                      ebi_response* out);
int ebi_server_get_stats(ebi_server* server, ebi_server_stats* out);
int ebi_server_destroy(ebi_server* server);
/* The same requests answered one at a time with ebi_filter_agg per column
 * (plain per-query launches), on the calling thread. */
int ebi_run_plain(ebi_column* const* columns, uint32_t n_columns, const ebi_request* reqs, uint64_t n,
                  ebi_response* out, void* stream);

/* ---- multi-column aggregation ---------------------------------------------- */

/* Expr (decoder/expr.rs:31-40) in postfix order: an EBI_EXPR_INDEX node
 * (column `index` of the call's column list) or an EBI_EXPR_LITERAL node
 * pushes a value; an operator node pops rhs, then lhs, and pushes lhs OP rhs
 * (Op::doit, expr.rs:19-28: one IEEE f64 operation, never fused). */
enum { EBI_EXPR_INDEX = 0, EBI_EXPR_LITERAL = 1, EBI_EXPR_ADD = 2, EBI_EXPR_SUB = 3, EBI_EXPR_MUL = 4,
       EBI_EXPR_DIV = 5 };
#define EBI_EXPR_MAX_NODES 64
typedef struct {
    int32_t kind;     /* EBI_EXPR_*              */
    uint32_t index;   /* EBI_EXPR_INDEX: column  */
    double literal;   /* EBI_EXPR_LITERAL: value */
} ebi_expr_node;

/* AggregationKind (api/decoder.rs:755-761) */
enum { EBI_AGGR_NONE = 0, EBI_AGGR_MAX = 1, EBI_AGGR_MIN = 2, EBI_AGGR_SUM = 3 };

/* Aggregation { kind, expr } (api/decoder.rs:840-856) with its result:
 * AggregationResult::Scalar in `scalar`, or for EBI_AGGR_NONE the
 * AggregationResult::Array written to the DEVICE buffer d_array (array_cap
 * values; n_array is the count, set even when the buffer is too small). */
typedef struct {
    int32_t kind;                 /* EBI_AGGR_*                                */
    uint32_t n_nodes;             /* 1 .. EBI_EXPR_MAX_NODES                   */
    const ebi_expr_node* nodes;   /* host, postfix                             */
    double* d_array;              /* EBI_AGGR_NONE: device output              */
    uint64_t array_cap;
    double scalar;                /* out: Max / Min / Sum                      */
    uint64_t n_array;             /* out: EBI_AGGR_NONE                        */
} ebi_aggregation;

/* Aggregation::compute_multiple (api/decoder.rs:881-916); n_aggs = 1 is
 * Aggregation::compute (:858-879).  An aggregation whose expression is a bare
 * Index runs that column's own sum / min / max (in-situ, as
 * AggregationKind::dispatch does); the others are evaluated chunk by chunk
 * over cols[0]'s chunk count: in chunk i every Index leaf stands for the
 * values of its column's chunk i selected by the mask, the operands of an
 * operator are zipped to the shorter one (Expr::compute_chunk,
 * expr.rs:67-135), and the chunk results combine in chunk order
 * (AggregationResult::concat).  Sums: on chunk-aligned BUFF columns whose
 * intermediates provably stay below 2^53 (integer evaluation) the exactly
 * rounded sum; otherwise within 16 eps of the exact sum relative to the sum
 * of magnitudes.  Against the reference's per-chunk sequential f64 sums the
 * difference stays within their own rounding-error bound, (n - 1) 2^-53 of
 * the magnitudes per chunk of n values: below 1e-12 for chunks up to 9,007
 * values.  Min / max ignore NaN operands as f64::min / f64::max do.
 * d_mask (device, NULL = None) covers the rows of every column read.
 * Errors: EBI_E_PRECONDITION for a Literal root or an operator over two
 * literals (when cols[0] has chunks); EBI_E_INVALID where the reference
 * panics (an index past n_cols, a column with fewer chunks than cols[0]) or
 * for a malformed program; EBI_E_UNSUPPORTED for EBI_AGGR_NONE over a bare
 * Index (the reference's todo!()). */
int ebi_aggregate(ebi_column* const* cols, uint32_t n_cols, ebi_aggregation* aggs, uint32_t n_aggs,
                  const uint64_t* d_mask, void* stream);

/* ---- encoder (host) -------------------------------------------------------- */

/* Encoder::new(.., chunk_option, compressor_config).encode()
 * (api/encoder.rs:121-178) on an in-memory f64 column.  `scale` is the BUFF
 * scale (ignored by the other codecs).  The result is malloc'ed; release it
 * with ebi_free.  The two timing fields of the footer are written as zero. */
int ebi_encode(const double* values, uint64_t n, int scheme, int chunk_kind, uint64_t chunk_value,
               uint64_t scale, uint8_t** out, uint64_t* out_len);
void ebi_free(void* p);

/* ---- diagnostics ------------------------------------------------------------ */

/* Device time of the last query on a column, by segment, in milliseconds
 * (the counterpart of Decoder::segmented_execution_times, api/decoder.rs:163-166,
 * and SegmentKind, time.rs:11-22).  `scan` covers the codec kernels that read
 * the chunks (decode, compare, aggregate: the reference's Xor / BitPacking /
 * Decompression + CompareInsert + Sum segments), `finalize` the chunk-ordered
 * fold, `total` the whole query from its first enqueued operation (output
 * clears and chunk selection included).  Filled only while timing is enabled
 * (CUDA events on the query's stream). */
typedef struct {
    double scan_ms;
    double finalize_ms;
    double total_ms;
    uint64_t kernels;  /* kernels the query launched */
} ebi_segment_times;
int ebi_column_set_timing(ebi_column* col, int enable);
int ebi_column_last_times(const ebi_column* col, ebi_segment_times* out);

/* Message of the last error raised on this thread (empty when none). */
const char* ebi_last_error(void);
/* Number of kernels this library launched since load (for launch accounting). */
uint64_t ebi_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif /* EBI_GPU_H */
