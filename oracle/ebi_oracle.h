/*
 * ebi_oracle.h -- CPU restatement of lemolatoon/ebi's chunked decode-and-query path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the GPU
 * engine in ebi_gb300/ and the timed CPU baseline ("port") of bench.py.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it;
 * the product never links or calls it.
 *
 * It restates, in plain C, the reference's
 *   - EBI1 file writer/reader          (ebi/src/encoder.rs, ebi/src/decoder.rs, ebi/src/format*.rs)
 *   - encoders                          (ebi/src/compressor/{gorilla,chimp,chimp_n,buff,run_length,uncompressed}.rs)
 *   - decoders and in-situ operators    (ebi/src/decoder/chunk_reader/ and its buff/ directory)
 *   - the Decoder chunk loop            (ebi/src/api/decoder.rs:202-439)
 *   - the default operators             (ebi/src/decoder/query.rs:14-154)
 * Bitmasks are dense little-endian u64 words over global row ids; bit r%64 of
 * word r/64 is row r.  They stand in for the reference's RoaringBitmap (the
 * same set of u32 row ids).
 *
 * Parity pin: the known-answer vectors held by the reference's own tests
 * (tests/golden/kat.json, generated by tests/golden/make_golden.py).
 */
#ifndef EBI_ORACLE_H
#define EBI_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes; same numbering as include/ebi_gpu.h. */
enum {
    ORA_OK = 0,
    ORA_E_IO = 1,              /* DecoderError::IO (short read)              */
    ORA_E_CONVERSION = 2,      /* DecoderError::ConversionError              */
    ORA_E_UNEXPECTED_END = 3,  /* DecoderError::UnexpectedEndOfChunk         */
    ORA_E_PRECONDITION = 4,    /* DecoderError::PreconditionsNotMet          */
    ORA_E_CORRUPT = 6,         /* stream breaks an invariant (debug panic)   */
    ORA_E_INVALID = 7,         /* bad argument                               */
    ORA_E_OOM = 8
};

enum { ORA_UNCOMPRESSED = 0, ORA_RLE = 1, ORA_BUFF = 2, ORA_GORILLA = 3, ORA_CHIMP = 4, ORA_CHIMP128 = 5,
       ORA_ELF_ON_CHIMP = 6, ORA_ELF = 7 };
enum { ORA_CHUNK_FULL = 0, ORA_CHUNK_RECORD_COUNT = 1, ORA_CHUNK_BYTE_SIZE = 2 };
enum { ORA_PRED_EQ = 0, ORA_PRED_NE = 1, ORA_PRED_RANGE = 2 };
enum { ORA_BOUND_NONE = 0, ORA_BOUND_INCLUSIVE = 1, ORA_BOUND_EXCLUSIVE = 2 };

/* Predicate = PredicateImpl<f64> {Eq, Ne, Range{start, end}} (query.rs:352-446). */
typedef struct {
    int32_t kind;        /* ORA_PRED_*            */
    int32_t start_kind;  /* ORA_BOUND_* (Range)   */
    int32_t end_kind;    /* ORA_BOUND_* (Range)   */
    int32_t reserved;
    double value;        /* Eq / Ne operand       */
    double start;
    double end;
} ora_pred;

typedef struct ora_file ora_file;

/* ---- encoder: Encoder::encode (api/encoder.rs:140-178) ---------------- */
int ora_encode(const double* values, uint64_t n, int scheme, int chunk_kind,
               uint64_t chunk_value, uint64_t scale, uint8_t** out, uint64_t* out_len);
void ora_free(void* p);

/* ---- decoder: Decoder::new (api/decoder.rs:136-156) ------------------- */
int ora_open(const uint8_t* file, uint64_t len, ora_file** out);
void ora_close(ora_file* f);
uint64_t ora_num_records(const ora_file* f);
uint64_t ora_num_chunks(const ora_file* f);
int ora_scheme(const ora_file* f);
/* chunk geometry: GeneralChunkHandle (decoder.rs:283-352) */
int ora_chunk_info(const ora_file* f, uint64_t i, uint64_t* phys_off, uint64_t* size,
                   uint64_t* row_off, uint64_t* n_rows);
/* Decoder::with_precision (api/decoder.rs:159-161); -1 clears it. */
void ora_set_precision(ora_file* f, int32_t precision);

/* Operators.  mask may be NULL (= None); chunk_id < 0 means None.
 * threads <= 1 runs the reference's single-threaded chunk loop; > 1 decodes
 * chunks in parallel and combines in chunk order (identical results). */
int ora_materialize(ora_file* f, const uint64_t* mask, int64_t chunk_id, double* out,
                    uint64_t out_cap, uint64_t* n_out, int threads);
int ora_filter(ora_file* f, const ora_pred* p, const uint64_t* mask, int64_t chunk_id,
               uint64_t* out_mask, int threads);
int ora_filter_materialize(ora_file* f, const ora_pred* p, const uint64_t* mask,
                           int64_t chunk_id, double* out, uint64_t out_cap, uint64_t* n_out,
                           int threads);
int ora_sum(ora_file* f, const uint64_t* mask, int64_t chunk_id, double* out, int threads);
int ora_min(ora_file* f, const uint64_t* mask, int64_t chunk_id, double* out, int threads);
int ora_max(ora_file* f, const uint64_t* mask, int64_t chunk_id, double* out, int threads);
/* filter -> sum/min/max over the filter result, as the two-call sequence
 * Decoder::filter then Decoder::{sum,min,max}(Some(&result)) computes it,
 * but reading each chunk once.  Any output pointer may be NULL. */
int ora_filter_agg(ora_file* f, const ora_pred* p, const uint64_t* mask, int64_t chunk_id,
                   uint64_t* out_mask, double* sum, double* mn, double* mx, int threads);

/* ---- multi-column aggregation (api/decoder.rs:755-917, decoder/expr.rs) ---
 * Expr (expr.rs:31-40) in postfix order: INDEX and LITERAL nodes push a
 * value, an operator node pops rhs, then lhs, and pushes lhs OP rhs
 * (Op::doit, expr.rs:19-28). */
enum { ORA_EXPR_INDEX = 0, ORA_EXPR_LITERAL = 1, ORA_EXPR_ADD = 2, ORA_EXPR_SUB = 3, ORA_EXPR_MUL = 4,
       ORA_EXPR_DIV = 5 };
typedef struct { int32_t kind; uint32_t index; double literal; } ora_expr_node;
/* AggregationKind (api/decoder.rs:755-761) */
enum { ORA_AGGR_NONE = 0, ORA_AGGR_MAX = 1, ORA_AGGR_MIN = 2, ORA_AGGR_SUM = 3 };
/* Aggregation::compute (api/decoder.rs:858-879): an Index expression runs
 * that decoder's sum / min / max; any other expression is evaluated chunk by
 * chunk over files[0]'s chunk count (Expr::compute_chunk, expr.rs:67-135:
 * each Index leaf materializes its file's chunk under the mask, operands are
 * zipped to the shorter one), aggregated per chunk (dispatch_on_vec) and
 * combined in chunk order (AggregationResult::concat).  NONE writes the
 * concatenated values to array (cap values; *n_array is set even when cap is
 * too small, which fails with ORA_E_INVALID).  Errors: PRECONDITION for a
 * Literal root or an operator over two literals, INVALID where the reference
 * panics (index out of range, a file with fewer chunks than files[0]) or
 * reaches todo!() (NONE over an Index root). */
int ora_aggregate(ora_file* const* files, uint32_t n_files, int kind, const ora_expr_node* nodes,
                  uint32_t n_nodes, const uint64_t* mask, double* scalar, double* array, uint64_t cap,
                  uint64_t* n_array);

/* ---- building blocks exposed for known-answer tests ---------------------- */
/* BufferedBitReader::read_bits over buf (io/bit_read.rs:293-318); returns 1
 * and the value, or 0 when fewer than n bits remain.  *bitpos advances. */
int ora_read_bits(const uint8_t* buf, uint64_t len, uint64_t* bitpos, int n, uint64_t* out);
/* Raw chunk bitstream of one codec over values (no file framing). */
int ora_encode_chunk(const double* values, uint64_t n, int scheme, uint64_t scale,
                     uint8_t** out, uint64_t* out_len);
/* Decodes one raw chunk; returns the decoded count in *n_out. */
int ora_decode_chunk(const uint8_t* chunk, uint64_t len, int scheme, uint64_t n_rows,
                     double* out, uint64_t out_cap, uint64_t* n_out);
/* into_fixed_representation_with_fractional_part_bits_length (compression_common/buff.rs:40-51) */
int64_t ora_buff_fixed(double v, int32_t frac_bits);
/* precision for a BUFF scale (compressor/buff.rs:131-135) */
int32_t ora_buff_precision(uint64_t scale);

#ifdef __cplusplus
}
#endif
#endif
