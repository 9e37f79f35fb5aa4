// column.cu -- host side of the engine: the EBI1 reader, the resident column
// and the Decoder-shaped query entry points of include/ebi_gpu.h.
//
// Decoder::new (api/decoder.rs:136-156) becomes ebi_column_open: the header
// and footer are parsed on the host exactly as FileReader::fetch_header /
// fetch_footer do (decoder.rs:131-220, format/deserialize.rs:117-300), the
// chunk table (GeneralChunkHandle geometry, decoder.rs:283-352) is built once,
// and the unmodified file bytes are copied to HBM where they stay.  Every
// query then runs the codec's kernel over the chunk table and a fold of the
// per-chunk results (query.cu; the fused BUFF scans fold in their last CTA).
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "column.h"

namespace ebi {

static std::atomic<uint64_t> g_launches{0};
static thread_local std::string g_last_error;

void count_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
void set_last_error(const std::string& msg) { g_last_error = msg; }

cudaError_t allow_dynamic_smem(const void* fn, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    struct Grant {
        const void* fn;
        int dev;
        size_t bytes;
    };
    static std::mutex mu;
    static std::vector<Grant> grants;
    std::lock_guard<std::mutex> lk(mu);
    Grant* g = nullptr;
    for (Grant& x : grants)
        if (x.fn == fn && x.dev == dev) g = &x;
    if (g && g->bytes >= bytes) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
    if (e != cudaSuccess) return e;
    if (g) g->bytes = bytes;
    else grants.push_back(Grant{fn, dev, bytes});
    return cudaSuccess;
}

static int fail(int code, const std::string& msg) {
    set_last_error(msg);
    return code;
}
static int cuda_fail(cudaError_t e, const char* what) {
    return fail(EBI_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(expr)                                              \
    do {                                                      \
        cudaError_t _e = (expr);                              \
        if (_e != cudaSuccess) return cuda_fail(_e, #expr);   \
    } while (0)

static uint32_t rd32(const uint8_t* p) {
    return uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24);
}
static uint64_t rd64(const uint8_t* p) { return uint64_t(rd32(p)) | (uint64_t(rd32(p + 4)) << 32); }

// The device's default stream-ordered pool keeps freed memory for reuse, so
// reopening columns of similar size does not go back to the CUDA driver for memory.
static void tune_pool_once() {
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0;
        cudaMemPool_t pool;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t keep = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        cudaGetLastError();
    });
}

// Pinned result slots: every column needs one small pinned QueryResult for
// its scalar outputs.  cudaMallocHost / cudaFreeHost are slow, synchronizing
// calls, so the slots come from pinned slabs allocated once and recycled.
template <typename T>
class PinnedSlots {
  public:
    T* take() {
        std::lock_guard<std::mutex> lk(mu_);
        if (free_.empty()) {
            constexpr size_t kSlab = 1024;
            void* p = nullptr;
            if (cudaMallocHost(&p, kSlab * sizeof(T)) != cudaSuccess) return nullptr;
            T* q = static_cast<T*>(p);
            for (size_t i = 0; i < kSlab; ++i) free_.push_back(q + i);
        }
        T* r = free_.back();
        free_.pop_back();
        return r;
    }
    void give(T* r) {
        std::lock_guard<std::mutex> lk(mu_);
        free_.push_back(r);
    }

  private:
    std::mutex mu_;
    std::vector<T*> free_;  // slabs are kept for the life of the process
};
static PinnedSlots<QueryResult> g_pinned;
static PinnedSlots<ScanTotals> g_pinned_tot;

// Pinned staging for the small tables a column open uploads (chunk table,
// tiles, units, repack segments, chunk headers), one per host thread, grown on
// demand and kept: copies from it are asynchronous, so none of them holds the
// host, and they queue behind the column's own bytes without delaying them.
class TableStage {
  public:
    ~TableStage() {
        if (p_) cudaFreeHost(p_);
    }
    // Room for `bytes` (16-byte aligned pieces); false when pinned memory runs out.
    bool reserve(size_t bytes) {
        used_ = 0;
        if (bytes <= cap_) return true;
        if (p_) cudaFreeHost(p_);
        p_ = nullptr;
        cap_ = 0;
        void* q = nullptr;
        if (cudaMallocHost(&q, bytes * 2) != cudaSuccess) return false;
        p_ = static_cast<uint8_t*>(q);
        cap_ = bytes * 2;
        return true;
    }
    // Copies n bytes into the stage and returns their pinned address (null
    // when they do not fit the room reserved).
    const void* put(const void* src, size_t n) {
        const size_t step = (n + 15) & ~size_t(15);
        if (step > cap_ - used_) return nullptr;
        uint8_t* d = p_ + used_;
        std::memcpy(d, src, n);
        used_ += step;
        return d;
    }

  private:
    uint8_t* p_ = nullptr;
    size_t cap_ = 0, used_ = 0;
};
static thread_local TableStage t_stage;

// (double)x / 2^frac as the device's fold_scale rounds it (one conversion, one
// exact power-of-two scaling).
static double host_fold_scale(long long x, uint32_t frac) {
    auto pow2 = [](int e) {  // 2^e for -1022 <= e <= 1023
        const uint64_t b = uint64_t(1023 + e) << 52;
        double d;
        std::memcpy(&d, &b, sizeof d);
        return d;
    };
    const double v = static_cast<double>(x);
    if (frac <= 1022) return v * pow2(-static_cast<int>(frac));
    return v / (frac <= 1023 ? pow2(1023) : HUGE_VAL);
}

}  // namespace ebi

using namespace ebi;


namespace {

// FileReader::fetch_header + fetch_footer (decoder.rs:131-220).
int parse_file(const uint8_t* d, uint64_t len, ebi_column* c) {
    if (len < 30) return fail(EBI_E_IO, "file shorter than the 30-byte FileHeader");
    if (d[4] != 0) return fail(EBI_E_CONVERSION, "Failed to convert FieldType");
    if (d[5] > 12) return fail(EBI_E_CONVERSION, "Failed to convert CompressionScheme");
    if (d[6] > 2) return fail(EBI_E_CONVERSION, "Failed to convert ChunkOptionKind");
    const int scheme = d[5];
    const uint64_t fo = rd64(d + 16);  // FileHeader::footer_offset (format.rs:143-151)
    if (fo > len || len - fo < 16) return fail(EBI_E_IO, "footer offset past the end of the file");
    const uint64_t nrec = rd64(d + fo), nch = rd64(d + fo + 8);
    const uint64_t p = fo + 16;
    if (nch > (len - p) / 16) return fail(EBI_E_IO, "chunk footers past the end of the file");
    const uint64_t cf = p + nch * 16;
    if (cf + 1 > len) return fail(EBI_E_IO, "compressor config past the end of the file");
    const uint64_t csz = d[cf];
    if (cf + 1 + csz > len) return fail(EBI_E_IO, "compressor config past the end of the file");
    if (csz < 8) return fail(EBI_E_CORRUPT, "compressor config shorter than 8 bytes");
    if (cf + 1 + csz + 164 > len) return fail(EBI_E_IO, "FileFooter3 past the end of the file");
    if (scheme > EBI_ELF) return fail(EBI_E_UNSUPPORTED, "compression scheme outside this engine");
    if (nrec > 0xffffffffull) return fail(EBI_E_UNSUPPORTED, "more than 2^32 - 1 records (row ids are u32)");
    c->scheme = scheme;
    c->n_records = nrec;
    c->n_chunks = nch;
    c->footer_off = fo;
    c->file_len = len;
    c->chunks.resize(nch);
    for (uint64_t i = 0; i < nch; ++i) {
        const uint64_t phys = rd64(d + p + 16 * i), logi = rd64(d + p + 16 * i + 8);
        const uint64_t nphys = i + 1 < nch ? rd64(d + p + 16 * (i + 1)) : fo;
        const uint64_t nlogi = i + 1 < nch ? rd64(d + p + 16 * (i + 1) + 8) : nrec;
        ChunkDesc cd{};
        cd.byte_off = phys;
        cd.byte_len = nphys - phys;
        cd.row_off = logi;
        cd.n_rows = static_cast<uint32_t>(nlogi - logi);
        if (nphys < phys || phys > len || nphys > len) { cd.flags |= kChunkBadGeometry; cd.byte_len = 0; }
        if (nlogi < logi || nlogi - logi > 0xffffffffull || nlogi > nrec) { cd.flags |= kChunkBadGeometry; cd.n_rows = 0; }
        if (logi % 32) c->rows_aligned32 = false;
        if (i > 0 && logi < c->chunks[i - 1].row_off) c->rows_in_order = false;
        c->chunks[i] = cd;
    }
    // Uncompressed chunks decode exactly their rows; an RLE chunk decodes the
    // sum of its run lengths (decoder/chunk_reader/run_length.rs:68-91), read
    // here for every chunk whose field table fits (the others fail when read).
    c->rows_bounded = scheme == EBI_UNCOMPRESSED;
    if (scheme == EBI_RLE) {
        c->rows_bounded = true;
        for (uint64_t i = 0; i < nch && c->rows_bounded; ++i) {
            const ChunkDesc& cd = c->chunks[i];
            if ((cd.flags & kChunkBadGeometry) || cd.byte_len < 8) continue;
            const uint8_t* p = d + cd.byte_off;
            const uint64_t nf = rd64(p);
            if (nf > (cd.byte_len - 8) / 9) continue;
            uint64_t rows = 0;
            for (uint64_t k = 0; k < nf; ++k) rows += p[8 + 9 * k];
            if (rows > cd.n_rows) c->rows_bounded = false;
        }
    }
    return EBI_OK;
}

// BUFF chunk headers (decoder/chunk_reader/buff/decode.rs:5-17) and the
// checks every reader of the chunk applies; a failing chunk keeps its status
// and raises it only when a query reads the chunk.
std::vector<BuffChunkInfo> parse_buff_headers(const uint8_t* file, const std::vector<ChunkDesc>& chunks) {
    std::vector<BuffChunkInfo> out(chunks.size());
    for (size_t i = 0; i < chunks.size(); ++i) {
        const ChunkDesc& cd = chunks[i];
        BuffChunkInfo b{};
        if (cd.flags & kChunkBadGeometry) { b.status = EBI_E_IO; out[i] = b; continue; }
        if (cd.byte_len < 20) { b.status = EBI_E_UNEXPECTED_END; out[i] = b; continue; }
        const uint8_t* p = file + cd.byte_off;
        b.base = static_cast<int64_t>(rd64(p));
        b.n = rd32(p + 8);
        b.bits = rd32(p + 12);
        b.frac = rd32(p + 16);
        if (b.bits > 64 || b.n != cd.n_rows) { b.status = EBI_E_CORRUPT; out[i] = b; continue; }
        const uint64_t np = b.bits / 8, tb = b.bits % 8;
        const uint64_t need = 20 + np * b.n + (uint64_t(b.n) * tb + 7) / 8;
        if (b.bits > 0 && need > cd.byte_len) { b.status = EBI_E_UNEXPECTED_END; out[i] = b; continue; }
        b.planes = cd.byte_off + 20;
        b.tail = b.planes + np * b.n;
        out[i] = b;
    }
    return out;
}

template <typename T>
int dev_alloc(T** p, size_t count, cudaStream_t s) {
    void* v = nullptr;
    const cudaError_t e = cudaMallocAsync(&v, count ? count * sizeof(T) : 16, s);
    if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? fail(EBI_E_OOM, "device allocation failed")
                                                               : cuda_fail(e, "cudaMallocAsync");
    *p = static_cast<T*>(v);
    return EBI_OK;
}
// A buffer the column keeps until close (counted in c->device_bytes).
template <typename T>
int col_alloc(ebi_column* c, T** p, size_t count, cudaStream_t s) {
    const int st = dev_alloc(p, count, s);
    if (!st) c->device_bytes += count ? count * sizeof(T) : 16;
    return st;
}

QueryParams base_params(const ebi_column* c) {
    QueryParams q{};
    q.file = c->d_file;
    q.copy_wait = c->copy_wait;
    q.chunks = c->d_chunks;
    q.acc = c->d_acc;
    q.tiles = c->d_tiles;
    q.n_tiles = static_cast<uint32_t>(c->tiles.tiles.size());
    q.n_chunks = static_cast<uint32_t>(c->n_chunks);
    q.n_records = c->n_records;
    q.chunk_id = -1;
    q.precision = c->precision;
    q.scheme = c->scheme;
    q.agg = AGG_ALL;
    q.binfo = c->d_buff;
    q.stage_bytes = c->stage_bytes;
    q.dec_tab = c->dec_tab;
    return q;
}

int check_supported(const ebi_column* c) {
    if (c->scheme < EBI_UNCOMPRESSED || c->scheme > EBI_ELF) return fail(EBI_E_UNSUPPORTED, "compression scheme outside this engine");
    return EBI_OK;
}

// The value codecs (everything but BUFF) run one CTA per chunk; their tiles are the chunks.
cudaError_t launch_values(const ebi_column* c, const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                          const unsigned long long* chunk_offsets, cudaStream_t s) {
    switch (c->scheme) {
    case EBI_UNCOMPRESSED: return launch_raw(q, chunk_begin, n_chunks, mode, chunk_offsets, s);
    case EBI_RLE: return launch_rle(q, chunk_begin, n_chunks, mode, chunk_offsets, s);
    default: return launch_xor(q, chunk_begin, n_chunks, mode, chunk_offsets, s);
    }
}

// The totals block of the next scan.
ScanTotals* scan_totals(ebi_column* c) {
    return reinterpret_cast<ScanTotals*>(reinterpret_cast<uint8_t*>(c->d_tot) + (c->tot_flip ? kScanTotalsBytes : 0));
}

// Tile range of the query: all tiles, or those of chunk_id (none when out of range).
void tile_range(const ebi_column* c, int64_t chunk_id, uint32_t* begin, uint32_t* count) {
    if (chunk_id < 0) { *begin = 0; *count = static_cast<uint32_t>(c->tiles.tiles.size()); return; }
    if (static_cast<uint64_t>(chunk_id) >= c->n_chunks) { *begin = 0; *count = 0; return; }
    *begin = c->tiles.first_tile[chunk_id];
    *count = c->tiles.first_tile[chunk_id + 1] - *begin;
}

int ensure_scratch(ebi_column* c, cudaStream_t s) {
    if (c->d_tile_counts) return EBI_OK;
    const size_t nt = c->tiles.tiles.size();
    int st = col_alloc(c, &c->d_tile_counts, nt, s);
    if (!st) st = col_alloc(c, &c->d_tile_offsets, nt + 1, s);
    if (!st) st = col_alloc(c, &c->d_scratch_mask, c->mask_words, s);
    return st;
}

// Query timing: events at the query's start (ev[0]), right before the first
// codec kernel (ev[3], after the query's memsets and chunk selection; the
// scan is timed from ev[0] when a query marks none), after the codec kernels
// (ev[1]) and after the finalize fold (ev[2]; a query whose totals the host
// scales has no fold and ends at ev[1]).  Only events that delimit work are
// recorded: each one is a timestamp write on the device's timeline.
int begin_query(ebi_column* c, cudaStream_t s) {
    c->launches_at_start = ebi_kernel_launches();
    c->scan_marked = false;
    if (c->timing) CK(cudaEventRecord(c->ev[0], s));
    return EBI_OK;
}

int mark_scan(ebi_column* c, cudaStream_t s) {
    if (c->timing) CK(cudaEventRecord(c->ev[3], s));
    c->scan_marked = true;
    return EBI_OK;
}

// Ends a pass that cannot raise and folds nothing (a quiet BUFF materialize):
// one synchronisation, no finalize launch.
int finish_quiet(ebi_column* c, cudaStream_t s) {
    if (c->timing) CK(cudaEventRecord(c->ev[1], s));
    CK(cudaStreamSynchronize(s));
    c->last.kernels = ebi_kernel_launches() - c->launches_at_start;
    if (c->timing) {
        float a = 0.f, t = 0.f;
        CK(cudaEventElapsedTime(&a, c->scan_marked ? c->ev[3] : c->ev[0], c->ev[1]));
        CK(cudaEventElapsedTime(&t, c->ev[0], c->ev[1]));
        c->last.scan_ms = a;
        c->last.finalize_ms = 0.f;
        c->last.total_ms = t;
    }
    return EBI_OK;
}

// Enqueues finalize (unless the scan kernel already folded, or left exact
// totals for the host to scale), copies the result back and waits.
int finish(ebi_column* c, const QueryParams& q, cudaStream_t s) {
    if (c->timing) CK(cudaEventRecord(c->ev[1], s));
    bool done = false, folded = false;
    if (c->totals_pending) {
        c->totals_pending = false;
        CK(cudaMemcpyAsync(c->h_tot, c->pending_tot, sizeof(ScanTotals), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        const ScanTotals t = *c->h_tot;
        if (t.bad_chunk == 0xffffffffu && !t.nonexact && t.abs_bound < (1ull << 52)) {
            // every chunk total and prefix of the chunk-ordered fold is an exact
            // multiple of 2^-frac below 2^53 of them: the fold equals the exact total
            QueryResult& r = *c->h_res;
            r.status = 0;
            r.bad_chunk = 0xffffffffu;
            r.count = t.count;
            r.sum = 0.0;
            r.min = HUGE_VAL;
            r.max = -HUGE_VAL;
            if (t.count) {
                r.sum = host_fold_scale(static_cast<long long>(t.sum_fixed), c->buff_frac);
                r.max = host_fold_scale(t.max_fixed, c->buff_frac);
                r.min = host_fold_scale(t.min_fixed, c->buff_frac);
            }
            done = true;
        } else {
            c->fused_pending = false;  // a failing chunk: the chunk-ordered fold reports it and re-arms
        }
    }
    if (!done) {
        if (!c->fused_pending) CK(launch_finalize(q, c->d_res, c->d_parts, s));
        c->fused_pending = false;
        if (c->timing) CK(cudaEventRecord(c->ev[2], s));
        folded = true;
        CK(cudaMemcpyAsync(c->h_res, c->d_res, sizeof(QueryResult), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    c->last.kernels = ebi_kernel_launches() - c->launches_at_start;
    if (c->timing) {
        float a = 0.f, b = 0.f, t = 0.f;
        cudaEvent_t end = folded ? c->ev[2] : c->ev[1];
        CK(cudaEventElapsedTime(&a, c->scan_marked ? c->ev[3] : c->ev[0], c->ev[1]));
        if (folded) CK(cudaEventElapsedTime(&b, c->ev[1], c->ev[2]));
        CK(cudaEventElapsedTime(&t, c->ev[0], end));
        c->last.scan_ms = a;
        c->last.finalize_ms = b;
        c->last.total_ms = t;
    }
    if (c->h_res->status) {
        char buf[96];
        std::snprintf(buf, sizeof buf, "chunk %u: status %u", c->h_res->bad_chunk, c->h_res->status);
        return fail(static_cast<int>(c->h_res->status), buf);
    }
    return EBI_OK;
}

// Runs filter / filter+agg / agg over the column.
int run_scan(ebi_column* c, int op, const ebi_predicate* pred, const uint64_t* d_mask, int64_t chunk_id,
             uint64_t* d_out_mask, unsigned long long* tile_counts, cudaStream_t s, uint32_t agg = AGG_ALL) {
    if (int st = begin_query(c, s)) return st;
    QueryParams q = base_params(c);
    q.agg = agg;
    q.op = op;
    q.chunk_id = chunk_id;
    q.in_mask = reinterpret_cast<const uint32_t*>(d_mask);
    q.out_mask = reinterpret_cast<uint32_t*>(d_out_mask);
    q.tile_counts = tile_counts;
    if (pred) q.pred = *pred;
    q.pred_on = pred != nullptr;
    uint32_t tb, tn;
    tile_range(c, chunk_id, &tb, &tn);
    if (c->scheme != EBI_BUFF) {
        // Value codecs OR their rows into a zeroed output (decoded runs may
        // start on any row).  When every chunk is scanned, chunks start on
        // 32-row boundaries in row order and none decodes rows past its range
        // (whose bits would land in the next chunk's words), each chunk's CTA
        // zeroes its own words.
        q.own_words = c->rows_aligned32 && c->rows_in_order && c->rows_bounded;
        q.segs = c->d_segs;
        q.zero_out = d_out_mask && tn > 0 && tn == c->n_chunks && q.own_words;
        if (d_out_mask && !q.zero_out) CK(cudaMemsetAsync(d_out_mask, 0, c->mask_words * 8, s));
        if (d_mask) CK(launch_select_chunks(q, s));
        if (int st = mark_scan(c, s)) return st;
        CK(launch_values(c, q, tb, tn, VAL_SCAN, nullptr, s));
        return EBI_OK;
    }
    if (d_out_mask) {
        // Words shared by two chunks, or words of chunks that are not read, need
        // a zeroed output; otherwise every word is written by exactly one thread.
        q.out_atomic = !c->rows_aligned32 || chunk_id >= 0;
        if (q.out_atomic || tn == 0) CK(cudaMemsetAsync(d_out_mask, 0, c->mask_words * 8, s));
        else if ((c->n_records + 31) / 32 % 2 == 1)  // last u32 of the last u64 word
            CK(cudaMemsetAsync(reinterpret_cast<uint32_t*>(d_out_mask) + 2 * c->mask_words - 1, 0, 4, s));
    }
    if (d_mask) CK(launch_select_chunks(q, s));
    if (int st = mark_scan(c, s)) return st;
    if (c->scheme == EBI_BUFF) {
        if (tile_counts || tn == 0) {
            CK(launch_buff_query(q, tb, tn, s));
        } else if (c->stream_ok) {
            const uint32_t ub = chunk_id < 0 ? 0u : c->first_unit[chunk_id];
            const uint32_t un = chunk_id < 0 ? c->first_unit.back() : c->first_unit[chunk_id + 1] - ub;
            // exact columns without an input bitmask: totals only, scaled on the host
            const bool totals_only = c->buff_exact && !d_mask;
            const uint32_t fold = (c->buff_fast_ok ? 1u : 0u) | (c->buff_exact ? 2u : 0u) |
                                  (totals_only ? 4u | (c->tot_flip ? 8u : 0u) : 0u);
            ScanTotals* T = scan_totals(c);
            CK(launch_buff_stream(q, c->d_buff, c->d_units, ub, un, c->units_per_chunk, c->stream_bits, c->sms, T, c->d_res,
                                  c->buff_frac, fold, s));
            if (totals_only) {
                c->totals_pending = true;
                c->pending_tot = T;
                c->tot_flip ^= 1u;  // the launch set the other block at rest
            } else {
                c->fused_pending = true;
            }
        } else {
            CK(launch_buff_scan(q, c->d_buff, tb, tn, c->layout, c->scan_grid, scan_totals(c), c->d_res, c->buff_frac,
                                c->buff_fast_ok, s));
            c->fused_pending = true;
        }
    }
    return EBI_OK;
}

int check_pred(const ebi_predicate* p) {
    if (!p) return fail(EBI_E_INVALID, "predicate is null");
    if (p->kind < EBI_PRED_EQ || p->kind > EBI_PRED_RANGE) return fail(EBI_E_INVALID, "bad predicate kind");
    if (p->kind == EBI_PRED_RANGE && (p->start_kind < 0 || p->start_kind > 2 || p->end_kind < 0 || p->end_kind > 2))
        return fail(EBI_E_INVALID, "bad range bound kind");
    return EBI_OK;
}

// Materialize / filter_materialize of a value codec: a count pass, a scan of
// the per-chunk counts and a pass that writes every chunk's rows at its offset.
int run_materialize_values(ebi_column* c, const ebi_predicate* pred, const uint64_t* d_mask, int64_t chunk_id,
                           double* d_out, uint64_t out_cap, uint64_t* n_out, cudaStream_t s) {
    if (int st = begin_query(c, s)) return st;
    QueryParams q = base_params(c);
    q.op = OP_FILTER;  // only the status is folded
    q.chunk_id = chunk_id;
    q.in_mask = reinterpret_cast<const uint32_t*>(d_mask);
    q.out_vals = d_out;
    q.out_cap = out_cap;
    q.tile_counts = c->d_tile_counts;
    q.pred_on = pred != nullptr;
    if (pred) q.pred = *pred;
    uint32_t tb, tn;
    tile_range(c, chunk_id, &tb, &tn);
    CK(launch_values(c, q, tb, tn, VAL_COUNT, nullptr, s));
    CK(launch_tile_scan(c->d_tile_counts, c->d_tile_offsets, tn, s));
    CK(launch_values(c, q, tb, tn, VAL_MATERIALIZE, c->d_tile_offsets, s));
    CK(cudaMemcpyAsync(&c->h_res->count, c->d_tile_offsets + tn, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const uint64_t total = c->h_res->count;
    int st = finish(c, q, s);
    if (st) return st;
    if (n_out) *n_out = total;
    if (total > out_cap) return fail(EBI_E_INVALID, "output buffer smaller than the values to write");
    return EBI_OK;
}

// Materializes the rows of d_mask (all rows when null) into d_out.
int run_materialize(ebi_column* c, const uint64_t* d_mask, int64_t chunk_id, double* d_out, uint64_t out_cap,
                    uint64_t* n_out, cudaStream_t s, bool mask_is_scratch, const QueryParams* prior) {
    QueryParams q = prior ? *prior : base_params(c);
    q.op = OP_FILTER;  // only status is folded
    q.chunk_id = chunk_id;
    q.in_mask = reinterpret_cast<const uint32_t*>(d_mask);
    q.out_mask = nullptr;
    q.out_vals = d_out;
    q.out_cap = out_cap;
    uint32_t tb, tn;
    tile_range(c, chunk_id, &tb, &tn);
    if (!mask_is_scratch) {
        if (int st = begin_query(c, s)) return st;
    }
    uint64_t total = 0;
    if (!d_mask) {
        for (uint32_t t = tb; t < tb + tn; ++t) {
            const Tile& tl = c->tiles.tiles[t];
            const uint32_t n = c->chunks[tl.chunk].n_rows;
            total += tl.begin < n ? std::min<uint64_t>(kBuffTileRows, n - tl.begin) : 0;
        }
        if (total > out_cap) {
            if (n_out) *n_out = total;
            return fail(EBI_E_INVALID, "output buffer smaller than the values to write");
        }
        q.tile_counts = nullptr;
    } else {
        q.tile_counts = c->d_tile_counts;
        if (!mask_is_scratch) CK(launch_buff_count(q, tb, tn, s));
        CK(launch_tile_scan(c->d_tile_counts, c->d_tile_offsets, tn, s));
    }
    const uint64_t base_row = chunk_id >= 0 && static_cast<uint64_t>(chunk_id) < c->n_chunks ? c->chunks[chunk_id].row_off : 0;
    // without a bitmask over readable chunks nothing can raise: no fold
    const bool quiet = !d_mask && c->buff_all_readable;
    CK(launch_buff_materialize(q, tb, tn, c->d_tile_offsets, base_row, c->buff_max_bits > 32, quiet, s));
    if (quiet) {
        if (int st = finish_quiet(c, s)) return st;
        if (n_out) *n_out = total;
        return EBI_OK;
    }
    if (d_mask) CK(cudaMemcpyAsync(&c->h_res->count, c->d_tile_offsets + tn, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (d_mask) total = c->h_res->count;
    int st = finish(c, q, s);
    if (st) return st;
    if (n_out) *n_out = total;
    if (total > out_cap) return fail(EBI_E_INVALID, "output buffer smaller than the values to write");
    return EBI_OK;
}

}  // namespace

QueryParams ebi::column_params(const ebi_column* c) { return base_params(c); }

extern "C" {

int ebi_column_open(const uint8_t* file, uint64_t len, void* stream, ebi_column** out) {
    if (!out) return fail(EBI_E_INVALID, "out is null");
    *out = nullptr;
    if (!file && len) return fail(EBI_E_INVALID, "file is null");
    tune_pool_once();
    ebi_column* c = new (std::nothrow) ebi_column();
    if (!c) return fail(EBI_E_OOM, "host allocation failed");
    c->stream = static_cast<cudaStream_t>(stream);
    cudaGetDevice(&c->device);
    int st = parse_file(file, len, c);
    if (st) { delete c; return st; }
    cudaStream_t s = c->stream;
    std::vector<BuffChunkInfo> binfo;
    std::vector<RepackSeg> segs;
    uint64_t dev_len = len;  // bytes of the column in HBM
    if (c->scheme == EBI_BUFF) {
        c->tiles = buff_tiles(c->chunks);
        binfo = parse_buff_headers(file, c->chunks);
        dev_len = buff_plan_layout(binfo, segs);
        uint32_t np_max = 0, tb_max = 0;
        bool first = true;
        c->buff_fast_ok = true;
        c->stream_ok = true;
        for (const BuffChunkInfo& b : binfo) {
            if (b.status) continue;
            if (b.bits < 1 || b.bits > 32) c->stream_ok = false;  // constant and > 32-bit chunks: the pipelined scan
            np_max = std::max(np_max, b.bits / 8);
            tb_max = std::max(tb_max, b.bits % 8);
            if (first) { c->buff_frac = b.frac; first = false; }
            if (b.frac != c->buff_frac || b.frac > 1022 || b.bits == 0) c->buff_fast_ok = false;
        }
        // bound of sum |base + delta| over every readable row, and of each |base + delta|
        long double bound = 0.0L, widest = 0.0L;
        c->buff_same_frac = true;
        bool seen = false;
        uint32_t frac0 = 0;
        for (const BuffChunkInfo& b : binfo) {
            if (b.status) continue;
            const long double lo = static_cast<long double>(b.base);
            const long double hi = lo + (b.bits >= 64 ? 18446744073709551615.0L : static_cast<long double>((1ull << b.bits) - 1));
            const long double m = std::max(lo < 0 ? -lo : lo, hi < 0 ? -hi : hi);
            bound += static_cast<long double>(b.n) * m;
            widest = std::max(widest, m);
            if (!seen) { frac0 = b.frac; seen = true; }
            if (b.frac != frac0 || b.frac > 1022) c->buff_same_frac = false;
        }
        c->buff_fixed_bits = 0;
        while (c->buff_fixed_bits < 64 && std::ldexp(1.0L, static_cast<int>(c->buff_fixed_bits)) <= widest) ++c->buff_fixed_bits;
        c->buff_exact = c->buff_fast_ok && bound < 4503599627370496.0L;  // 2^52
        uint32_t per_sm = 1;
        c->layout = buff_stage_layout(np_max, tb_max, &per_sm);
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        c->scan_grid = static_cast<uint32_t>(std::max(sms, 1)) * per_sm;
        c->sms = static_cast<uint32_t>(std::max(sms, 1));
        uint64_t rows_of[65] = {};
        c->buff_all_readable = true;
        for (const BuffChunkInfo& b : binfo)
            if (!b.status) {
                rows_of[b.bits] += b.n;
                c->buff_max_bits = std::max(c->buff_max_bits, b.bits);
            } else {
                c->buff_all_readable = false;
            }
        c->stream_bits = static_cast<uint32_t>(std::max_element(rows_of + 1, rows_of + 33) - rows_of);
    } else {
        if (c->scheme == EBI_GORILLA) c->stage_bytes = gorilla_stage_bytes(c->chunks.data(), c->n_chunks);
        if (c->scheme == EBI_ELF || c->scheme == EBI_ELF_ON_CHIMP) {
            const cudaError_t e = elf_tables(&c->dec_tab);
            if (e != cudaSuccess) {
                delete c;
                return fail(EBI_E_CUDA, std::string("Elf decimal tables: ") + cudaGetErrorString(e));
            }
        }
        c->tiles.tiles.resize(c->n_chunks);
        c->tiles.first_tile.resize(c->n_chunks + 1);
        for (uint64_t i = 0; i < c->n_chunks; ++i) {
            c->tiles.tiles[i] = Tile{static_cast<uint32_t>(i), 0};
            c->tiles.first_tile[i] = static_cast<uint32_t>(i);
        }
        c->tiles.first_tile[c->n_chunks] = static_cast<uint32_t>(c->n_chunks);
    }
    c->mask_words = (c->n_records + 63) / 64;
    if (c->mask_words == 0) c->mask_words = 1;
    st = col_alloc(c, &c->d_file, dev_len + kFilePad, s);
    // BUFF: the planes are repacked into d_file straight from the caller's
    // buffer when the device can read it (pinned host memory: one pass over
    // the host link), else from a device copy of the file
    const uint8_t* src = nullptr;
    if (c->scheme == EBI_BUFF) {
        cudaPointerAttributes pa{};
        if (cudaPointerGetAttributes(&pa, file) == cudaSuccess &&
            (pa.type == cudaMemoryTypeHost || pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged) &&
            pa.devicePointer)
            src = static_cast<const uint8_t*>(pa.devicePointer);
        cudaGetLastError();  // a pageable pointer is not an error here
    }
    uint8_t* raw = nullptr;       // BUFF: the file as read, repacked into d_file
    RepackSeg* d_segs = nullptr;
    if (!st && c->scheme == EBI_BUFF && !src) st = dev_alloc(&raw, len + kFilePad, s);
    if (!st && c->scheme == EBI_BUFF) st = dev_alloc(&d_segs, segs.size(), s);
    static const ScanTotals kRest = {0, 0, 0, LLONG_MIN, LLONG_MAX, 0, 0xffffffffu, 0, 0, 0};
    // every table the open uploads (units: at most one per 2,048 rows of a chunk), 16-byte pieces
    const size_t table_bytes = segs.size() * sizeof(RepackSeg) + c->n_chunks * sizeof(ChunkDesc) +
                               c->tiles.tiles.size() * sizeof(Tile) + binfo.size() * sizeof(BuffChunkInfo) +
                               size_t(c->n_records / kBuffUnitRows + c->n_chunks + 1) * sizeof(uint2) +
                               2 * sizeof(ScanTotals) + 8 * 16;
    if (!st && !t_stage.reserve(table_bytes)) st = fail(EBI_E_OOM, "pinned allocation failed");
    cudaError_t e = cudaSuccess;
    // the column's bytes first: the link is the long pole of an open
    if (!st) {
        if (!src) {
            uint8_t* dst = raw ? raw : c->d_file;
            e = cudaMemcpyAsync(dst, file, len, cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaMemsetAsync(dst + len, 0, kFilePad, s);
            if (raw) src = raw;
        }
        if (e == cudaSuccess && c->scheme == EBI_BUFF) {
            e = cudaMemsetAsync(c->d_file + dev_len, 0, kFilePad, s);
            if (e == cudaSuccess && !segs.empty()) {
                const void* h = t_stage.put(segs.data(), segs.size() * sizeof(RepackSeg));
                e = h ? cudaMemcpyAsync(d_segs, h, segs.size() * sizeof(RepackSeg), cudaMemcpyHostToDevice, s)
                      : cudaErrorMemoryAllocation;
            }
            if (e == cudaSuccess) e = launch_buff_repack(src, c->d_file, d_segs, static_cast<uint32_t>(segs.size()), s);
        }
    }
    // the rest of the column's tables, built while the bytes cross the link
    std::vector<uint2> units;
    if (c->scheme == EBI_BUFF) {
        units = buff_units(c->chunks, c->first_unit);
        c->units_per_chunk = buff_uniform_units(c->first_unit);
    }
    if (!st && c->scheme == EBI_BUFF) st = col_alloc(c, &c->d_units, units.size(), s);
    if (!st) st = col_alloc(c, &c->d_chunks, c->n_chunks, s);
    if (!st) st = col_alloc(c, &c->d_tiles, c->tiles.tiles.size(), s);
    if (!st) st = col_alloc(c, &c->d_acc, c->n_chunks, s);
    if (!st) st = col_alloc(c, &c->d_res, 1, s);
    if (!st && c->scheme != EBI_BUFF)
        st = col_alloc(c, &c->d_parts, value_slices(static_cast<uint32_t>(c->n_chunks)) + 1, s);
    // the XOR chunk pass's segment starts, converged ahead of it by a separate
    // kernel; not for columns of chunks so small that the scratch would exceed
    // a quarter of the file (their chunks converge in a round or two anyway)
    const bool xor_segs = c->scheme == EBI_CHIMP || c->scheme == EBI_CHIMP128 || c->scheme == EBI_ELF ||
                          c->scheme == EBI_ELF_ON_CHIMP;
    if (!st && xor_segs && c->n_chunks * kSegsPerChunk * sizeof(SegState) <= c->file_len / 4)
        st = col_alloc(c, &c->d_segs, c->n_chunks * kSegsPerChunk, s);
    if (!st && !binfo.empty()) st = col_alloc(c, &c->d_buff, binfo.size(), s);
    // the scan totals and, behind them, one slot per CTA of a scan launch
    // two totals blocks (totals-only queries alternate between them)
    if (!st) st = col_alloc(c, &c->d_tot, (2 * kScanTotalsBytes + sizeof(ScanTotals) - 1) / sizeof(ScanTotals), s);
    if (!st && !(c->h_res = g_pinned.take())) st = fail(EBI_E_OOM, "pinned allocation failed");
    if (!st && !(c->h_tot = g_pinned_tot.take())) st = fail(EBI_E_OOM, "pinned allocation failed");
    if (!st) {
        auto up = [&](void* dst, const void* host, size_t n) {
            if (e != cudaSuccess || !n) return;
            const void* h = t_stage.put(host, n);
            e = h ? cudaMemcpyAsync(dst, h, n, cudaMemcpyHostToDevice, s) : cudaErrorMemoryAllocation;
        };
        if (c->scheme == EBI_BUFF) up(c->d_units, units.data(), units.size() * sizeof(uint2));
        up(c->d_chunks, c->chunks.data(), c->n_chunks * sizeof(ChunkDesc));
        up(c->d_tiles, c->tiles.tiles.data(), c->tiles.tiles.size() * sizeof(Tile));
        up(c->d_buff, binfo.data(), binfo.size() * sizeof(BuffChunkInfo));
        up(c->d_tot, &kRest, sizeof kRest);
        up(reinterpret_cast<uint8_t*>(c->d_tot) + kScanTotalsBytes, &kRest, sizeof kRest);
        if (e == cudaSuccess && c->d_parts)
            e = cudaMemsetAsync(c->d_parts, 0, (value_slices(static_cast<uint32_t>(c->n_chunks)) + 1) * sizeof(ValPart), s);
        if (e == cudaSuccess) e = launch_acc_init(c->d_acc, static_cast<uint32_t>(c->n_chunks), s);
    }
    // the staged tables must stay until the copies ran
    if (cudaError_t e2 = cudaStreamSynchronize(s); e == cudaSuccess) e = e2;
    if (!st && e != cudaSuccess) st = cuda_fail(e, "ebi_column_open upload");
    if (raw) cudaFreeAsync(raw, s);
    if (d_segs) cudaFreeAsync(d_segs, s);
    if (st) { ebi_column_close(c); return st; }
    *out = c;
    return EBI_OK;
}

// The staging buffer of ebi_column_open_file: pinned, grown on demand, kept.
namespace {
std::mutex g_file_mu;
uint8_t* g_file_buf = nullptr;
uint64_t g_file_cap = 0;
}  // namespace

int ebi_column_open_file(const char* path, void* stream, ebi_column** out) {
    if (!path || !out) return fail(EBI_E_INVALID, "path or out is null");
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(EBI_E_IO, std::string("cannot open ") + path);
    uint64_t len = 0;
    if (std::fseek(f, 0, SEEK_END) == 0) {
        const long n = std::ftell(f);
        len = n > 0 ? static_cast<uint64_t>(n) : 0;
    }
    std::rewind(f);
    std::lock_guard<std::mutex> lock(g_file_mu);
    if (len > g_file_cap) {
        if (g_file_buf) cudaFreeHost(g_file_buf);
        g_file_buf = nullptr;
        g_file_cap = 0;
        void* p = nullptr;
        if (cudaHostAlloc(&p, len, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            std::fclose(f);
            return fail(EBI_E_OOM, "pinned staging allocation failed");
        }
        g_file_buf = static_cast<uint8_t*>(p);
        g_file_cap = len;
    }
    const uint64_t got = len ? std::fread(g_file_buf, 1, len, f) : 0;
    std::fclose(f);
    if (got != len) return fail(EBI_E_IO, std::string("short read of ") + path);
    return ebi_column_open(g_file_buf, len, stream, out);
}

int ebi_column_close(ebi_column* c) {
    if (!c) return EBI_OK;
    cudaStream_t s = c->stream;
    for (cudaEvent_t e : c->ev) if (e) cudaEventDestroy(e);
    void* ptrs[] = {c->d_file, c->d_chunks, c->d_tiles, c->d_acc, c->d_res, c->d_tile_counts, c->d_tile_offsets,
                    c->d_scratch_mask, c->d_buff, c->d_tot, c->d_units, c->d_parts, c->d_segs};
    for (void* p : ptrs) if (p) cudaFreeAsync(p, s);
    if (c->h_res || c->h_tot) {
        cudaStreamSynchronize(s);  // no copy into the slots is pending when they are recycled
        if (c->h_res) g_pinned.give(c->h_res);
        if (c->h_tot) g_pinned_tot.give(c->h_tot);
    }
    delete c;
    return EBI_OK;
}

uint64_t ebi_column_num_records(const ebi_column* c) { return c ? c->n_records : 0; }
uint64_t ebi_column_num_chunks(const ebi_column* c) { return c ? c->n_chunks : 0; }
uint64_t ebi_column_device_bytes(const ebi_column* c) { return c ? c->device_bytes : 0; }
int ebi_column_set_copy_wait(ebi_column* c, int64_t cycles) {
    if (!c) return fail(EBI_E_INVALID, "column is null");
    c->copy_wait = cycles < 0 ? kWaitCycles : cycles;
    return EBI_OK;
}
int ebi_column_scheme(const ebi_column* c) { return c ? c->scheme : -1; }

int ebi_column_chunk_info(const ebi_column* c, uint64_t i, uint64_t* phys, uint64_t* size, uint64_t* row,
                          uint64_t* rows) {
    if (!c || i >= c->n_chunks) return fail(EBI_E_INVALID, "chunk index out of range");
    const ChunkDesc& cd = c->chunks[i];
    if (phys) *phys = cd.byte_off;
    if (size) *size = cd.byte_len;
    if (row) *row = cd.row_off;
    if (rows) *rows = cd.n_rows;
    return EBI_OK;
}

int ebi_column_set_precision(ebi_column* c, int32_t precision) {
    if (!c) return fail(EBI_E_INVALID, "column is null");
    if (precision > 12) return fail(EBI_E_INVALID, "precision past PRECISION_MAP (0..12)");
    c->precision = precision < 0 ? -1 : precision;
    return EBI_OK;
}

int ebi_filter(ebi_column* c, const ebi_predicate* pred, const uint64_t* d_mask, int64_t chunk_id,
               uint64_t* d_out_mask, void* stream) {
    if (!c || !d_out_mask) return fail(EBI_E_INVALID, "column or output is null");
    int st = check_pred(pred);
    if (!st) st = check_supported(c);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    st = run_scan(c, OP_FILTER, pred, d_mask, chunk_id, d_out_mask, nullptr, s);
    if (st) return st;
    QueryParams q = base_params(c);
    q.op = OP_FILTER;
    q.chunk_id = chunk_id;
    return finish(c, q, s);
}

int ebi_filter_agg(ebi_column* c, const ebi_predicate* pred, const uint64_t* d_mask, int64_t chunk_id,
                   uint64_t* d_out_mask, double* sum, double* mn, double* mx, uint64_t* n_selected, void* stream) {
    if (!c) return fail(EBI_E_INVALID, "column is null");
    int st = check_pred(pred);
    if (!st) st = check_supported(c);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t agg = (sum ? AGG_SUM : 0u) | (mn ? AGG_MIN : 0u) | (mx ? AGG_MAX : 0u);
    st = run_scan(c, OP_FILTER_AGG, pred, d_mask, chunk_id, d_out_mask, nullptr, s, agg);
    if (st) return st;
    QueryParams q = base_params(c);
    q.agg = agg;
    q.op = OP_FILTER_AGG;
    q.chunk_id = chunk_id;
    q.in_mask = reinterpret_cast<const uint32_t*>(d_mask);
    st = finish(c, q, s);
    if (st) return st;
    if (sum) *sum = c->h_res->sum;
    if (mn) *mn = c->h_res->min;
    if (mx) *mx = c->h_res->max;
    if (n_selected) *n_selected = c->h_res->count;
    return EBI_OK;
}

static int agg_common(ebi_column* c, const uint64_t* d_mask, int64_t chunk_id, void* stream, uint32_t agg) {
    if (!c) return fail(EBI_E_INVALID, "column is null");
    int st = check_supported(c);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    st = run_scan(c, OP_AGG, nullptr, d_mask, chunk_id, nullptr, nullptr, s, agg);
    if (st) return st;
    QueryParams q = base_params(c);
    q.agg = agg;
    q.op = OP_AGG;
    q.chunk_id = chunk_id;
    q.in_mask = reinterpret_cast<const uint32_t*>(d_mask);
    return finish(c, q, s);
}

int ebi_sum(ebi_column* c, const uint64_t* d_mask, int64_t chunk_id, double* out, void* stream) {
    const int st = agg_common(c, d_mask, chunk_id, stream, AGG_SUM);
    if (!st && out) *out = c->h_res->sum;
    return st;
}
int ebi_min(ebi_column* c, const uint64_t* d_mask, int64_t chunk_id, double* out, void* stream) {
    const int st = agg_common(c, d_mask, chunk_id, stream, AGG_MIN);
    if (!st && out) *out = c->h_res->min;
    return st;
}
int ebi_max(ebi_column* c, const uint64_t* d_mask, int64_t chunk_id, double* out, void* stream) {
    const int st = agg_common(c, d_mask, chunk_id, stream, AGG_MAX);
    if (!st && out) *out = c->h_res->max;
    return st;
}

int ebi_materialize(ebi_column* c, const uint64_t* d_mask, int64_t chunk_id, double* d_out, uint64_t out_cap,
                    uint64_t* n_out, void* stream) {
    if (!c || (!d_out && out_cap)) return fail(EBI_E_INVALID, "column or output is null");
    int st = check_supported(c);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (c->scheme != EBI_BUFF) {
        if ((st = ensure_scratch(c, s))) return st;
        return run_materialize_values(c, nullptr, d_mask, chunk_id, d_out, out_cap, n_out, s);
    }
    if (d_mask && (st = ensure_scratch(c, s))) return st;
    return run_materialize(c, d_mask, chunk_id, d_out, out_cap, n_out, s, false, nullptr);
}

int ebi_filter_materialize(ebi_column* c, const ebi_predicate* pred, const uint64_t* d_mask, int64_t chunk_id,
                           double* d_out, uint64_t out_cap, uint64_t* n_out, void* stream) {
    if (!c || (!d_out && out_cap)) return fail(EBI_E_INVALID, "column or output is null");
    int st = check_pred(pred);
    if (!st) st = check_supported(c);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if ((st = ensure_scratch(c, s))) return st;
    if (c->scheme != EBI_BUFF) return run_materialize_values(c, pred, d_mask, chunk_id, d_out, out_cap, n_out, s);
    // filter into the scratch mask, counting per tile, then materialize it
    st = run_scan(c, OP_FILTER, pred, d_mask, chunk_id, c->d_scratch_mask, c->d_tile_counts, s);
    if (st) return st;
    return run_materialize(c, c->d_scratch_mask, chunk_id, d_out, out_cap, n_out, s, true, nullptr);
}

// Decoder::materialize without allocating: the per-tile counts and offsets go
// to the fixed scratch of static_scratch.cu instead of the column's scratch.
int ebi_materialize_static(ebi_column* c, const uint64_t* d_mask, int64_t chunk_id, double* d_out, uint64_t out_cap,
                           uint64_t* n_out, void* stream) {
    if (!c || (!d_out && out_cap)) return fail(EBI_E_INVALID, "column or output is null");
    int st = check_supported(c);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t tb, tn;
    tile_range(c, chunk_id, &tb, &tn);
    if (tn > kStaticTiles) {
        char buf[160];
        std::snprintf(buf, sizeof buf,
                      "ebi_materialize_static: the query covers %u tiles, the fixed scratch holds at most %u "
                      "(use ebi_materialize)", tn, kStaticTiles);
        return fail(EBI_E_INVALID, buf);
    }
    int dev = -1;
    CK(cudaGetDevice(&dev));
    if (dev != c->device) {
        char buf[128];
        std::snprintf(buf, sizeof buf, "ebi_materialize_static: the column lives on device %d, device %d is current",
                      c->device, dev);
        return fail(EBI_E_INVALID, buf);
    }
    unsigned long long* counts = nullptr;
    unsigned long long* offsets = nullptr;
    CK(static_scratch(&counts, &offsets));
    // Nothing here has to start at zero: the count pass writes the count of
    // every tile in [0, tn) and the scan writes every offset it reads back.
    if (int st2 = begin_query(c, s)) return st2;
    QueryParams q = base_params(c);
    q.op = OP_FILTER;  // only the status is folded
    q.chunk_id = chunk_id;
    q.in_mask = reinterpret_cast<const uint32_t*>(d_mask);
    q.out_vals = d_out;
    q.out_cap = out_cap;
    uint64_t total = 0;
    if (c->scheme == EBI_BUFF && !d_mask) {
        for (uint32_t t = tb; t < tb + tn; ++t) {
            const Tile& tl = c->tiles.tiles[t];
            const uint32_t n = c->chunks[tl.chunk].n_rows;
            total += tl.begin < n ? std::min<uint64_t>(kBuffTileRows, n - tl.begin) : 0;
        }
        if (total > out_cap) {
            if (n_out) *n_out = total;
            return fail(EBI_E_INVALID, "output buffer smaller than the values to write");
        }
        const uint64_t base_row = chunk_id >= 0 && static_cast<uint64_t>(chunk_id) < c->n_chunks ? c->chunks[chunk_id].row_off : 0;
        const bool quiet = c->buff_all_readable;  // nothing can raise: no fold
        CK(launch_buff_materialize(q, tb, tn, offsets, base_row, c->buff_max_bits > 32, quiet, s));
        if (quiet) {
            if (int st3 = finish_quiet(c, s)) return st3;
            if (n_out) *n_out = total;
            return EBI_OK;
        }
    } else {
        q.tile_counts = counts;
        if (c->scheme == EBI_BUFF) {
            CK(launch_buff_count(q, tb, tn, s));
            CK(launch_tile_scan(counts, offsets, tn, s));
            const uint64_t base_row = chunk_id >= 0 && static_cast<uint64_t>(chunk_id) < c->n_chunks ? c->chunks[chunk_id].row_off : 0;
            CK(launch_buff_materialize(q, tb, tn, offsets, base_row, c->buff_max_bits > 32, false, s));
        } else {
            CK(launch_values(c, q, tb, tn, VAL_COUNT, nullptr, s));
            CK(launch_tile_scan(counts, offsets, tn, s));
            CK(launch_values(c, q, tb, tn, VAL_MATERIALIZE, offsets, s));
        }
        CK(cudaMemcpyAsync(&c->h_res->count, offsets + tn, 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        total = c->h_res->count;
    }
    st = finish(c, q, s);
    if (st) return st;
    if (n_out) *n_out = total;
    if (total > out_cap) return fail(EBI_E_INVALID, "output buffer smaller than the values to write");
    return EBI_OK;
}

int ebi_column_set_timing(ebi_column* c, int enable) {
    if (!c) return fail(EBI_E_INVALID, "column is null");
    if (enable && !c->ev[0]) {
        for (cudaEvent_t& e : c->ev) CK(cudaEventCreate(&e));
    }
    c->timing = enable != 0;
    return EBI_OK;
}

int ebi_column_last_times(const ebi_column* c, ebi_segment_times* out) {
    if (!c || !out) return fail(EBI_E_INVALID, "column or output is null");
    *out = c->last;
    return EBI_OK;
}

const char* ebi_last_error(void) { return g_last_error.c_str(); }
uint64_t ebi_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

}  // extern "C"
