// column.h -- the resident column (ebi_column of include/ebi_gpu.h), shared
// by the single-query entry points (column.cu) and the batch / serving layer.
#pragma once

#include <vector>

#include "internal.h"

// internal header: the engine's own types, unqualified
using namespace ebi;

struct ebi_column {
    cudaStream_t stream = nullptr;  // stream of open/close (allocation order)
    int device = -1;                // the device current at open: every buffer of the column lives there
    uint64_t device_bytes = 0;      // device memory the column holds (resident file, tables, query scratch)
    long long copy_wait = kWaitCycles;  // limit of its kernels' waits for bulk copies (ebi_column_set_copy_wait)
    int scheme = 0;
    uint64_t n_records = 0, n_chunks = 0, file_len = 0, footer_off = 0;
    std::vector<ChunkDesc> chunks;
    TileMap tiles;
    bool rows_aligned32 = true;
    bool rows_in_order = true;  // chunk row offsets never decrease (a well-formed footer)
    bool rows_bounded = false;  // no chunk decodes rows past its range (Uncompressed; RLE with run totals checked)
    int32_t precision = -1;
    uint8_t* d_file = nullptr;
    ChunkDesc* d_chunks = nullptr;
    Tile* d_tiles = nullptr;
    ChunkAcc* d_acc = nullptr;
    QueryResult* d_res = nullptr;
    ValPart* d_parts = nullptr;  // codecs other than BUFF: the fold's slice partials and counter
    SegState* d_segs = nullptr;  // Chimp / Chimp128 / Elf / ElfOnChimp: converged segment starts (or null)
    QueryResult* h_res = nullptr;
    unsigned long long* d_tile_counts = nullptr;   // n_tiles
    unsigned long long* d_tile_offsets = nullptr;  // n_tiles + 1
    uint64_t* d_scratch_mask = nullptr;            // mask_words
    uint64_t mask_words = 0;
    // BUFF: header facts per chunk and the scan's shared-memory ring
    BuffChunkInfo* d_buff = nullptr;
    StageLayout layout{};
    uint32_t scan_grid = 0;
    ScanTotals* d_tot = nullptr;
    uint32_t buff_frac = 0;
    bool buff_fast_ok = false;
    bool buff_exact = false;     // fast_ok and sum |value| over all rows < 2^52: every query's totals exact
    bool buff_same_frac = false; // every readable chunk has frac buff_frac <= 1022 (constant chunks included)
    uint32_t buff_fixed_bits = 64;  // |base + delta| < 2^buff_fixed_bits on every readable row
    // register-streaming scan (every readable chunk 8..32 bits wide)
    bool stream_ok = false;
    uint2* d_units = nullptr;
    std::vector<uint32_t> first_unit;  // n_chunks + 1
    uint32_t units_per_chunk = 0;      // when uniform (buff_uniform_units), else 0
    uint32_t stream_bits = 0;    // most common width of the readable chunks
    uint32_t buff_max_bits = 0;  // widest readable chunk
    bool buff_all_readable = false;  // no chunk header carries an error
    uint32_t sms = 0;            // SMs of the column's device
    bool fused_pending = false;  // the last query's kernel already folded into d_res
    bool totals_pending = false; // the last query's kernel left exact totals in pending_tot for the host
    ScanTotals* pending_tot = nullptr;
    ScanTotals* h_tot = nullptr; // pinned copy of those totals
    uint32_t tot_flip = 0;       // which of the two totals blocks the next scan uses
    uint32_t stage_bytes = 0;    // Gorilla: shared-memory staging per chunk
    const double* dec_tab = nullptr;  // Elf / ElfOnChimp: the device's decimal tables
    // segment timing (ebi_column_set_timing)
    bool timing = false;
    // query start, scan end, finalize end, scan start
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool scan_marked = false;    // the query recorded ev[3]
    ebi_segment_times last{};
    uint64_t launches_at_start = 0;
};

namespace ebi {
// The column's query parameters with no query set (file, chunk table, tiles,
// accumulators, BUFF facts, staging size).
QueryParams column_params(const ebi_column* c);
}  // namespace ebi
