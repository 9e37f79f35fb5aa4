// internal.h -- host-side interfaces between the engine's translation units.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "common.cuh"

namespace ebi {

// Counts kernel launches (ebi_kernel_launches()).
void count_launch(uint64_t n = 1);
void set_last_error(const std::string& msg);
// Raises fn's dynamic shared-memory limit to at least `bytes` on the current
// device (the limit belongs to the function in each device's context); a
// no-op below the 48 KB default and once a device already allows as much.
cudaError_t allow_dynamic_smem(const void* fn, size_t bytes);

// Tiles of a column: chunk c owns tiles [first_tile[c], first_tile[c + 1]).
struct TileMap {
    std::vector<Tile> tiles;
    std::vector<uint32_t> first_tile;  // n_chunks + 1
};

// ---- BUFF (buff.cu) --------------------------------------------------------
constexpr uint32_t kBuffTileRows = 8192;  // 256 threads x 32 rows
TileMap buff_tiles(const std::vector<ChunkDesc>& chunks);
// Filter / filter+agg / agg over tiles [tile_begin, tile_begin + n_tiles).
cudaError_t launch_buff_query(const QueryParams& q, uint32_t tile_begin, uint32_t n_tiles, cudaStream_t s);
// Shared-memory ring for columns whose widest chunk has np_max byte planes
// and tb_max tail bits; *ctas_per_sm receives the CTAs that fit one SM.
StageLayout buff_stage_layout(uint32_t np_max, uint32_t tb_max, uint32_t* ctas_per_sm);
// Pipelined scan (bulk copies into a shared-memory ring): filter without tile
// counts, filter+agg and agg.  grid = persistent CTAs.
// The last CTA folds the query into *res (no finalize launch): exactly, from
// integer totals, when fast_ok (one frac for every chunk, no constant chunk)
// and the totals stay below 2^53 ulps; else in chunk order from acc.
cudaError_t launch_buff_scan(const QueryParams& q, const BuffChunkInfo* info, uint32_t tile_begin, uint32_t n_tiles,
                            const StageLayout& L, uint32_t grid, ScanTotals* T, QueryResult* res, uint32_t frac,
                            bool fast_ok, cudaStream_t s);
// Rows of the bitmask per tile into q.tile_counts[tile - tile_begin].
cudaError_t launch_buff_count(const QueryParams& q, uint32_t tile_begin, uint32_t n_tiles, cudaStream_t s);
// Writes the decoded values of the selected rows at tile_offsets[tile - tile_begin] + rank
// (with a bitmask) or at their row - first row of the query (without).
// wide: some readable chunk is more than 32 bits wide (else the kernel built
// for 32-bit deltas runs).  quiet: every chunk the pass reads is readable and
// no bitmask is given, so the chunks' accumulators are left untouched and the
// caller folds nothing.
cudaError_t launch_buff_materialize(const QueryParams& q, uint32_t tile_begin, uint32_t n_tiles,
                                    const unsigned long long* tile_offsets, uint64_t base_row, bool wide, bool quiet,
                                    cudaStream_t s);

// ---- register-streaming BUFF scan (buff_stream.cu) -------------------------
// Columns whose readable chunks are all 8..32 bits wide.  A unit is 2,048
// rows of one chunk ({chunk, first row}); chunk c owns units
// [first_unit[c], first_unit[c + 1]).
constexpr uint32_t kBuffUnitRows = 2048;
std::vector<uint2> buff_units(const std::vector<ChunkDesc>& chunks, std::vector<uint32_t>& first_unit);
// Units per chunk when every chunk but the last holds the same number of units
// and the last no more, else 0.
uint32_t buff_uniform_units(const std::vector<uint32_t>& first_unit);
// Filter / filter+agg / agg over units [unit_base, unit_base + n_units) with
// persistent CTAs, by the kernel built for chunks `bits` wide (the column's
// most common width; other widths run a slower general path); the last CTA
// folds the query into *res as launch_buff_scan does.  fold: bit 0 the exact
// integer total may apply (fast_ok of launch_buff_scan), bit 1 it always
// applies (no per-chunk accumulators).
// upc: units per chunk when every chunk but the last holds exactly upc units
// (and the last at most upc; unit_base a multiple of upc), else 0.
cudaError_t launch_buff_stream(const QueryParams& q, const BuffChunkInfo* info, const uint2* units, uint32_t unit_base,
                               uint32_t n_units, uint32_t upc, uint32_t bits, uint32_t sms, ScanTotals* T,
                               QueryResult* res, uint32_t frac, uint32_t fold, cudaStream_t s);

// ---- BUFF plane layout (buff_layout.cu) ------------------------------------
// One block of the repack at column open: `len` 16-byte words from
// src + src_off to dst + dst_off (dst_off 16-byte aligned).
struct RepackSeg {
    uint64_t src_off, dst_off, len;
};
// Plane layout of a BUFF file: fills every readable chunk's planes / tail /
// stride in `info` (device offsets), appends its copies (as blocks of at most
// 64 KB) to `segs` and returns the device buffer size (before padding).
uint64_t buff_plan_layout(std::vector<BuffChunkInfo>& info, std::vector<RepackSeg>& segs);
// Copies the segments from the raw file image `src` (device memory) into `dst`.
cudaError_t launch_buff_repack(const uint8_t* src, uint8_t* dst, const RepackSeg* d_segs, uint32_t n_segs,
                               cudaStream_t s);

// ---- value codecs: one CTA per chunk, modes of values.cuh (VAL_*) ----------
// chunk_offsets[chunk - chunk_begin] (+1 entry) are the exclusive scan of a
// VAL_COUNT pass; the count pass writes q.tile_counts[chunk - chunk_begin].
cudaError_t launch_rle(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                       const unsigned long long* chunk_offsets, cudaStream_t s);
cudaError_t launch_raw(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                       const unsigned long long* chunk_offsets, cudaStream_t s);
// Gorilla: one warp per chunk following the stream several records per step.
// Chunks whose aligned byte span is at most kGorillaStageCap are staged in
// shared memory; gorilla_stage_bytes is the per-CTA staging size of a column.
constexpr uint32_t kGorillaStageCap = 100 * 1024;
uint32_t gorilla_stage_bytes(const ChunkDesc* chunks, uint64_t n);
cudaError_t launch_gorilla(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                           const unsigned long long* chunk_offsets, cudaStream_t s);
// Gorilla, Chimp, Chimp128, ElfOnChimp, Elf (q.scheme selects the decoder).
cudaError_t launch_xor(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                       const unsigned long long* chunk_offsets, cudaStream_t s);

// ---- Elf decimal tables (elf_tables.cu) ------------------------------------
// Device address of the tables of elf_dev.cuh for the current device; built
// and uploaded on first use per device (a synchronous copy).
cudaError_t elf_tables(const double** out);

// ---- fixed scratch of ebi_materialize_static (static_scratch.cu) ----------
constexpr uint32_t kStaticTiles = 16384;  // tiles per call: 2 x 128 KB of counts and offsets
// Device addresses of the fixed per-tile counts (kStaticTiles entries) and
// offsets (kStaticTiles + 1) for the current device; looked up on first use.
cudaError_t static_scratch(unsigned long long** counts, unsigned long long** offsets);

// ---- batched queries (batch.cu) --------------------------------------------
enum BatchItemKind : uint32_t {
    ITEM_BUFF_TILE = 0,  // unit = tile index of the query's column
    ITEM_RAW = 1,        // unit = chunk
    ITEM_RLE = 2,
    ITEM_GORILLA = 3,    // chunks [unit, unit + count), one warp each
    ITEM_CHIMP = 4,
    ITEM_CHIMP128 = 5,
    ITEM_ELF_CHIMP = 6,  // unit = chunk
    ITEM_ELF = 7,
};
struct BatchItem {
    uint32_t query;  // index into the batch's QueryParams
    uint32_t kind;   // BatchItemKind
    uint32_t unit;   // first tile (BUFF) or chunk
    // BUFF / Uncompressed / RLE: tiles or chunks [unit, unit + count);
    // Chimp family: queries sharing the chunk; Gorilla: chunks | (queries sharing them) << 8
    uint32_t count;
};
// Queries over one Gorilla column that one batch item serves at once: up to
// kGorillaShare with the walk's state in registers, up to kGorillaShareWide
// with it in shared memory.
constexpr uint32_t kGorillaShare = 3;
constexpr uint32_t kGorillaShareWide = 8;

// Work-item tiling of a batch, per codec family and column-size bucket
// (size_bucket): how many 8,192-row BUFF tiles, Uncompressed / RLE chunks and
// Gorilla chunks (one warp each, eight warps per item) one item covers.
constexpr int kSizeBuckets = 3;
constexpr uint32_t kMaxItemTiles = 16;     // BUFF tiles or value chunks per item
constexpr uint32_t kMaxGorillaChunks = 64;  // Gorilla chunks per item
struct BatchTiling {
    uint32_t buff_tiles[kSizeBuckets];
    uint32_t value_chunks[kSizeBuckets];
    uint32_t gorilla_chunks[kSizeBuckets];
};
// Bucket of a column of n_records rows: < 262,144, < 4,194,304, larger.
int size_bucket(uint64_t n_records);
BatchTiling default_tiling();
// Appends the items of one query over a column.  Gorilla items carry their
// chunk count in the low byte of count (callers add a sharing count above it).
void column_items(int scheme, uint64_t n_chunks, uint32_t n_tiles, uint64_t n_records, const BatchTiling& t,
                  uint32_t query, std::vector<BatchItem>& out);
// The items of queries [first, first + n) of a batch, all over one column:
// a Chimp-family chunk is decoded once for up to 32 of them, a Gorilla chunk
// group walked once for up to kGorillaShareWide; other codecs get one set of
// items per query.
void shared_column_items(int scheme, uint64_t n_chunks, uint32_t n_tiles, uint64_t n_records, const BatchTiling& t,
                         uint32_t first, uint32_t n, std::vector<BatchItem>& out);
// How many items column_items appends for such a column.
uint64_t column_item_count(int scheme, uint64_t n_chunks, uint32_t n_tiles, uint64_t n_records, const BatchTiling& t);
// Relative cost of one item (device time of the 8,192-row units it covers,
// measured on the single-column kernels), for the cost-descending order.
double item_cost(uint32_t kind, uint32_t count);
// Stable reorder of items by descending item_cost, in linear time (the costs
// take a handful of values).
void order_by_cost(std::vector<BatchItem>& items);
// Dynamic shared memory of the batch kernel; prepare_batch_kernel raises the
// kernel's shared-memory limit to it on the current device (outside any capture).
size_t batch_smem_bytes();
cudaError_t prepare_batch_kernel();
// Runs every item (persistent grid of `grid` CTAs pulling from *d_counter,
// which the launch resets); each query's partials land in its own acc.
cudaError_t launch_batch(const QueryParams* d_qp, const BatchItem* d_items, uint32_t n_items, unsigned int* d_counter,
                         uint32_t grid, cudaStream_t s);
// Folds query i into d_res[i] (one CTA per query) and re-arms its acc.
cudaError_t launch_batch_finalize(const QueryParams* d_qp, QueryResult* d_res, uint32_t n_queries, cudaStream_t s);

// ---- shared kernels (query.cu) ---------------------------------------------
// acc[c].selected = chunk passes chunk_id and intersects the mask (or no mask).
cudaError_t launch_select_chunks(const QueryParams& q, cudaStream_t s);
// Exclusive scan of n tile counts into offsets (n + 1 entries; offsets[n] = total).
cudaError_t launch_tile_scan(const unsigned long long* counts, unsigned long long* offsets, uint32_t n,
                             cudaStream_t s);
// Folds the per-chunk partials in chunk order into *res and re-arms acc.
// Codecs other than BUFF fold over a grid through `parts`: value_slices(n_chunks)
// ValParts and a counter behind them (at rest 0).
cudaError_t launch_finalize(const QueryParams& q, QueryResult* res, ValPart* parts, cudaStream_t s);
// Sets acc to its rest values (once, at open).
cudaError_t launch_acc_init(ChunkAcc* acc, uint32_t n, cudaStream_t s);

}  // namespace ebi
