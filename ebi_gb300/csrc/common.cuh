// common.cuh -- types and device helpers shared by the engine's translation units.
//
// Layout in HBM (one column = one EBI1 file):
//   file      the EBI1 bytes exactly as stored on disk, plus 64 zero bytes of
//             padding so that aligned 16-byte over-reads at a chunk's end stay
//             inside the allocation;
//   chunks    one ChunkDesc (32 B) per chunk: byte range and row range;
//   tiles     the unit of work of the codec's main kernel (Tile, 8 B each);
//   acc       one ChunkAcc per chunk: exact/compensated partial results.
//             Every query leaves them "at rest" (neutral) for the next one.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/ebi_gpu.h"

namespace ebi {

constexpr uint64_t kNanBits = 0x7ff8000000000000ull;  // f64::NAN.to_bits()
constexpr int kFilePad = 64;                           // zero bytes after the file in HBM
constexpr long long kWaitCycles = 4000000000ll;        // default limit of a bounded wait: about 2 s at 2 GHz

// Chunk geometry (GeneralChunkHandle, decoder.rs:283-352).
struct ChunkDesc {
    uint64_t byte_off;  // physical offset of the chunk in the file
    uint64_t byte_len;  // chunk_size()
    uint64_t row_off;   // logical offset (first global row id)
    uint32_t n_rows;    // number_of_records()
    uint32_t flags;     // kChunkBadGeometry: byte range outside the file
};
constexpr uint32_t kChunkBadGeometry = 1;

// BUFF chunk header facts, parsed on the host at open (query independent).
// BUFF chunks live in HBM in the column's plane layout (buff_layout.cu),
// not at their file offsets: every byte plane and the tail plane start on a
// 128-byte boundary, planes `stride` bytes apart.
struct BuffChunkInfo {
    uint64_t planes;   // device-buffer offset of the first byte plane
    uint64_t tail;     // device-buffer offset of the tail plane
    int64_t base;      // fixed-point base
    uint32_t n, bits, frac;
    uint32_t status;   // error to raise when the chunk is read (0: readable)
    uint64_t stride;   // bytes from one byte plane to the next
};

// Shared-memory ring of the pipelined BUFF scan.
struct StageLayout {
    uint32_t stages;        // ring depth
    uint32_t plane_stride;  // bytes per plane slot
    uint32_t np_max;        // plane slots per stage
    uint32_t tail_stride;   // bytes of the tail slot
    uint32_t stage_bytes;   // np_max * plane_stride + tail_stride
    uint32_t data_offset;   // start of the stages (after barriers and per-stage metadata)
};

struct Tile {
    uint32_t chunk;
    uint32_t begin;  // first row (BUFF), first field (RLE) or first segment (XOR) of the tile
};

// Per-chunk partial results.  Written by the codec kernels, consumed and
// re-armed (back to these rest values) by finalize_kernel.
struct ChunkAcc {
    unsigned long long isum;   // BUFF: wrapping u64 sum of selected deltas       (rest 0)
    unsigned long long count;  // rows selected                                   (rest 0)
    unsigned long long dmax;   // BUFF: max selected delta                        (rest 0)
    unsigned long long dmin;   // BUFF: min selected delta                        (rest ~0)
    double fsum_hi;            // other codecs: double-double chunk sum           (rest 0)
    double fsum_lo;            //                                                 (rest 0)
    double fmin;               // other codecs: min / max of selected values      (rest +inf / -inf)
    double fmax;
    uint32_t status;           // first error of the chunk                        (rest 0)
    uint32_t selected;         // chunk passes chunk_id / bitmask selection       (rest 0)
    uint32_t ndecoded;         // XOR/RLE: decoded length (NaN end marker)        (rest 0)
    uint32_t pad;
};

// Query-wide totals of the fused BUFF scans.  Every CTA stores its totals in
// its own slot (kScanSlots of them follow this struct in the same
// allocation, from byte kSlotOffset) and counts itself in `done`; the last CTA reduces the slots and
// folds.  At rest (re-armed by that CTA): zeros, max_fixed = INT64_MIN,
// min_fixed = INT64_MAX, bad_chunk = ~0.
struct ScanTotals {
    unsigned long long sum_fixed;  // wrapping sum of every (CTA, chunk) piece of sum_with_bitmask's integer
    unsigned long long abs_bound;  // saturating sum of |piece|: bounds every chunk total and their prefix sums
    unsigned long long count;      // rows selected
    long long max_fixed, min_fixed;
    unsigned int done;             // CTAs finished
    unsigned int bad_chunk;        // lowest chunk index that raised an error
    unsigned int nonexact;         // a piece reached 2^53
    unsigned int next;             // streaming scan: the next batch of units to hand out
    unsigned int pad;
};
constexpr uint32_t kScanSlots = 1024;  // CTAs of one scan launch, at most

// Running query totals of one warp (kept by lane 0), and of one CTA in its slot.
struct alignas(16) WarpTot {
    unsigned long long sum_fixed, count;
    unsigned long long abs_bound;  // saturating (integer pipes: no FP64 on the scan's tail)
    long long max_fixed, min_fixed;
    unsigned int nonexact;
};
// The CTA slots start 64 bytes into the scan-totals allocation (16-byte loads
// and stores of whole slots stay aligned).
constexpr size_t kSlotOffset = 64;
static_assert(sizeof(ScanTotals) <= kSlotOffset, "slots follow the totals");
static_assert(sizeof(WarpTot) % 16 == 0, "whole 16-byte words per slot");
__host__ __device__ inline WarpTot* scan_slots(ScanTotals* T) {
    return reinterpret_cast<WarpTot*>(reinterpret_cast<char*>(T) + kSlotOffset);
}
constexpr size_t kScanTotalsBytes = kSlotOffset + kScanSlots * sizeof(WarpTot);


struct QueryResult {
    uint32_t status;       // status of the first failing chunk in chunk order
    uint32_t bad_chunk;    // its index
    double sum, min, max;
    unsigned long long count;  // rows selected / values written
};

// A partial fold of the non-BUFF codecs' chunk results over one slice of
// kSliceChunks chunks (finalize.cuh): the signed 192-bit fixed-point sum of
// the chunks' compensated sums, min / max as ordered keys, rows, and the
// lowest failing chunk.  The column's fold scratch holds one per slice; the
// first word after the last one is the fold's CTA counter (rest 0).
struct alignas(16) ValPart {
    unsigned long long w0, w1, w2;  // the sum, two's complement, in units of 2^(top - 1172)
    unsigned long long mn, mx;      // ordered keys (rest: +inf / -inf)
    unsigned long long cnt;
    uint32_t top;      // largest exponent field of the slice's finite nonzero terms (0: none)
    uint32_t special;  // 1: a NaN term, 2: +inf, 4: -inf
    uint32_t bad;      // lowest chunk index with an error status (0xffffffff: none)
    uint32_t bad_st;   // its status
};
static_assert(sizeof(ValPart) == 64, "four 16-byte words per slice");
constexpr uint32_t kSliceChunks = 64;
__host__ __device__ inline uint32_t value_slices(uint32_t n_chunks) {
    return (n_chunks + kSliceChunks - 1) / kSliceChunks;
}

enum Op : int {
    OP_FILTER = 0,      // bitmask only
    OP_FILTER_AGG = 1,  // bitmask + sum/min/max/count of the selected rows
    OP_AGG = 2,         // sum/min/max of the mask rows (all rows without a mask)
    OP_COUNT = 3,       // per-tile counts of the mask rows (materialize pass 1)
};

// Arguments of the per-chunk query kernels (passed by value).
struct QueryParams {
    const uint8_t* file;
    const ChunkDesc* chunks;
    ChunkAcc* acc;
    const Tile* tiles;
    uint32_t n_tiles;
    uint32_t n_chunks;
    uint64_t n_records;
    int64_t chunk_id;          // < 0: all chunks
    const uint32_t* in_mask;   // u32 view of the u64 bitmask, or null
    uint32_t* out_mask;        // u32 view, or null
    int op;                    // Op
    int out_atomic;            // out_mask is pre-zeroed and words may be shared: atomicOr
    ebi_predicate pred;
    // materialize
    double* out_vals;
    uint64_t out_cap;
    unsigned long long* tile_counts;  // per tile
    int32_t precision;         // BUFF controlled precision, < 0: full
    int scheme;
    uint32_t agg;              // AGG_* aggregates the caller asked for (the count is always kept)
    const BuffChunkInfo* binfo;  // BUFF: header facts per chunk
    int pred_on;               // value codecs: the predicate selects rows (filter, filter+agg, filter_materialize)
    uint32_t stage_bytes;      // Gorilla: shared-memory staging size per chunk (0: read through L1)
    const double* dec_tab;     // Elf / ElfOnChimp: decimal tables of elf_dev.cuh (device memory)
    long long copy_wait;       // limit (SM clocks) of a kernel's waits for its bulk copies to land; <= 0: one look
    int zero_out;              // Uncompressed / RLE: each chunk's CTA zeroes its own out_mask words first (no memset)
    int own_words;             // chunks start on 32-row boundaries in row order and decode no row past their range
    // Chimp / Chimp128 / Elf / ElfOnChimp single-column scans: the segment
    // starts of every launched chunk are converged by a separate kernel into
    // this scratch (kSegsPerChunk per chunk, by launch index); null: in the
    // chunk's own kernel
    struct SegState* segs;
};

// One segment of an XOR chunk's control parse after convergence: its start
// state (PState packed), and the records and first error of its parse from there.
struct SegState {
    unsigned long long in;
    uint32_t n, fail;
};
constexpr uint32_t kSegsPerChunk = 256;

// Passes of the value-codec kernels (one CTA per chunk).
//   VAL_SCAN         filter / filter+agg / agg into the output bitmask and acc
//   VAL_COUNT        rows a materialize will write, per chunk (tile_counts)
//   VAL_MATERIALIZE  writes those rows at chunk_offsets[chunk] onwards
enum ValMode : int { VAL_SCAN = 0, VAL_COUNT = 1, VAL_MATERIALIZE = 2 };

enum : uint32_t { AGG_SUM = 1, AGG_MIN = 2, AGG_MAX = 4, AGG_ALL = 7 };

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 ldg16(const void* p) { return __ldg(reinterpret_cast<const uint4*>(p)); }

// 32 bytes starting at an arbitrary address p, as 8 little-endian words.
// Reads the three aligned 16-byte blocks that cover them (two when p is
// 16-byte aligned) and realigns in registers.  Over-reads up to 15 bytes past
// p + 32, which the file padding keeps inside the allocation.
__device__ __forceinline__ void load32(const uint8_t* p, uint32_t (&w)[8]) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uint8_t* q = reinterpret_cast<const uint8_t*>(a & ~uintptr_t(15));
    const uint32_t s = static_cast<uint32_t>(a & 15);
    uint4 x0 = ldg16(q), x1 = ldg16(q + 16);
    uint4 x2 = s ? ldg16(q + 32) : make_uint4(0, 0, 0, 0);
    uint32_t v[12] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w, x2.x, x2.y, x2.z, x2.w};
    const bool s8 = s & 8, s4 = s & 4;
#pragma unroll
    for (int j = 0; j < 10; ++j) v[j] = s8 ? v[j + 2] : v[j];
#pragma unroll
    for (int j = 0; j < 9; ++j) v[j] = s4 ? v[j + 1] : v[j];
    const uint32_t bs = (s & 3) * 8;
#pragma unroll
    for (int j = 0; j < 8; ++j) w[j] = __funnelshift_r(v[j], v[j + 1], bs);
}

__device__ __forceinline__ uint32_t load_u32_unaligned(const uint8_t* p) {
    return uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24);
}
__device__ __forceinline__ uint64_t load_u64_unaligned(const uint8_t* p) {
    return uint64_t(load_u32_unaligned(p)) | (uint64_t(load_u32_unaligned(p + 4)) << 32);
}

// The 32 mask bits of global rows [r, r + 32), zero past n_records.
__device__ __forceinline__ uint32_t mask_word(const uint32_t* m, uint64_t r, uint64_t n_records) {
    if (r >= n_records) return 0;
    const uint64_t w = r >> 5;
    const uint32_t sh = static_cast<uint32_t>(r & 31);
    uint32_t lo = m[w];
    uint32_t hi = (sh && ((w + 1) << 5) < n_records) ? m[w + 1] : 0u;
    uint32_t v = __funnelshift_r(lo, hi, sh);
    const uint64_t left = n_records - r;
    if (left < 32) v &= (1u << left) - 1u;
    return v;
}

// Writes the 32 result bits of global rows [r, r + 32).
__device__ __forceinline__ void store_mask_word(uint32_t* m, uint64_t r, uint32_t bits, bool atomic) {
    const uint64_t w = r >> 5;
    const uint32_t sh = static_cast<uint32_t>(r & 31);
    if (!atomic) { m[w] = bits; return; }
    if (sh == 0) { if (bits) atomicOr(&m[w], bits); return; }
    const uint32_t lo = bits << sh, hi = bits >> (32 - sh);
    if (lo) atomicOr(&m[w], lo);
    if (hi) atomicOr(&m[w + 1], hi);
}

__device__ __forceinline__ void set_status(ChunkAcc* a, uint32_t code) { atomicCAS(&a->status, 0u, code); }

// With q.zero_out (an Uncompressed or RLE scan over every chunk of a column
// whose chunks start on 32-row boundaries, in row order, and decode no more
// rows than their range), chunk c's words of the output bitmask belong to its
// CTA alone: every thread of the CTA calls this before the CTA's first
// barrier, and the chunk's ORs follow that barrier.  The last chunk also
// zeroes the rest of the mask's last u64 word.
__device__ __forceinline__ void zero_chunk_words(const QueryParams& q, const ChunkDesc& cd, uint32_t c) {
    if (!q.zero_out) return;
    const uint64_t end = ((q.n_records + 63) >> 6) * 2;  // u32 words of the mask
    const uint64_t w0 = min(cd.row_off >> 5, end);
    const uint64_t w1 = c + 1 == q.n_chunks ? end : min((cd.row_off + cd.n_rows + 31) >> 5, end);
    for (uint64_t w = w0 + threadIdx.x; w < w1; w += blockDim.x) q.out_mask[w] = 0u;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) { unsigned long long x = __shfl_xor_sync(0xffffffffu, v, o); v = x > v ? x : v; }
    return v;
}
__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) { unsigned long long x = __shfl_xor_sync(0xffffffffu, v, o); v = x < v ? x : v; }
    return v;
}

// Evaluation of a Predicate on a decoded value (decoder/query.rs:396-437).
__device__ __forceinline__ bool pred_eval(const ebi_predicate& p, double v) {
    if (p.kind == EBI_PRED_EQ) return v == p.value;
    if (p.kind == EBI_PRED_NE) return v != p.value;
    const bool s = p.start_kind == EBI_BOUND_INCLUSIVE ? v >= p.start
                 : p.start_kind == EBI_BOUND_EXCLUSIVE ? v > p.start : true;
    const bool e = p.end_kind == EBI_BOUND_INCLUSIVE ? v <= p.end
                 : p.end_kind == EBI_BOUND_EXCLUSIVE ? v < p.end : true;
    return s && e;
}

// Error-free transformation of a + b (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
// (hi, lo) += (bh, bl) in double-double arithmetic.  Once the leading sum is
// infinite or NaN the error terms are meaningless (inf - inf): the pair then
// carries the plain IEEE sum, as the sequential f64 sum does.
__device__ __forceinline__ void dd_add(double& hi, double& lo, double bh, double bl) {
    double s, e;
    two_sum(hi, bh, s, e);
    if (!isfinite(s)) {
        hi = s;
        lo = 0.0;
        return;
    }
    e += lo + bl;
    hi = s + e;
    lo = e - (hi - s);
}

}  // namespace ebi
