// buff_stream.cuh -- the register-streaming BUFF scan: filter / filter+aggregate
// / aggregate over a column whose chunks are 1 to 32 bits wide, in one launch.
//
// The column's planes sit in HBM in the aligned plane layout (buff_layout.cu),
// so a group of 64 consecutive rows owns 64 bytes of every byte plane and
// 8 * tb bytes of tail, all on 16-byte (odd tb: 8-byte) boundaries.  A unit
// of work is 2,048 rows of one chunk: lane i of a warp takes rows
// [64 i, 64 i + 64) of the unit, loads its bytes straight into registers with
// 16-byte loads (no shared memory, no barriers), assembles the u32 deltas
// with byte permutes, applies the chunk's range test (one subtract and one
// unsigned compare per row), builds its two 32-bit bitmask words and keeps
// exact per-chunk partials.  Warps take batches of 4 units from a device
// counter in column order (faster SMs take more batches) and compile the
// predicate (compile_pred: the reference's in-situ decisions) only when the
// chunk changes.  The last CTA folds the query as in the
// pipelined scan (buff_query_dev.cuh).
#pragma once

#include "buff_query_dev.cuh"

namespace ebi {
namespace {

constexpr int kStreamThreads = 256;
constexpr int kStreamWarps = kStreamThreads / 32;
constexpr uint32_t kStreamBatch = 4;  // units a warp takes at a time
static_assert(kBuffUnitRows == 32 * 64, "a unit is 64 rows per lane");

// Plain (L1-allocating) loads: the two 16-byte halves of a 32-byte sector go
// to the same lane in consecutive loads, so the second half hits L1.
__device__ __forceinline__ uint4 ldg16(const uint8_t* p) { return *reinterpret_cast<const uint4*>(p); }
__device__ __forceinline__ uint2 ldg8(const uint8_t* p) { return *reinterpret_cast<const uint2*>(p); }

// The warp's current chunk.
struct StreamChunk {
    const uint8_t* planes;
    const uint8_t* tail;
    uint64_t stride, row_off;
    int64_t base;
    uint32_t chunk, n, bits;
    uint32_t state;            // kSkip: zero words; kEmpty: no row passes; kTest
    uint32_t lo, span;         // rows pass when delta - lo <= span (unsigned)
    uint32_t use_mask, negate;
};
enum : uint32_t { kSkip = 0, kEmpty = 1, kTest = 2 };

__device__ StreamChunk stream_chunk(const QueryParams& q, ScanTotals* T, uint32_t c, bool first_unit, bool exact) {
    StreamChunk k{};
    const BuffChunkInfo ci = q.binfo[c];
    const ChunkDesc cd = q.chunks[c];
    const bool has_mask = q.in_mask != nullptr;
    const bool selected = has_mask ? q.acc[c].selected != 0 : (q.chunk_id < 0 || static_cast<uint64_t>(q.chunk_id) == c);
    if (selected && first_unit && (threadIdx.x & 31) == 0) {
        if (!has_mask && !exact) q.acc[c].selected = 1;  // read only by the chunk-ordered fold
        if (ci.status) chunk_error(q, T, c, ci.status);
    }
    k.chunk = c;
    k.n = cd.n_rows;
    k.row_off = cd.row_off;
    k.base = ci.base;
    k.bits = ci.bits;
    k.planes = q.file + ci.planes;
    k.tail = q.file + ci.tail;
    k.stride = ci.stride;
    k.state = kSkip;
    if (!selected || ci.status) return k;
    BuffPred bp;
    compile_pred(q.pred, ci.base, ci.bits, ci.frac, has_mask, bp);
    const RangeProg g = compile_prog(q, bp, ci.bits, has_mask);
    const uint64_t dmax = (1ull << ci.bits) - 1;  // bits <= 32 here
    const uint64_t hi = g.hi < dmax ? g.hi : dmax;
    k.use_mask = g.use_mask;
    k.negate = g.negate;
    if (g.empty || g.lo > hi) {
        // nothing passes the test; a negated test then passes every row
        k.state = g.negate ? kTest : kEmpty;
        k.lo = 1;
        k.span = 0;
        if (g.negate) { k.lo = 0; k.span = 0xffffffffu; k.negate = 0; }
        return k;
    }
    k.state = kTest;
    k.lo = static_cast<uint32_t>(g.lo);
    k.span = static_cast<uint32_t>(hi - g.lo);
    return k;
}

// Byte-plane words of a lane's group: NP planes (one row of storage for
// tail-only chunks, NP = 0, which read none).
template <int NP>
using PlaneWords = uint32_t[NP > 0 ? NP : 1][16];

// The four deltas of rows 4j .. 4j + 3 of a lane's group.
template <int NP, int TB>
__device__ __forceinline__ void quad_deltas(const PlaneWords<NP>& pw, const uint32_t* tw, int j, uint32_t (&d)[4]) {
    uint32_t x[NP > 0 ? NP : 1];
#pragma unroll
    for (int p = 0; p < NP; ++p) x[p] = pw[p][j] ^ 0x80808080u;
    uint32_t v[4] = {0u, 0u, 0u, 0u};
    if constexpr (NP == 0) {
        // tail-only chunk (1..7 bits): the deltas are the tail bits
    } else if constexpr (NP == 1) {
#pragma unroll
        for (int k = 0; k < 4; ++k) v[k] = __byte_perm(x[0], 0u, 0x4440u | k);
    } else if constexpr (NP == 2) {
        const uint32_t P = __byte_perm(x[1], x[0], 0x5140u), Q = __byte_perm(x[1], x[0], 0x7362u);
        v[0] = P & 0xffffu; v[1] = P >> 16; v[2] = Q & 0xffffu; v[3] = Q >> 16;
    } else if constexpr (NP == 3) {
        const uint32_t P = __byte_perm(x[1], x[0], 0x5140u), Q = __byte_perm(x[1], x[0], 0x7362u);
        // byte 3 of each selection is a don't-care byte, cleared by the mask
        v[0] = __byte_perm(x[2], P, 0x0540u) & 0xffffffu; v[1] = __byte_perm(x[2], P, 0x0761u) & 0xffffffu;
        v[2] = __byte_perm(x[2], Q, 0x0542u) & 0xffffffu; v[3] = __byte_perm(x[2], Q, 0x0763u) & 0xffffffu;
    } else {
        const uint32_t P = __byte_perm(x[1], x[0], 0x5140u), Q = __byte_perm(x[1], x[0], 0x7362u);
        const uint32_t R = __byte_perm(x[3], x[2], 0x5140u), S = __byte_perm(x[3], x[2], 0x7362u);
        v[0] = __byte_perm(R, P, 0x5410u); v[1] = __byte_perm(R, P, 0x7632u);
        v[2] = __byte_perm(S, Q, 0x5410u); v[3] = __byte_perm(S, Q, 0x7632u);
    }
    if constexpr (TB > 0) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int pos = (4 * j + k) * TB, wi = pos >> 5, sh = pos & 31;
            const uint32_t f = sh + TB <= 32 ? (tw[wi] >> sh) : __funnelshift_r(tw[wi], tw[wi + 1], sh);
            d[k] = (v[k] << TB) | (f & ((1u << TB) - 1u));
        }
    } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) d[k] = v[k];
    }
}

// The results of one lane's group of 64 rows.
struct GroupOut {
    uint32_t w0, w1;  // bitmask words of rows g0 .. g0 + 31 and g0 + 32 .. g0 + 63
    uint32_t mx, mn;  // over the selected rows' deltas
    unsigned long long sum;
};

// One lane's group of 64 rows (rows g0 .. g0 + 63 of its chunk).
//   MODE 0: every row valid, no input bitmask, not negated; sum
//   MODE 1: as 0, with min / max
//   MODE 2: rows of m0 / m1 only (input bitmask, rows past the chunk end),
//           test negated when `neg`; sum, min / max
template <int NP, int TB, int MODE>
__device__ __forceinline__ GroupOut group_body(const uint8_t* planes, const uint8_t* tail, uint64_t stride, uint32_t g0,
                                               uint32_t lo, uint32_t span, uint32_t m0, uint32_t m1, bool neg) {
    constexpr bool kSum32 = NP * 8 + TB <= 26;  // 64 deltas fit a u32 sum
    const uint8_t* pp = planes + g0;
    PlaneWords<NP> pw;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint4 x = ldg16(pp + p * stride + 16 * j);
            pw[p][4 * j] = x.x; pw[p][4 * j + 1] = x.y; pw[p][4 * j + 2] = x.z; pw[p][4 * j + 3] = x.w;
        }
    }
    uint32_t tw[2 * TB + 1];
    tw[2 * TB] = 0;
    if constexpr (TB > 0) {
        const uint8_t* tp = tail + uint64_t(g0 / 64) * (8 * TB);
        if constexpr (TB % 2 == 0) {
#pragma unroll
            for (int j = 0; j < TB / 2; ++j) {
                const uint4 x = ldg16(tp + 16 * j);
                tw[4 * j] = x.x; tw[4 * j + 1] = x.y; tw[4 * j + 2] = x.z; tw[4 * j + 3] = x.w;
            }
        } else {
#pragma unroll
            for (int j = 0; j < TB; ++j) {
                const uint2 x = ldg8(tp + 8 * j);
                tw[2 * j] = x.x; tw[2 * j + 1] = x.y;
            }
        }
    }
    uint32_t bits[2] = {0u, 0u};
    uint32_t s32 = 0, mx = 0, mn = ~0u;
    unsigned long long s64 = 0;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        uint32_t d[4];
        quad_deltas<NP, TB>(pw, tw, j, d);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const uint32_t b = (4 * j + e) & 31;
            bool in = d[e] - lo <= span;
            if constexpr (MODE == 2) in = (in != neg) && (((j < 8 ? m0 : m1) >> b) & 1u);
            if (in) {
                bits[j >> 3] |= 1u << b;
                if constexpr (kSum32) s32 += d[e]; else s64 += d[e];
                if constexpr (MODE >= 1) { mx = max(mx, d[e]); mn = min(mn, d[e]); }
            }
        }
    }
    return GroupOut{bits[0], bits[1], mx, mn, kSum32 ? s32 : s64};
}

// The general case out of line, so that the common loop keeps its registers.
template <int NP, int TB>
__device__ __noinline__ GroupOut group_general(const uint8_t* planes, const uint8_t* tail, uint64_t stride, uint32_t g0,
                                               uint32_t lo, uint32_t span, uint32_t m0, uint32_t m1, uint32_t neg) {
    return group_body<NP, TB, 2>(planes, tail, stride, g0, lo, span, m0, m1, neg != 0);
}

// A lane's partials over the current chunk (deltas are at most 32 bits wide).
struct Part32 {
    unsigned long long sum;
    uint32_t cnt, mx, mn;
};

__device__ __forceinline__ void add_group(Part32& part, const GroupOut& o) {
    part.cnt += __popc(o.w0) + __popc(o.w1);
    part.sum += o.sum;
    part.mx = o.mx > part.mx ? o.mx : part.mx;
    part.mn = o.mn < part.mn ? o.mn : part.mn;
}

// The warp's run of units [u, u_end) that belong to chunk k (its units are
// consecutive: rows r0, r0 + 2048, ...).  Returns the first unit after them.
template <int NP, int TB>
__device__ __forceinline__ uint32_t run_chunk(const QueryParams& q, const StreamChunk& k, uint32_t u, uint32_t u_end,
                                           uint32_t r0, bool store, bool want_mm, Part32& acc) {
    const uint32_t lane = threadIdx.x & 31;
    Part32 part = acc;
    const bool simple = !k.use_mask && !k.negate;
#pragma unroll 1
    for (uint32_t r = r0; u < u_end && r < k.n; ++u, r += kBuffUnitRows) {
        const uint32_t g0 = r + 64 * lane;
        if (g0 < k.n) {
            GroupOut o;
            const uint32_t left = k.n - g0;
            if (simple && left >= 64) {
                if (want_mm) o = group_body<NP, TB, 1>(k.planes, k.tail, k.stride, g0, k.lo, k.span, 0u, 0u, false);
                else o = group_body<NP, TB, 0>(k.planes, k.tail, k.stride, g0, k.lo, k.span, 0u, 0u, false);
            } else {
                uint32_t m0 = left >= 32 ? ~0u : ((1u << left) - 1u);
                uint32_t m1 = left >= 64 ? ~0u : (left > 32 ? ((1u << (left - 32)) - 1u) : 0u);
                if (k.use_mask) {
                    m0 &= mask_word(q.in_mask, k.row_off + g0, q.n_records);
                    m1 &= mask_word(q.in_mask, k.row_off + g0 + 32, q.n_records);
                }
                o = group_general<NP, TB>(k.planes, k.tail, k.stride, g0, k.lo, k.span, m0, m1, k.negate);
            }
            add_group(part, o);
            if (store) {
                const uint64_t row = k.row_off + g0;
                if (!q.out_atomic && left >= 64 && (row & 63) == 0) {
                    // one 8-byte store: a warp's 64 words go out as one coalesced 256-byte store
                    *reinterpret_cast<uint2*>(q.out_mask + (row >> 5)) = make_uint2(o.w0, o.w1);
                } else {
                    if (!q.out_atomic || o.w0) store_mask_word(q.out_mask, row, o.w0, q.out_atomic);
                    if (left > 32 && (!q.out_atomic || o.w1)) store_mask_word(q.out_mask, row + 32, o.w1, q.out_atomic);
                }
            }
        }
    }
    acc = part;
    return u;
}

// Any width (0..4 byte planes, 0..7 tail bits) decided at run time: chunks
// whose width differs from the one the kernel is built for.
__device__ __noinline__ GroupOut group_any(const uint8_t* planes, const uint8_t* tail, uint64_t stride, uint32_t np,
                                           uint32_t tb, uint32_t g0, uint32_t lo, uint32_t span, uint32_t m0,
                                           uint32_t m1, uint32_t neg) {
    uint32_t tw[15];
#pragma unroll
    for (int j = 0; j < 15; ++j) tw[j] = 0;
    const uint8_t* tp = tail + uint64_t(g0 / 64) * (8 * tb);
    for (uint32_t j = 0; j < tb; ++j) {
        const uint2 x = ldg8(tp + 8 * j);
        tw[2 * j] = x.x;
        tw[2 * j + 1] = x.y;
    }
    GroupOut o{0u, 0u, 0u, ~0u, 0ull};
    for (uint32_t i = 0; i < 64; ++i) {
        uint32_t v = 0;
        for (uint32_t p = 0; p < np; ++p) v = (v << 8) | (__ldg(planes + p * stride + g0 + i) ^ 0x80u);
        uint32_t d = v;
        if (tb) {
            const uint32_t pos = i * tb, wi = pos >> 5, sh = pos & 31;
            const uint32_t f = sh + tb <= 32 ? (tw[wi] >> sh) : __funnelshift_r(tw[wi], tw[wi + 1], sh);
            d = (v << tb) | (f & ((1u << tb) - 1u));
        }
        const bool in = ((d - lo <= span) != (neg != 0)) && (((i < 32 ? m0 : m1) >> (i & 31)) & 1u);
        if (in) {
            if (i < 32) o.w0 |= 1u << i; else o.w1 |= 1u << (i - 32);
            o.sum += d;
            o.mx = max(o.mx, d);
            o.mn = min(o.mn, d);
        }
    }
    return o;
}

// run_chunk for a chunk of another width: every group through group_any.
__device__ __forceinline__ uint32_t run_chunk_any(const QueryParams& q, const StreamChunk& k, uint32_t u, uint32_t u_end,
                                                  uint32_t r0, bool store, Part32& part) {
    const uint32_t lane = threadIdx.x & 31;
#pragma unroll 1
    for (uint32_t r = r0; u < u_end && r < k.n; ++u, r += kBuffUnitRows) {
        const uint32_t g0 = r + 64 * lane;
        if (g0 >= k.n) continue;
        const uint32_t left = k.n - g0;
        uint32_t m0 = left >= 32 ? ~0u : ((1u << left) - 1u);
        uint32_t m1 = left >= 64 ? ~0u : (left > 32 ? ((1u << (left - 32)) - 1u) : 0u);
        if (k.use_mask) {
            m0 &= mask_word(q.in_mask, k.row_off + g0, q.n_records);
            m1 &= mask_word(q.in_mask, k.row_off + g0 + 32, q.n_records);
        }
        const GroupOut o = group_any(k.planes, k.tail, k.stride, k.bits / 8, k.bits % 8, g0, k.lo, k.span, m0, m1,
                                     k.negate);
        add_group(part, o);
        if (store) {
            const uint64_t row = k.row_off + g0;
            if (!q.out_atomic || o.w0) store_mask_word(q.out_mask, row, o.w0, q.out_atomic);
            if (left > 32 && (!q.out_atomic || o.w1)) store_mask_word(q.out_mask, row + 32, o.w1, q.out_atomic);
        }
    }
    return u;
}

// The kernel built for chunks of NP byte planes and TB tail bits (NP = 0:
// tail-only chunks of 1..7 bits; the
// column's most common width); chunks of other widths take run_chunk_any.
// Narrow widths keep fewer registers and fit four CTAs per SM (64 registers:
// a few spilled words, measured faster than three CTAs at 80 registers).
template <int NP, int TB>
__global__ void __launch_bounds__(kStreamThreads, NP <= 2 ? 4 : 2)
buff_stream_kernel(QueryParams q, const BuffChunkInfo* info, const uint2* __restrict__ units, uint32_t unit_base,
                   uint32_t n_units, uint32_t upc, ScanTotals* T, QueryResult* res, uint32_t frac, uint32_t fold) {
    __shared__ WarpTot wtot[kStreamWarps];
    const bool exact = (fold & 2u) != 0;
    const bool totals_only = (fold & 4u) != 0;
    // totals-only queries alternate between two totals blocks (fold bit 3: the
    // upper one); this launch sets the other block at rest for the next query
    if (totals_only && blockIdx.x == 0 && threadIdx.x == 0)
        scan_totals_rest(reinterpret_cast<ScanTotals*>(reinterpret_cast<uint8_t*>(T) +
                                                      ((fold & 8u) ? -static_cast<ptrdiff_t>(kScanTotalsBytes)
                                                                   : static_cast<ptrdiff_t>(kScanTotalsBytes))));
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const bool store = (q.op == OP_FILTER || q.op == OP_FILTER_AGG) && q.out_mask;
    const bool want_mm = (q.op == OP_FILTER_AGG || q.op == OP_AGG) && (q.agg & (AGG_MIN | AGG_MAX));
    // the warp's query totals stay in shared memory (lane 0 updates them once per chunk)
    if (lane == 0) wtot[wid] = WarpTot{0, 0, 0, LLONG_MIN, LLONG_MAX, 0};
    StreamChunk k{};
    k.chunk = 0xffffffffu;
    Part32 part{0, 0, 0, ~0u};
    // Batches of units in column order: warp w's first batch is batch w, the
    // later ones come from a counter, so that warps on SMs that run ahead take
    // more of them and warps busy at the same time read neighbouring rows.
    const uint32_t n_warps = gridDim.x * kStreamWarps;
    uint32_t u = (blockIdx.x * kStreamWarps + wid) * kStreamBatch;
    for (bool first = true;; first = false) {
        if (!first) {
            if (lane == 0) u = n_warps * kStreamBatch + atomicAdd(&T->next, kStreamBatch);
            u = __shfl_sync(0xffffffffu, u, 0);
        }
        if (u >= n_units) break;
        const uint32_t ue = u + kStreamBatch < n_units ? u + kStreamBatch : n_units;
        while (u < ue) {
            // (chunk, first row) of unit u: by arithmetic when every chunk but
            // the last holds upc units, else from the unit table
            const uint2 un = upc ? make_uint2(unit_base / upc + u / upc, (u % upc) * kBuffUnitRows)
                                 : units[unit_base + u];
            if (un.x != k.chunk) {
                if (k.chunk != 0xffffffffu) {
                    Partial p64{part.sum, part.cnt, part.mx, part.cnt ? part.mn : ~0ull};
                    flush_partial(q, k.chunk, k.base, p64, wtot[wid], !exact);
                }
                k = stream_chunk(q, T, un.x, un.y == 0, exact);
                part = Part32{0, 0, 0, ~0u};
            }
            if (k.state == kTest) {
                if (k.bits == NP * 8 + TB) u = run_chunk<NP, TB>(q, k, u, ue, un.y, store, want_mm, part);
                else u = run_chunk_any(q, k, u, ue, un.y, store, part);
            } else {
                // unselected, unreadable or empty: zero words (an atomic output is pre-zeroed)
                for (uint32_t r = un.y; u < ue && r < k.n; ++u, r += kBuffUnitRows) {
                    const uint32_t g0 = r + 64 * lane;
                    if (store && !q.out_atomic && g0 < k.n) {
                        store_mask_word(q.out_mask, k.row_off + g0, 0u, false);
                        if (k.n - g0 > 32) store_mask_word(q.out_mask, k.row_off + g0 + 32, 0u, false);
                    }
                }
            }
        }
    }
    if (k.chunk != 0xffffffffu) {
        Partial p64{part.sum, part.cnt, part.mx, part.cnt ? part.mn : ~0ull};
        flush_partial(q, k.chunk, k.base, p64, wtot[wid], !exact);
    }
    cta_finish(q, info, T, res, frac, (fold & 1u) != 0, wtot, kStreamWarps, exact, totals_only);
}

// Launch of the kernel for widths NP * 8 + TB (instantiated by buff_stream_np{0,1,2,3,4}.cu).
template <int NP, int TB>
cudaError_t launch_stream_kernel(const QueryParams& q, const BuffChunkInfo* info, const uint2* units, uint32_t unit_base,
                                 uint32_t n_units, uint32_t upc, uint32_t grid, ScanTotals* T, QueryResult* res,
                                 uint32_t frac, uint32_t fold, cudaStream_t s) {
    buff_stream_kernel<NP, TB><<<grid, kStreamThreads, 0, s>>>(q, info, units, unit_base, n_units, upc, T, res, frac,
                                                               fold);
    count_launch();
    return cudaGetLastError();
}

}  // namespace
}  // namespace ebi
