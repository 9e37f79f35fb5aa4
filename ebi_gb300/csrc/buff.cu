// buff.cu -- BUFF (byte-sliced fixed point) chunks decoded and queried in place.
//
// Chunk layout (compressor/buff.rs:234-307): a 20-byte header (base as two
// u32, row count, bit width `bits`, fractional bits `frac`), then bits/8 byte
// planes, most significant first, each one byte per row and XOR 0x80
// (`flip`), then a tail plane of bits%8 bits per row packed LSB-first.  A row
// decodes to (base + delta) as f64 / 2^frac.
//
// Work split: one CTA of 256 threads per tile of 8192 rows; every thread owns
// 32 consecutive rows, reads their 32 bytes of each plane with three aligned
// 16-byte loads realigned in registers (the file sits in HBM unmodified, so
// planes start at arbitrary byte addresses), and forms the 32 deltas.  The
// range / equality predicates are compiled per chunk into the fixed-point
// domain exactly as the reference's in-situ filters decide them
// (buff/filter_cmp.rs:299-451, buff/filter_eq.rs:74-200), including their
// shortcuts.  Sums are exact u64 sums of deltas (buff/sum.rs:60-119); min
// and max are exact via the deltas (buff/min_max.rs).
#include "internal.h"
#include "tma.cuh"
#include "fold.cuh"
#include <climits>

namespace ebi {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

__constant__ uint32_t c_precision_map[13] = {0, 5, 8, 11, 15, 18, 21, 25, 28, 31, 35, 38, 50};

// into_fixed_representation_with_fractional_part_bits_length
// (compression_common/buff.rs:11-51), with the reference's release-build
// wrapping shift.
__device__ int64_t buff_fixed(double value, int32_t frac) {
    const uint64_t vb = static_cast<uint64_t>(__double_as_longlong(value));
    const int32_t exp = static_cast<int32_t>((vb >> 52) & 0x7ff) - 1023;
    if (exp < -frac) return 0;
    const uint64_t sign = vb & 0x8000000000000000ull;
    const int64_t s = 63 - static_cast<int64_t>(exp) - frac;
    uint64_t fixed = s >= 64 ? 0 : (((vb << 11) | 0x8000000000000000ull) >> (static_cast<uint64_t>(s) & 63));
    if (sign) fixed = ~(fixed - 1);
    return static_cast<int64_t>(fixed);
}

__device__ __forceinline__ uint32_t bit_length(uint64_t x) { return x ? 64u - __clzll(static_cast<long long>(x)) : 0u; }

enum : uint32_t { SIDE_ABSENT = 0, SIDE_ALL = 1, SIDE_NONE = 2, SIDE_CMP = 3 };

// Per-chunk context, filled by thread 0 into shared memory.
struct BuffCtx {
    const uint8_t* planes;
    const uint8_t* tail;
    int64_t base;
    uint64_t row_off;
    double scale;       // 2^frac
    double inv_scale;   // 2^-frac when exact (frac <= 1022), else 0
    uint32_t n, bits, frac, np, tb;
    uint32_t np_load, load_tail;  // planes / tail read when materializing
    uint32_t ok;                  // selected and readable
    uint32_t selected;
    // predicate compiled into the delta domain
    uint32_t lmode, rmode, lincl, rincl, emode;
    uint64_t lthr, rthr, etgt;
};

// Predicate compiled into the delta domain of one chunk, exactly as the
// reference's in-situ filters decide it.
struct BuffPred {
    uint32_t lmode, rmode, lincl, rincl, emode;
    uint64_t lthr, rthr, etgt;
};

__device__ void compile_pred(const ebi_predicate& pr, int64_t base, uint32_t bits, uint32_t frac, bool has_mask,
                             BuffPred& k) {
    k.lmode = k.rmode = SIDE_ABSENT;
    k.emode = SIDE_NONE;
    k.lincl = k.rincl = 0;
    k.lthr = k.rthr = k.etgt = 0;
    const uint32_t np = bits / 8;
    if (pr.kind == EBI_PRED_RANGE) {
        // left side: buff_simd256_cmp_filter::<true, INCL> (filter_cmp.rs:299-451)
        if (pr.start_kind != EBI_BOUND_NONE) {
            const bool incl = pr.start_kind == EBI_BOUND_INCLUSIVE;
            const int64_t fp = buff_fixed(pr.start, static_cast<int32_t>(frac));
            if (fp < base) k.lmode = SIDE_ALL;
            else if (bits == 0) k.lmode = (incl ? base >= fp : base > fp) ? SIDE_ALL : SIDE_NONE;
            else {
                const uint64_t dp = static_cast<uint64_t>(fp) - static_cast<uint64_t>(base);
                if (bits < bit_length(dp)) k.lmode = SIDE_NONE;
                else { k.lmode = SIDE_CMP; k.lthr = dp; k.lincl = incl; }
            }
        }
        // right side: buff_simd256_cmp_filter::<false, INCL>
        if (pr.end_kind != EBI_BOUND_NONE) {
            const bool incl = pr.end_kind == EBI_BOUND_INCLUSIVE;
            const int64_t fp = buff_fixed(pr.end, static_cast<int32_t>(frac));
            if (fp < base) k.rmode = SIDE_NONE;
            else if (bits == 0) k.rmode = (incl ? base <= fp : base < fp) ? SIDE_ALL : SIDE_NONE;
            else {
                const uint64_t dp = static_cast<uint64_t>(fp) - static_cast<uint64_t>(base);
                if (bits < bit_length(dp)) k.rmode = SIDE_ALL;
                else { k.rmode = SIDE_CMP; k.rthr = dp; k.rincl = incl; }
            }
        }
    } else {
        // buff_simd256_equal_filter (filter_eq.rs:74-200)
        const int64_t fp = buff_fixed(pr.value, static_cast<int32_t>(frac));
        if (fp < base) k.emode = SIDE_NONE;
        else if (bits == 0) k.emode = fp == base ? SIDE_ALL : SIDE_NONE;
        else {
            const uint64_t dp = static_cast<uint64_t>(fp) - static_cast<uint64_t>(base);
            // Byte planes compare (u8)(dp >> shift) and the tail compares dp's low
            // bits: together delta == dp mod 2^bits.  With neither byte planes
            // nor an input bitmask the tail is compared with `dp as u8` (:190-196).
            const uint64_t wmask = bits >= 64 ? ~0ull : ((1ull << bits) - 1);
            k.emode = SIDE_CMP;
            k.etgt = (np > 0 || has_mask) ? (dp & wmask) : (dp & 0xffull);
        }
    }
}

__device__ void buff_setup(const QueryParams& q, uint32_t c, bool has_mask, BuffCtx& k) {
    const ChunkDesc cd = q.chunks[c];
    ChunkAcc* acc = q.acc + c;
    k.ok = 0;
    k.n = cd.n_rows;
    k.row_off = cd.row_off;
    k.selected = has_mask ? acc->selected : static_cast<uint32_t>(q.chunk_id < 0 || static_cast<uint64_t>(q.chunk_id) == c);
    if (!k.selected) return;
    if (!has_mask && acc->selected == 0) acc->selected = 1;  // finalize folds selected chunks
    if (cd.flags & kChunkBadGeometry) { set_status(acc, EBI_E_IO); return; }
    if (cd.byte_len < 20) { set_status(acc, EBI_E_UNEXPECTED_END); return; }
    const uint8_t* p = q.file + cd.byte_off;
    k.base = static_cast<int64_t>(load_u64_unaligned(p));
    const uint32_t n = load_u32_unaligned(p + 8);
    k.bits = load_u32_unaligned(p + 12);
    k.frac = load_u32_unaligned(p + 16);
    if (k.bits > 64 || n != cd.n_rows) { set_status(acc, EBI_E_CORRUPT); return; }
    k.np = k.bits / 8;
    k.tb = k.bits % 8;
    const uint64_t need = 20 + uint64_t(k.np) * n + (uint64_t(n) * k.tb + 7) / 8;
    if (k.bits > 0 && need > cd.byte_len) { set_status(acc, EBI_E_UNEXPECTED_END); return; }
    k.planes = p + 20;
    k.tail = k.planes + uint64_t(k.np) * n;
    k.scale = k.frac <= 1023 ? __longlong_as_double(static_cast<long long>(uint64_t(1023 + k.frac) << 52))
                             : __longlong_as_double(0x7ff0000000000000ll);
    k.inv_scale = k.frac <= 1022 ? __longlong_as_double(static_cast<long long>(uint64_t(1023 - k.frac) << 52)) : 0.0;

    // controlled precision (buff/controlled_precision.rs:5-75)
    k.np_load = k.np;
    k.load_tail = k.tb > 0;
    if (q.precision >= 0 && k.bits >= 8) {
        const uint32_t cf = c_precision_map[q.precision];
        const uint32_t unnecessary = k.frac > cf ? k.frac - cf : 0;
        uint32_t rem = k.bits - 8;
        uint32_t loaded = 1;
        while (rem >= 8 && rem > unnecessary) { rem -= 8; ++loaded; }
        k.np_load = loaded;
        k.load_tail = rem > 0 && rem > unnecessary;
    }

    BuffPred bp;
    compile_pred(q.pred, k.base, k.bits, k.frac, has_mask, bp);
    k.lmode = bp.lmode; k.rmode = bp.rmode; k.lincl = bp.lincl; k.rincl = bp.rincl; k.emode = bp.emode;
    k.lthr = bp.lthr; k.rthr = bp.rthr; k.etgt = bp.etgt;
    k.ok = 1;
}

// The 32 deltas of chunk rows [r0, r0 + 32); r0 is a multiple of 32.
template <int TB, typename D>
__device__ __forceinline__ void load_deltas(const BuffCtx& k, uint32_t r0, uint32_t np_load, uint32_t np_shift,
                                            bool tail, D (&d)[32]) {
#pragma unroll
    for (int i = 0; i < 32; ++i) d[i] = 0;
    for (uint32_t p = 0; p < np_load; ++p) {
        uint32_t w[8];
        load32(k.planes + uint64_t(p) * k.n + r0, w);
#pragma unroll
        for (int i = 0; i < 32; ++i)
            d[i] = (d[i] << 8) | static_cast<D>(((w[i >> 2] >> (8 * (i & 3))) & 0xffu) ^ 0x80u);
    }
    for (uint32_t p = np_load; p < np_shift; ++p) {
#pragma unroll
        for (int i = 0; i < 32; ++i) d[i] = static_cast<D>(d[i] << 8);
    }
    if constexpr (TB > 0) {
        uint32_t w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (tail) load32(k.tail + uint64_t(r0 / 8) * TB, w);
#pragma unroll
        for (int i = 0; i < 32; ++i) {
            constexpr uint32_t m = (1u << TB) - 1u;
            const int pos = i * TB, wi = pos >> 5, sh = pos & 31;
            uint32_t f;
            if (sh + TB <= 32) f = w[wi] >> sh;
            else f = __funnelshift_r(w[wi], w[wi + 1], sh);
            d[i] = static_cast<D>((d[i] << TB) | static_cast<D>(f & m));
        }
    }
}

template <typename D>
__device__ __forceinline__ uint32_t cmp_word(const D (&d)[32], uint64_t thr, bool greater, bool incl) {
    uint32_t w = 0;
#pragma unroll
    for (int i = 0; i < 32; ++i) {
        const uint64_t x = d[i];
        const bool s = greater ? (x > thr || (incl && x == thr)) : (x < thr || (incl && x == thr));
        w |= static_cast<uint32_t>(s) << i;
    }
    return w;
}

template <typename D>
__device__ __forceinline__ uint32_t eq_word(const D (&d)[32], uint64_t t) {
    uint32_t w = 0;
#pragma unroll
    for (int i = 0; i < 32; ++i) w |= static_cast<uint32_t>(static_cast<uint64_t>(d[i]) == t) << i;
    return w;
}

struct BlockRed {
    unsigned long long sum[kWarps], cnt[kWarps], mx[kWarps], mn[kWarps];
};

template <int TB, typename D>
__device__ void buff_query_tile(const QueryParams& q, const BuffCtx& k, uint32_t c, uint32_t li, uint32_t tile_begin,
                                BlockRed& red) {
    const uint32_t r0 = tile_begin + threadIdx.x * 32;
    const bool has_mask = q.in_mask != nullptr;
    const bool want_agg = q.op == OP_FILTER_AGG || q.op == OP_AGG;
    const bool in_chunk = r0 < k.n;
    uint32_t sel = 0;
    unsigned long long s = 0, mx = 0, mn = ~0ull;
    if (in_chunk && k.ok) {
        const uint32_t left = k.n - r0;
        const uint32_t valid = left >= 32 ? ~0u : ((1u << left) - 1u);
        const uint32_t m = has_mask ? (mask_word(q.in_mask, k.row_off + r0, q.n_records) & valid) : valid;
        const bool need_deltas = k.lmode == SIDE_CMP || k.rmode == SIDE_CMP || k.emode == SIDE_CMP;
        D d[32];
        if (need_deltas || want_agg) load_deltas<TB, D>(k, r0, k.np, k.np, true, d);
        if (q.op == OP_AGG) {
            sel = m;
        } else if (q.pred.kind == EBI_PRED_RANGE) {
            const bool la = k.lmode == SIDE_ABSENT, ra = k.rmode == SIDE_ABSENT;
            uint32_t L = 0, R = 0;
            if (k.lmode == SIDE_ALL) L = valid;
            else if (k.lmode == SIDE_CMP) L = cmp_word<D>(d, k.lthr, true, k.lincl) & m;
            if (k.rmode == SIDE_ALL) R = valid;
            else if (k.rmode == SIDE_CMP) R = cmp_word<D>(d, k.rthr, false, k.rincl) & m;
            sel = (la && ra) ? m : la ? R : ra ? L : (L & R);
        } else {
            uint32_t e = 0;
            if (k.emode == SIDE_ALL) e = valid;
            else if (k.emode == SIDE_CMP) e = eq_word<D>(d, k.etgt) & m;
            sel = q.pred.kind == EBI_PRED_EQ ? e : (m & ~e);
        }
        if (want_agg) {
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                if ((sel >> i) & 1u) {
                    const unsigned long long x = static_cast<unsigned long long>(d[i]);
                    s += x;
                    mx = x > mx ? x : mx;
                    mn = x < mn ? x : mn;
                }
            }
        }
    }
    if ((q.op == OP_FILTER || q.op == OP_FILTER_AGG) && in_chunk && q.out_mask) {
        if (!q.out_atomic || sel) store_mask_word(q.out_mask, k.row_off + r0, sel, q.out_atomic);
    }
    // block reduction of count (and sum / max / min)
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned long long cnt = warp_sum<unsigned long long>(static_cast<unsigned long long>(__popc(sel)));
    unsigned long long ws = 0, wmx = 0, wmn = ~0ull;
    if (want_agg) { ws = warp_sum(s); wmx = warp_max_u64(mx); wmn = warp_min_u64(mn); }
    if (lane == 0) { red.cnt[wid] = cnt; red.sum[wid] = ws; red.mx[wid] = wmx; red.mn[wid] = wmn; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long tc = 0, ts = 0, tmx = 0, tmn = ~0ull;
        for (int w = 0; w < kWarps; ++w) {
            tc += red.cnt[w]; ts += red.sum[w];
            tmx = red.mx[w] > tmx ? red.mx[w] : tmx;
            tmn = red.mn[w] < tmn ? red.mn[w] : tmn;
        }
        if (q.tile_counts) q.tile_counts[li] = tc;
        if (want_agg && k.ok && tc) {
            ChunkAcc* a = q.acc + c;
            atomicAdd(&a->isum, ts);
            atomicAdd(&a->count, tc);
            atomicMax(&a->dmax, tmx);
            atomicMin(&a->dmin, tmn);
        }
    }
}

template <typename D>
__device__ void buff_query_dispatch(const QueryParams& q, const BuffCtx& k, uint32_t c, uint32_t li,
                                    uint32_t begin, BlockRed& red) {
    switch (k.ok ? k.tb : 0) {
        case 0: buff_query_tile<0, D>(q, k, c, li, begin, red); break;
        case 1: buff_query_tile<1, D>(q, k, c, li, begin, red); break;
        case 2: buff_query_tile<2, D>(q, k, c, li, begin, red); break;
        case 3: buff_query_tile<3, D>(q, k, c, li, begin, red); break;
        case 4: buff_query_tile<4, D>(q, k, c, li, begin, red); break;
        case 5: buff_query_tile<5, D>(q, k, c, li, begin, red); break;
        case 6: buff_query_tile<6, D>(q, k, c, li, begin, red); break;
        default: buff_query_tile<7, D>(q, k, c, li, begin, red); break;
    }
}

__global__ void __launch_bounds__(kThreads) buff_query_kernel(QueryParams q, uint32_t tile_base) {
    __shared__ BuffCtx k;
    __shared__ BlockRed red;
    const Tile t = q.tiles[tile_base + blockIdx.x];
    if (threadIdx.x == 0) buff_setup(q, t.chunk, q.in_mask != nullptr, k);
    __syncthreads();
    if (k.ok && k.bits > 32) buff_query_dispatch<unsigned long long>(q, k, t.chunk, blockIdx.x, t.begin, red);
    else buff_query_dispatch<uint32_t>(q, k, t.chunk, blockIdx.x, t.begin, red);
}

// Materialize pass 1: rows of the bitmask per tile.  A chunk is read (and its
// header errors reported) only when the bitmask selects some of its rows.
__global__ void __launch_bounds__(kThreads) buff_count_kernel(QueryParams q, uint32_t tile_base) {
    __shared__ unsigned long long wsum[kWarps];
    __shared__ BuffCtx k;
    const Tile t = q.tiles[tile_base + blockIdx.x];
    const ChunkDesc cd = q.chunks[t.chunk];
    const uint32_t r0 = t.begin + threadIdx.x * 32;
    uint32_t cnt = 0;
    if (r0 < cd.n_rows) {
        const uint32_t left = cd.n_rows - r0;
        const uint32_t valid = left >= 32 ? ~0u : ((1u << left) - 1u);
        cnt = __popc(mask_word(q.in_mask, cd.row_off + r0, q.n_records) & valid);
    }
    const unsigned long long w = warp_sum<unsigned long long>(cnt);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = w;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long tot = 0;
        for (int i = 0; i < kWarps; ++i) tot += wsum[i];
        q.tile_counts[blockIdx.x] = tot;
        if (tot) buff_setup(q, t.chunk, false, k);
    }
}

// Materialization: the decoded values of the selected rows, in row order.
template <int TB, typename D>
__device__ void buff_mat_tile(const QueryParams& q, const BuffCtx& k, uint32_t tile, uint32_t begin,
                              const unsigned long long* tile_offsets, unsigned long long base_row,
                              unsigned int* warp_tot) {
    const uint32_t r0 = begin + threadIdx.x * 32;
    const bool has_mask = q.in_mask != nullptr;
    uint32_t sel = 0;
    D d[32];
    if (r0 < k.n && k.ok) {
        const uint32_t left = k.n - r0;
        const uint32_t valid = left >= 32 ? ~0u : ((1u << left) - 1u);
        sel = has_mask ? (mask_word(q.in_mask, k.row_off + r0, q.n_records) & valid) : valid;
        if (sel) load_deltas<TB, D>(k, r0, k.np_load, k.np, k.load_tail, d);
    }
    // block-exclusive prefix of the per-thread counts
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned int cnt = __popc(sel);
    unsigned int inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) warp_tot[wid] = inc;
    __syncthreads();
    unsigned int before = 0;
    for (int w = 0; w < wid; ++w) before += warp_tot[w];
    unsigned long long pos;
    if (has_mask) pos = tile_offsets[blockIdx.x] + before + (inc - cnt);
    else pos = k.row_off + r0 - base_row;
    if (!sel) return;
    for (int i = 0; i < 32; ++i) {
        if (!((sel >> i) & 1u)) continue;
        const long long fixed = static_cast<long long>(static_cast<unsigned long long>(k.base) + static_cast<unsigned long long>(d[i]));
        const double v = k.inv_scale != 0.0 ? static_cast<double>(fixed) * k.inv_scale : static_cast<double>(fixed) / k.scale;
        if (pos < q.out_cap) q.out_vals[pos] = v;
        ++pos;
    }
}

template <typename D>
__device__ void buff_mat_dispatch(const QueryParams& q, const BuffCtx& k, uint32_t tile, uint32_t begin,
                                  const unsigned long long* offs, unsigned long long base_row, unsigned int* wt) {
    switch (k.ok ? k.tb : 0) {
        case 0: buff_mat_tile<0, D>(q, k, tile, begin, offs, base_row, wt); break;
        case 1: buff_mat_tile<1, D>(q, k, tile, begin, offs, base_row, wt); break;
        case 2: buff_mat_tile<2, D>(q, k, tile, begin, offs, base_row, wt); break;
        case 3: buff_mat_tile<3, D>(q, k, tile, begin, offs, base_row, wt); break;
        case 4: buff_mat_tile<4, D>(q, k, tile, begin, offs, base_row, wt); break;
        case 5: buff_mat_tile<5, D>(q, k, tile, begin, offs, base_row, wt); break;
        case 6: buff_mat_tile<6, D>(q, k, tile, begin, offs, base_row, wt); break;
        default: buff_mat_tile<7, D>(q, k, tile, begin, offs, base_row, wt); break;
    }
}

__global__ void __launch_bounds__(kThreads) buff_materialize_kernel(QueryParams q, uint32_t tile_base,
                                                                    const unsigned long long* tile_offsets,
                                                                    unsigned long long base_row) {
    __shared__ BuffCtx k;
    __shared__ unsigned int warp_tot[kWarps];
    const uint32_t tile = tile_base + blockIdx.x;
    const Tile t = q.tiles[tile];
    if (threadIdx.x == 0) {
        // with a bitmask, tiles without selected rows were counted as 0 and
        // their chunk may be unselected: only tiles that select rows read
        buff_setup(q, t.chunk, false, k);
        if (q.in_mask && tile_offsets[blockIdx.x + 1] == tile_offsets[blockIdx.x]) k.ok = 0;
    }
    __syncthreads();
    if (k.ok && k.bits > 32) buff_mat_dispatch<unsigned long long>(q, k, tile, t.begin, tile_offsets, base_row, warp_tot);
    else buff_mat_dispatch<uint32_t>(q, k, tile, t.begin, tile_offsets, base_row, warp_tot);
}


// ---------------------------------------------------------------------------
// Pipelined scan: a persistent CTA streams its contiguous range of tiles
// through a ring of shared-memory stages.  Warp 8 is the producer: for every
// tile it reads the chunk's header facts, compiles the predicate and issues
// one bulk copy (cp.async.bulk, the TMA unit) per byte plane plus one for
// the tail plane, all completing on the stage's `full` mbarrier.  Warps 0-7
// consume: each thread decodes 32 rows from shared memory, evaluates the
// predicate, writes its 32-bit bitmask word and accumulates exact per-chunk
// partials in registers, flushed with one atomic per warp when the chunk
// changes.  Consumers release a stage through its `empty` mbarrier.
// ---------------------------------------------------------------------------
constexpr int kScanConsumers = 256;
constexpr int kScanThreads = kScanConsumers + 32;

// The query folded, per chunk, into one unsigned range test on the delta:
//   sel = (negate ? ~cmp : cmp) & (use_mask ? bitmask : valid rows)
// with cmp = lo <= delta <= hi (all rows when `full`, none when `empty`).
// It reproduces the reference's in-situ decisions, including the shortcuts
// that return all rows without looking at the input bitmask.
struct RangeProg {
    uint64_t lo, hi;
    uint32_t empty, full, negate, use_mask;
};

__device__ RangeProg compile_prog(const QueryParams& q, const BuffPred& k, uint32_t bits, bool has_mask) {
    RangeProg g{0, ~0ull, 0, 0, 0, 0};
    const uint64_t dmax = bits >= 64 ? ~0ull : ((1ull << bits) - 1);
    if (q.op == OP_AGG) {  // no predicate: the rows of the bitmask (all rows without one)
        g.full = 1;
        g.use_mask = has_mask;
        return g;
    }
    if (q.pred.kind == EBI_PRED_RANGE) {
        const bool la = k.lmode == SIDE_ABSENT, ra = k.rmode == SIDE_ABSENT;
        if (k.lmode == SIDE_NONE || k.rmode == SIDE_NONE) g.empty = 1;
        if (k.lmode == SIDE_CMP) {
            if (!k.lincl && k.lthr >= dmax) g.empty = 1;
            else g.lo = k.lincl ? k.lthr : k.lthr + 1;
        }
        if (k.rmode == SIDE_CMP) {
            if (!k.rincl && k.rthr == 0) g.empty = 1;
            else g.hi = k.rincl ? k.rthr : k.rthr - 1;
        }
        if (!g.empty && g.lo > g.hi) g.empty = 1;
        g.use_mask = k.lmode == SIDE_CMP || k.rmode == SIDE_CMP || (la && ra);
    } else {
        if (k.emode == SIDE_NONE) g.empty = 1;
        else if (k.emode == SIDE_CMP) { g.lo = g.hi = k.etgt; g.use_mask = 1; }
        if (q.pred.kind == EBI_PRED_NE) { g.negate = 1; g.use_mask = 1; }
    }
    g.full = !g.empty && g.lo == 0 && g.hi >= dmax;
    g.use_mask = g.use_mask && has_mask;
    return g;
}

struct ScanMeta {
    int64_t base;       // the chunk's fixed-point base
    uint64_t row0;      // global row of the tile's first row
    uint32_t chunk, rows, ok, np, tb, bits;
    uint32_t mis[8];    // offset of the tile's first byte inside each plane slot
    uint32_t mis_tail;  // offset of the tile's first tail byte inside the tail slot
    BuffPred pred;
    RangeProg prog;
};

__device__ __forceinline__ uint4 lds16(const uint8_t* p) { return *reinterpret_cast<const uint4*>(p); }

// 32 bytes at an arbitrary shared-memory address as 8 little-endian words.
__device__ __forceinline__ void load32_smem(const uint8_t* p, uint32_t (&w)[8]) {
    const uint32_t a = smem_addr(p);
    const uint32_t s = a & 15;
    const uint8_t* q = p - s;
    uint4 x0 = lds16(q), x1 = lds16(q + 16), x2 = s ? lds16(q + 32) : make_uint4(0, 0, 0, 0);
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

struct Partial {
    unsigned long long sum, cnt, mx, mn;
};

// Running query totals of one warp (kept by lane 0).
struct WarpTot {
    unsigned long long sum_fixed, count;
    double abs_bound;
    long long max_fixed, min_fixed;
    unsigned int nonexact;
};

// Ends a warp's run over one chunk: per-chunk partials (for the chunk-ordered
// fallback fold) and the warp's exact query totals.
__device__ __forceinline__ void flush_partial(const QueryParams& q, uint32_t chunk, int64_t base, Partial& p,
                                              WarpTot& wt) {
    const unsigned long long s = warp_sum(p.sum), c = warp_sum(p.cnt), mx = warp_max_u64(p.mx), mn = warp_min_u64(p.mn);
    if ((threadIdx.x & 31) == 0 && c) {
        ChunkAcc* a = q.acc + chunk;
        atomicAdd(&a->isum, s);
        atomicAdd(&a->count, c);
        atomicMax(&a->dmax, mx);
        atomicMin(&a->dmin, mn);
        const __int128 piece = static_cast<__int128>(s) + static_cast<__int128>(base) * static_cast<__int128>(c);
        const __int128 ap = piece < 0 ? -piece : piece;
        wt.sum_fixed += static_cast<unsigned long long>(piece);
        if (ap >= (static_cast<__int128>(1) << 53)) wt.nonexact = 1;
        else wt.abs_bound += static_cast<double>(static_cast<long long>(ap));
        wt.count += c;
        const long long fmax = static_cast<long long>(static_cast<unsigned long long>(base) + mx);
        const long long fmin = static_cast<long long>(static_cast<unsigned long long>(base) + mn);
        wt.max_fixed = fmax > wt.max_fixed ? fmax : wt.max_fixed;
        wt.min_fixed = fmin < wt.min_fixed ? fmin : wt.min_fixed;
    }
    p.sum = 0; p.cnt = 0; p.mx = 0; p.mn = ~0ull;
}

template <int TB, typename D>
__device__ __forceinline__ void scan_rows(const QueryParams& q, const ScanMeta& m, const uint8_t* stage,
                                          const StageLayout& L, Partial& part) {
    const uint32_t t = threadIdx.x;
    const uint32_t lr = 32 * t;
    const bool has_mask = q.in_mask != nullptr;
    const bool want_agg = q.op == OP_FILTER_AGG || q.op == OP_AGG;
    const bool in_tile = lr < m.rows;
    uint32_t sel = 0;
    if (in_tile && m.ok) {
        const uint32_t left = m.rows - lr;
        const uint32_t valid = left >= 32 ? ~0u : ((1u << left) - 1u);
        const uint32_t mw = has_mask ? (mask_word(q.in_mask, m.row0 + lr, q.n_records) & valid) : valid;
        D d[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) d[i] = 0;
        for (uint32_t p = 0; p < m.np; ++p) {
            uint32_t w[8];
            load32_smem(stage + p * L.plane_stride + m.mis[p] + lr, w);
#pragma unroll
            for (int j = 0; j < 8; ++j) w[j] ^= 0x80808080u;
#pragma unroll
            for (int i = 0; i < 32; ++i) d[i] = (d[i] << 8) | static_cast<D>((w[i >> 2] >> (8 * (i & 3))) & 0xffu);
        }
        if constexpr (TB > 0) {
            uint32_t w[8];
            load32_smem(stage + L.np_max * L.plane_stride + m.mis_tail + 4 * TB * t, w);
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                constexpr uint32_t msk = (1u << TB) - 1u;
                const int pos = i * TB, wi = pos >> 5, sh = pos & 31;
                const uint32_t f = (sh + TB <= 32) ? (w[wi] >> sh) : __funnelshift_r(w[wi], w[wi + 1], sh);
                d[i] = static_cast<D>((d[i] << TB) | static_cast<D>(f & msk));
            }
        }
        const BuffPred& k = m.pred;
        if (q.op == OP_AGG) {
            sel = mw;
        } else if (q.pred.kind == EBI_PRED_RANGE) {
            const bool la = k.lmode == SIDE_ABSENT, ra = k.rmode == SIDE_ABSENT;
            uint32_t Lw = 0, Rw = 0;
            if (k.lmode == SIDE_ALL) Lw = valid;
            else if (k.lmode == SIDE_CMP) Lw = cmp_word<D>(d, k.lthr, true, k.lincl) & mw;
            if (k.rmode == SIDE_ALL) Rw = valid;
            else if (k.rmode == SIDE_CMP) Rw = cmp_word<D>(d, k.rthr, false, k.rincl) & mw;
            sel = (la && ra) ? mw : la ? Rw : ra ? Lw : (Lw & Rw);
        } else {
            uint32_t e = 0;
            if (k.emode == SIDE_ALL) e = valid;
            else if (k.emode == SIDE_CMP) e = eq_word<D>(d, k.etgt) & mw;
            sel = q.pred.kind == EBI_PRED_EQ ? e : (mw & ~e);
        }
        if (want_agg && sel) {
            unsigned long long s64 = 0;
            D mx = 0, mn = static_cast<D>(~D(0));
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                const bool on = (sel >> i) & 1u;
                s64 += on ? static_cast<unsigned long long>(d[i]) : 0ull;
                mx = (on && d[i] > mx) ? d[i] : mx;
                mn = (on && d[i] < mn) ? d[i] : mn;
            }
            part.sum += s64;
            part.cnt += __popc(sel);
            part.mx = static_cast<unsigned long long>(mx) > part.mx ? static_cast<unsigned long long>(mx) : part.mx;
            part.mn = static_cast<unsigned long long>(mn) < part.mn ? static_cast<unsigned long long>(mn) : part.mn;
        }
    }
    if ((q.op == OP_FILTER || q.op == OP_FILTER_AGG) && in_tile && q.out_mask) {
        if (!q.out_atomic || sel) store_mask_word(q.out_mask, m.row0 + lr, sel, q.out_atomic);
    }
}


// Fast path for chunks of 8 to 32 bits.  Each lane handles quads of 4
// consecutive rows; quad j * 256 + t of the tile belongs to thread t, so the
// 32 lanes of a warp read consecutive words of every plane (no shared-memory
// bank conflicts).  Deltas are u32, assembled with byte permutes; the
// predicate is one unsigned range test per row; the loop is straight-line.
template <int NP, int TB, bool SUM, bool MINMAX, bool FAST>
__device__ __forceinline__ void scan_quads(const QueryParams& q, const ScanMeta& m, const uint8_t* stage,
                                           const StageLayout& L, Partial& part) {
    static_assert(NP >= 1 && NP <= 4 && NP * 8 + TB <= 32, "u32 deltas");
    constexpr bool kSum32 = NP * 8 + TB <= 27;  // 32 rows of deltas fit a u32 sum
    const uint32_t t = threadIdx.x, lane = t & 31;
    const bool has_mask = q.in_mask != nullptr;
    const bool store = (q.op == OP_FILTER || q.op == OP_FILTER_AGG) && q.out_mask;
    const RangeProg& g = m.prog;
    const uint32_t lo = static_cast<uint32_t>(g.lo), span = static_cast<uint32_t>(g.hi - g.lo);
    const bool test = !(g.empty || g.full);
    const uint32_t fixed_cw = g.full ? 0xfu : 0u;
    const uint32_t neg = g.negate ? 0xfu : 0u;
    const bool use_mask = g.use_mask && has_mask;
    const uint32_t* slot[NP];
    uint32_t rsh[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        slot[p] = reinterpret_cast<const uint32_t*>(stage + p * L.plane_stride + (m.mis[p] & ~3u));
        rsh[p] = 8 * (m.mis[p] & 3);
    }
    const uint32_t* tslot = reinterpret_cast<const uint32_t*>(stage + L.np_max * L.plane_stride);
    const uint32_t tbit0 = 8 * m.mis_tail;
    uint32_t cnt = 0, mx = 0, mn = ~0u;
    uint32_t s32 = 0;
    unsigned long long s64 = 0;
#pragma unroll 2
    for (int j = 0; j < 8; ++j) {
        const uint32_t qd = j * kScanConsumers + t;  // quad index in the tile
        const uint32_t r = 4 * qd;                   // first row of the quad in the tile
        uint32_t nib = 0;
        if (FAST || r < m.rows) {
            const uint32_t left = m.rows - r;
            const uint32_t valid = FAST ? 0xfu : (left >= 4 ? 0xfu : ((1u << left) - 1u));
            uint32_t w[NP];
#pragma unroll
            for (int p = 0; p < NP; ++p) w[p] = __funnelshift_r(slot[p][qd], slot[p][qd + 1], rsh[p]) ^ 0x80808080u;
            uint32_t v[4];
            if constexpr (NP == 1) {
#pragma unroll
                for (int k = 0; k < 4; ++k) v[k] = __byte_perm(w[0], 0u, 0x4440u | k);
            } else if constexpr (NP == 2) {
                const uint32_t P = __byte_perm(w[1], w[0], 0x5140u), Q = __byte_perm(w[1], w[0], 0x7362u);
                v[0] = P & 0xffffu; v[1] = P >> 16; v[2] = Q & 0xffffu; v[3] = Q >> 16;
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    uint32_t x = 0;
#pragma unroll
                    for (int p = 0; p < NP; ++p) x = (x << 8) | ((w[p] >> (8 * k)) & 0xffu);
                    v[k] = x;
                }
            }
            uint32_t d[4];
            if constexpr (TB > 0) {
                const uint32_t b = tbit0 + 4 * TB * qd;
                const uint32_t f = __funnelshift_r(tslot[b >> 5], tslot[(b >> 5) + 1], b & 31);
#pragma unroll
                for (int k = 0; k < 4; ++k) d[k] = (v[k] << TB) | ((f >> (TB * k)) & ((1u << TB) - 1u));
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) d[k] = v[k];
            }
            if constexpr (FAST) {
                // full tile, no input bitmask, predicate not negated: the range
                // test itself drives the bitmask bit and the accumulators
                if (test) {
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const bool in = d[k] - lo <= span;
                        nib |= static_cast<uint32_t>(in) << k;
                        if constexpr (SUM) { if (in) { if constexpr (kSum32) s32 += d[k]; else s64 += d[k]; } }
                        if constexpr (MINMAX) { if (in) { mx = max(mx, d[k]); mn = min(mn, d[k]); } }
                    }
                } else if (g.full) {
                    nib = 0xfu;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        if constexpr (SUM) { if constexpr (kSum32) s32 += d[k]; else s64 += d[k]; }
                        if constexpr (MINMAX) { mx = max(mx, d[k]); mn = min(mn, d[k]); }
                    }
                }
                cnt += __popc(nib);
            } else {
            uint32_t cw = fixed_cw;
            if (test) {
#pragma unroll
                for (int k = 0; k < 4; ++k) cw |= static_cast<uint32_t>(d[k] - lo <= span) << k;
            }
            uint32_t base_set = valid;
            if (use_mask) base_set &= mask_word(q.in_mask, m.row0 + r, q.n_records);
            nib = (cw ^ neg) & base_set;
            cnt += __popc(nib);
            if constexpr (SUM) {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const uint32_t x = ((nib >> k) & 1u) ? d[k] : 0u;
                    if constexpr (kSum32) s32 += x; else s64 += x;
                }
            }
            if constexpr (MINMAX) {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const bool on = (nib >> k) & 1u;
                    mx = max(mx, on ? d[k] : 0u);
                    mn = min(mn, on ? d[k] : ~0u);
                }
            }
            }
        }
        if (store) {
            // 8 lanes hold the 32 rows of one bitmask word: gather their nibbles
            uint32_t x = nib << (4 * (lane & 7));
            x |= __shfl_xor_sync(0xffffffffu, x, 1);
            x |= __shfl_xor_sync(0xffffffffu, x, 2);
            x |= __shfl_xor_sync(0xffffffffu, x, 4);
            const uint32_t r0 = 4 * (j * kScanConsumers + (t & ~7u));  // first row of the word in the tile
            if ((lane & 7) == 0 && r0 < m.rows && (!q.out_atomic || x))
                store_mask_word(q.out_mask, m.row0 + r0, x, q.out_atomic);
        }
    }
    if (q.op == OP_FILTER_AGG || q.op == OP_AGG) {
        part.cnt += cnt;
        part.sum += kSum32 ? s32 : s64;
        part.mx = mx > part.mx ? mx : part.mx;
        part.mn = mn < part.mn ? mn : part.mn;
    }
}

template <int NP, int TB>
__device__ __forceinline__ void scan_quads_agg(const QueryParams& q, const ScanMeta& m, const uint8_t* st,
                                               const StageLayout& L, Partial& part) {
    const bool agg = q.op == OP_FILTER_AGG || q.op == OP_AGG;
    const bool sum = agg && (q.agg & AGG_SUM), mm = agg && (q.agg & (AGG_MIN | AGG_MAX));
    const bool fast = m.rows == kBuffTileRows && !(m.prog.use_mask && q.in_mask) && !m.prog.negate;
    if (fast) {
        if (mm) scan_quads<NP, TB, true, true, true>(q, m, st, L, part);
        else if (sum) scan_quads<NP, TB, true, false, true>(q, m, st, L, part);
        else scan_quads<NP, TB, false, false, true>(q, m, st, L, part);
    } else {
        if (mm) scan_quads<NP, TB, true, true, false>(q, m, st, L, part);
        else if (sum) scan_quads<NP, TB, true, false, false>(q, m, st, L, part);
        else scan_quads<NP, TB, false, false, false>(q, m, st, L, part);
    }
}

#define EBI_Q(NP, TB) case NP * 8 + TB: scan_quads_agg<NP, TB>(q, m, st, L, part); return true;
// Chunks of 8..32 bits; false for the others (they take the generic path).
__device__ bool scan_fast_dispatch(const QueryParams& q, const ScanMeta& m, const uint8_t* st, const StageLayout& L,
                                   Partial& part) {
    switch (m.bits) {
        EBI_Q(1, 0) EBI_Q(1, 1) EBI_Q(1, 2) EBI_Q(1, 3) EBI_Q(1, 4) EBI_Q(1, 5) EBI_Q(1, 6) EBI_Q(1, 7)
        EBI_Q(2, 0) EBI_Q(2, 1) EBI_Q(2, 2) EBI_Q(2, 3) EBI_Q(2, 4) EBI_Q(2, 5) EBI_Q(2, 6) EBI_Q(2, 7)
        EBI_Q(3, 0) EBI_Q(3, 1) EBI_Q(3, 2) EBI_Q(3, 3) EBI_Q(3, 4) EBI_Q(3, 5) EBI_Q(3, 6) EBI_Q(3, 7)
        EBI_Q(4, 0)
        default: return false;
    }
}
#undef EBI_Q

template <typename D>
__device__ __forceinline__ void scan_dispatch(const QueryParams& q, const ScanMeta& m, const uint8_t* stage,
                                              const StageLayout& L, Partial& part) {
    switch (m.ok ? m.tb : 0) {
        case 0: scan_rows<0, D>(q, m, stage, L, part); break;
        case 1: scan_rows<1, D>(q, m, stage, L, part); break;
        case 2: scan_rows<2, D>(q, m, stage, L, part); break;
        case 3: scan_rows<3, D>(q, m, stage, L, part); break;
        case 4: scan_rows<4, D>(q, m, stage, L, part); break;
        case 5: scan_rows<5, D>(q, m, stage, L, part); break;
        case 6: scan_rows<6, D>(q, m, stage, L, part); break;
        default: scan_rows<7, D>(q, m, stage, L, part); break;
    }
}

__device__ __forceinline__ void chunk_error(const QueryParams& q, ScanTotals* T, uint32_t c, uint32_t code) {
    set_status(q.acc + c, code);
    atomicMin(&T->bad_chunk, c);
}

// The last CTA's fold of the query totals (chunk-ordered fallback when the
// exact integer total does not apply).
__device__ void scan_finalize(const QueryParams& q, const BuffChunkInfo* info, ScanTotals* T, QueryResult* res,
                              uint32_t frac, bool fast_ok) {
    __shared__ QueryResult r;
    if (threadIdx.x == 0) {
        const ScanTotals t = *T;
        const double inf = __longlong_as_double(0x7ff0000000000000ll);
        r.status = 0;
        r.bad_chunk = t.bad_chunk;
        if (t.bad_chunk != 0xffffffffu) r.status = q.acc[t.bad_chunk].status;
        r.count = t.count;
        r.sum = 0.0; r.min = inf; r.max = -inf;
        if (fast_ok && !t.nonexact && t.abs_bound < 4503599627370496.0 /* 2^52 */) {
            // Every chunk sum and every prefix of the chunk-ordered fold is an
            // exact multiple of 2^-frac below 2^53 of them: the reference's
            // sequential f64 fold is exact and equals the exact total.
            if (t.count) {
                r.sum = fold_scale(static_cast<long long>(t.sum_fixed), frac);
                r.max = fold_scale(t.max_fixed, frac);
                r.min = fold_scale(t.min_fixed, frac);
            }
        } else {
            fold_buff_chunks(q, r);
        }
        *res = r;
        T->sum_fixed = 0; T->abs_bound = 0.0; T->count = 0;
        T->max_fixed = LLONG_MIN; T->min_fixed = LLONG_MAX;
        T->done = 0; T->bad_chunk = 0xffffffffu; T->nonexact = 0;
    }
    __syncthreads();
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    for (uint32_t c = threadIdx.x; c < q.n_chunks; c += blockDim.x) {
        ChunkAcc a = {};
        a.dmin = ~0ull;
        a.fmin = inf;
        a.fmax = -inf;
        q.acc[c] = a;
    }
}

__global__ void __launch_bounds__(kScanThreads, 2)
buff_scan_kernel(QueryParams q, const BuffChunkInfo* info, uint32_t tile_base, uint32_t n_tiles, StageLayout L,
                 ScanTotals* T, QueryResult* res, uint32_t frac, uint32_t fast_ok) {
    extern __shared__ __align__(128) uint8_t smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem);
    uint64_t* empty = full + L.stages;
    ScanMeta* meta = reinterpret_cast<ScanMeta*>(smem + 128);
    uint8_t* stages = smem + L.data_offset;
    // contiguous tile range of this CTA
    const uint32_t t_first = static_cast<uint32_t>((uint64_t(n_tiles) * blockIdx.x) / gridDim.x);
    const uint32_t t_end = static_cast<uint32_t>((uint64_t(n_tiles) * (blockIdx.x + 1)) / gridDim.x);
    const uint32_t count = t_end - t_first;
    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < L.stages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kScanConsumers / 32);
        }
        fence_mbar_init();
    }
    __syncthreads();
    const bool has_mask = q.in_mask != nullptr;

    if (threadIdx.x == kScanConsumers) {
        // ---- producer: one lane of warp 8 issues; the other lanes wait at the epilogue ----
        for (uint32_t i = 0; i < count; ++i) {
            const uint32_t s = i % L.stages, k = i / L.stages;
            if (k > 0 && !mbar_wait(&empty[s], (k - 1) & 1)) {
                chunk_error(q, T, 0, EBI_E_CUDA);
                break;  // consumers stopped; nothing of this stage is in flight
            }
            const Tile tl = q.tiles[tile_base + t_first + i];
            const uint32_t c = tl.chunk;
            const ChunkDesc cd = q.chunks[c];
            const BuffChunkInfo ci = info[c];
            ScanMeta& m = meta[s];
            const bool selected = has_mask ? q.acc[c].selected != 0
                                           : (q.chunk_id < 0 || static_cast<uint64_t>(q.chunk_id) == c);
            if (selected && tl.begin == 0) {
                if (!has_mask) q.acc[c].selected = 1;
                if (ci.status) chunk_error(q, T, c, ci.status);
            }
            m.chunk = c;
            m.base = ci.base;
            m.row0 = cd.row_off + tl.begin;
            m.rows = min(kBuffTileRows, cd.n_rows - tl.begin);
            m.ok = selected && ci.status == 0;
            uint32_t bytes = 0;
            const uint8_t* file = q.file;
            uint8_t* st = stages + size_t(s) * L.stage_bytes;
            if (m.ok) {
                m.np = ci.bits / 8;
                m.tb = ci.bits % 8;
                m.bits = ci.bits;
                compile_pred(q.pred, ci.base, ci.bits, ci.frac, has_mask, m.pred);
                m.prog = compile_prog(q, m.pred, ci.bits, has_mask);
                for (uint32_t p = 0; p < m.np; ++p) {
                    const uintptr_t src = reinterpret_cast<uintptr_t>(file + ci.planes + uint64_t(p) * ci.n + tl.begin);
                    const uintptr_t a = src & ~uintptr_t(15);
                    m.mis[p] = static_cast<uint32_t>(src - a);
                    bytes += static_cast<uint32_t>(((src + m.rows + 15) & ~uintptr_t(15)) - a);
                }
                if (m.tb) {
                    const uintptr_t src = reinterpret_cast<uintptr_t>(file + ci.tail + uint64_t(tl.begin / 8) * m.tb);
                    const uintptr_t a = src & ~uintptr_t(15);
                    m.mis_tail = static_cast<uint32_t>(src - a);
                    bytes += static_cast<uint32_t>(((src + (uint64_t(m.rows) * m.tb + 7) / 8 + 15) & ~uintptr_t(15)) - a);
                }
            } else {
                m.np = 0;
                m.tb = 0;
            }
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&full[s], bytes);
            if (m.ok) {
                for (uint32_t p = 0; p < m.np; ++p) {
                    const uintptr_t src = reinterpret_cast<uintptr_t>(file + ci.planes + uint64_t(p) * ci.n + tl.begin);
                    const uintptr_t a = src & ~uintptr_t(15);
                    const uint32_t len = static_cast<uint32_t>(((src + m.rows + 15) & ~uintptr_t(15)) - a);
                    bulk_g2s(st + p * L.plane_stride, reinterpret_cast<const void*>(a), len, &full[s]);
                }
                if (m.tb) {
                    const uintptr_t src = reinterpret_cast<uintptr_t>(file + ci.tail + uint64_t(tl.begin / 8) * m.tb);
                    const uintptr_t a = src & ~uintptr_t(15);
                    const uint32_t len =
                        static_cast<uint32_t>(((src + (uint64_t(m.rows) * m.tb + 7) / 8 + 15) & ~uintptr_t(15)) - a);
                    bulk_g2s(st + L.np_max * L.plane_stride, reinterpret_cast<const void*>(a), len, &full[s]);
                }
            }
        }
        // drain: the last stages' copies complete before this lane leaves
        for (uint32_t i = count > L.stages ? count - L.stages : 0; i < count; ++i)
            if (!mbar_wait(&full[i % L.stages], (i / L.stages) & 1)) { chunk_error(q, T, 0, EBI_E_CUDA); break; }
    }
    __shared__ WarpTot wtot[kScanConsumers / 32];
    if (threadIdx.x < kScanConsumers) {
    // ---- consumer warps ----
    Partial part{0, 0, 0, ~0ull};
    WarpTot wt{0, 0, 0.0, LLONG_MIN, LLONG_MAX, 0};
    uint32_t cur = 0xffffffffu;
    int64_t cur_base = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const uint32_t s = i % L.stages, k = i / L.stages;
        if (!mbar_wait(&full[s], k & 1)) {
            chunk_error(q, T, 0, EBI_E_CUDA);
            break;
        }
        const ScanMeta& m = meta[s];
        if (m.chunk != cur) {
            if (cur != 0xffffffffu) flush_partial(q, cur, cur_base, part, wt);
            cur = m.chunk;
            cur_base = m.base;
        }
        const uint8_t* st = stages + size_t(s) * L.stage_bytes;
        if (!m.ok) scan_dispatch<uint32_t>(q, m, st, L, part);  // writes zero words only
        else if (m.bits > 32) scan_dispatch<unsigned long long>(q, m, st, L, part);
        else if (!scan_fast_dispatch(q, m, st, L, part)) scan_dispatch<uint32_t>(q, m, st, L, part);
        __syncwarp();
        if ((threadIdx.x & 31) == 0) mbar_arrive(&empty[s]);
    }
    if (cur != 0xffffffffu) flush_partial(q, cur, cur_base, part, wt);
    if ((threadIdx.x & 31) == 0) wtot[threadIdx.x >> 5] = wt;
    }
    // ---- CTA totals, then the last CTA folds the query ----
    __syncthreads();
    __shared__ unsigned int s_last;
    if (threadIdx.x == 0) {
        WarpTot c{0, 0, 0.0, LLONG_MIN, LLONG_MAX, 0};
        for (int w = 0; w < kScanConsumers / 32; ++w) {
            c.sum_fixed += wtot[w].sum_fixed;
            c.count += wtot[w].count;
            c.abs_bound += wtot[w].abs_bound;
            c.max_fixed = wtot[w].max_fixed > c.max_fixed ? wtot[w].max_fixed : c.max_fixed;
            c.min_fixed = wtot[w].min_fixed < c.min_fixed ? wtot[w].min_fixed : c.min_fixed;
            c.nonexact |= wtot[w].nonexact;
        }
        if (c.count) {
            atomicAdd(&T->sum_fixed, c.sum_fixed);
            atomicAdd(&T->count, c.count);
            atomicAdd(&T->abs_bound, c.abs_bound);
            atomicMax(&T->max_fixed, c.max_fixed);
            atomicMin(&T->min_fixed, c.min_fixed);
            if (c.nonexact) atomicOr(&T->nonexact, 1u);
        }
        __threadfence();
        s_last = atomicAdd(&T->done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    scan_finalize(q, info, T, res, frac, fast_ok != 0);
}

}  // namespace

TileMap buff_tiles(const std::vector<ChunkDesc>& chunks) {
    TileMap m;
    m.first_tile.reserve(chunks.size() + 1);
    for (uint32_t c = 0; c < chunks.size(); ++c) {
        m.first_tile.push_back(static_cast<uint32_t>(m.tiles.size()));
        const uint32_t n = chunks[c].n_rows;
        uint32_t b = 0;
        do { m.tiles.push_back(Tile{c, b}); b += kBuffTileRows; } while (b < n);
    }
    m.first_tile.push_back(static_cast<uint32_t>(m.tiles.size()));
    return m;
}

cudaError_t launch_buff_query(const QueryParams& q, uint32_t tile_begin, uint32_t n_tiles, cudaStream_t s) {
    if (n_tiles == 0) return cudaSuccess;
    buff_query_kernel<<<n_tiles, kThreads, 0, s>>>(q, tile_begin);
    count_launch();
    return cudaGetLastError();
}

StageLayout buff_stage_layout(uint32_t np_max, uint32_t tb_max, uint32_t* ctas_per_sm) {
    StageLayout L{};
    L.plane_stride = kBuffTileRows + 32;
    L.np_max = np_max;
    L.tail_stride = ((kBuffTileRows / 8) * tb_max + 48 + 15) & ~15u;
    L.stage_bytes = (np_max * L.plane_stride + L.tail_stride + 127) & ~127u;
    const uint32_t meta = 128 + 8 * static_cast<uint32_t>(sizeof(ScanMeta));  // barriers + up to 8 stages
    L.data_offset = (meta + 127) & ~127u;
    const uint32_t budget2 = 110 * 1024, budget1 = 220 * 1024;
    uint32_t st = (budget2 - L.data_offset) / L.stage_bytes;
    *ctas_per_sm = 2;
    if (st < 3) {
        st = (budget1 - L.data_offset) / L.stage_bytes;
        *ctas_per_sm = 1;
    }
    L.stages = st > 8 ? 8 : (st < 2 ? 2 : st);
    if (L.stages > 4 && *ctas_per_sm == 2) L.stages = 4;
    return L;
}

cudaError_t launch_buff_scan(const QueryParams& q, const BuffChunkInfo* info, uint32_t tile_begin, uint32_t n_tiles,
                            const StageLayout& L, uint32_t grid, ScanTotals* T, QueryResult* res, uint32_t frac,
                            bool fast_ok, cudaStream_t s) {
    if (n_tiles == 0) return cudaSuccess;
    const size_t smem = L.data_offset + size_t(L.stages) * L.stage_bytes;
    static size_t configured = 0;
    if (smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(buff_scan_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    buff_scan_kernel<<<grid < n_tiles ? grid : n_tiles, kScanThreads, smem, s>>>(q, info, tile_begin, n_tiles, L, T,
                                                                               res, frac, fast_ok ? 1u : 0u);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_buff_count(const QueryParams& q, uint32_t tile_begin, uint32_t n_tiles, cudaStream_t s) {
    if (n_tiles == 0) return cudaSuccess;
    buff_count_kernel<<<n_tiles, kThreads, 0, s>>>(q, tile_begin);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_buff_materialize(const QueryParams& q, uint32_t tile_begin, uint32_t n_tiles,
                                    const unsigned long long* tile_offsets, uint64_t base_row, cudaStream_t s) {
    if (n_tiles == 0) return cudaSuccess;
    buff_materialize_kernel<<<n_tiles, kThreads, 0, s>>>(q, tile_begin, tile_offsets, base_row);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ebi
