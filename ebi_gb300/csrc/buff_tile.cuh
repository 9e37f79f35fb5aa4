// buff_tile.cuh -- the per-tile BUFF query (one CTA of 256 threads, 8,192
// rows): chunk setup and the fixed-point filter / sum / min / max of a tile,
// shared by buff.cu's kernels and the batched launch (batch.cu).
#pragma once

#include "buff_common.cuh"
#include "fold.cuh"

namespace ebi {
namespace {
using namespace buff;

constexpr int kTileThreads = 256;
constexpr int kTileWarps = kTileThreads / 32;

__constant__ uint32_t c_precision_map[13] = {0, 5, 8, 11, 15, 18, 21, 25, 28, 31, 35, 38, 50};

// Per-chunk context, filled by thread 0 into shared memory.
struct BuffCtx {
    const uint8_t* planes;
    const uint8_t* tail;
    uint64_t stride;    // bytes from one byte plane to the next
    int64_t base;
    uint64_t row_off;
    double scale;       // 2^frac
    double inv_scale;   // 2^-frac when exact (frac <= 1022), else 0
    uint32_t n, bits, frac, np, tb;
    uint32_t np_load, load_tail;  // planes / tail read when materializing
    uint32_t ok;                  // selected and readable
    uint32_t fits32;              // every row's fixed value fits an int32 and frac <= 1022
    uint32_t selected;
    // predicate compiled into the delta domain
    uint32_t lmode, rmode, lincl, rincl, emode;
    uint64_t lthr, rthr, etgt;
};

// mark = false: the chunk's accumulator is left untouched (a pass whose
// chunks cannot raise and that folds nothing).
__device__ void buff_setup(const QueryParams& q, uint32_t c, bool has_mask, BuffCtx& k, bool mark = true) {
    const ChunkDesc cd = q.chunks[c];
    ChunkAcc* acc = q.acc + c;
    k.ok = 0;
    k.n = cd.n_rows;
    k.row_off = cd.row_off;
    k.selected = has_mask ? acc->selected : static_cast<uint32_t>(q.chunk_id < 0 || static_cast<uint64_t>(q.chunk_id) == c);
    if (!k.selected) return;
    if (mark && !has_mask && acc->selected == 0) acc->selected = 1;  // finalize folds selected chunks
    // the header facts were read and checked at open (the chunk's status)
    const BuffChunkInfo ci = q.binfo[c];
    if (ci.status) {
        if (mark) set_status(acc, ci.status);
        return;
    }
    k.base = ci.base;
    k.bits = ci.bits;
    k.frac = ci.frac;
    k.np = k.bits / 8;
    k.tb = k.bits % 8;
    k.planes = q.file + ci.planes;
    k.tail = q.file + ci.tail;
    k.stride = ci.stride;
    k.scale = k.frac <= 1023 ? __longlong_as_double(static_cast<long long>(uint64_t(1023 + k.frac) << 52))
                             : __longlong_as_double(0x7ff0000000000000ll);
    k.inv_scale = k.frac <= 1022 ? __longlong_as_double(static_cast<long long>(uint64_t(1023 - k.frac) << 52)) : 0.0;
    k.fits32 = k.frac <= 1022 && k.bits <= 31 && k.base >= -2147483648ll &&
               k.base + ((1ll << k.bits) - 1) <= 2147483647ll;

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
        load32(k.planes + uint64_t(p) * k.stride + r0, w);
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

struct BlockRed {
    unsigned long long sum[kTileWarps], cnt[kTileWarps], mx[kTileWarps], mn[kTileWarps];
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
        for (int w = 0; w < kTileWarps; ++w) {
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


}  // namespace
}  // namespace ebi
