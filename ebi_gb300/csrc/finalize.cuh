// finalize.cuh -- the chunk-ordered fold of per-chunk results (Decoder's
// `result += chunk`, `result = result.min(chunk)`, `result = result.max(chunk)`,
// api/decoder.rs:323-439), shared by the single-query finalize (query.cu) and
// the batched launch (batch.cu).
#pragma once

#include <climits>

#include "fold.cuh"

namespace ebi {
namespace {

constexpr int kFinThreads = 1024;

template <typename T, typename F>
__device__ __forceinline__ T block_reduce(T v, F op, T* sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = lane < static_cast<int>(blockDim.x >> 5) ? sh[lane] : sh[0];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) sh[0] = v;
    }
    __syncthreads();
    return sh[0];
}

// ---- the fold of the other codecs' partials (double-double sums, min / max)
// A fixed tree over chunk indices, computed the same way by every path:
// slices of kSliceChunks chunks, each by one warp (lane l adds chunks 2l and
// 2l + 1 of the slice in order, then a shuffle tree in lane order); then the
// slices by one warp (lane l adds slices l, l + 32, ... in order, then the
// same tree).  A slice's warp re-arms its chunks' accumulators once read.
// Few FP64 operations per warp and many warps: one CTA folding every chunk
// was bound by the FP64 pipe of its one SM.

__device__ __forceinline__ ValPart val_part_rest() {
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    return ValPart{0.0, 0.0, inf, -inf, 0ull, 0xffffffffu, 0u};
}

// a += b: sums in double-double, min / max, counts, the lowest failing chunk.
__device__ __forceinline__ void val_part_add(ValPart& a, const ValPart& b) {
    dd_add(a.hi, a.lo, b.hi, b.lo);
    a.mn = fmin(a.mn, b.mn);
    a.mx = fmax(a.mx, b.mx);
    a.cnt += b.cnt;
    if (b.bad < a.bad) { a.bad = b.bad; a.bad_st = b.bad_st; }
}

__device__ __forceinline__ ValPart val_part_shfl_down(const ValPart& v, int o) {
    ValPart r;
    r.hi = __shfl_down_sync(0xffffffffu, v.hi, o);
    r.lo = __shfl_down_sync(0xffffffffu, v.lo, o);
    r.mn = __shfl_down_sync(0xffffffffu, v.mn, o);
    r.mx = __shfl_down_sync(0xffffffffu, v.mx, o);
    r.cnt = __shfl_down_sync(0xffffffffu, v.cnt, o);
    r.bad = __shfl_down_sync(0xffffffffu, v.bad, o);
    r.bad_st = __shfl_down_sync(0xffffffffu, v.bad_st, o);
    return r;
}

// The lane-order tree of one warp; the result is valid in lane 0.
__device__ __forceinline__ ValPart val_part_warp(ValPart v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const ValPart b = val_part_shfl_down(v, o);
        if ((lane & (2 * o - 1)) == 0) val_part_add(v, b);
    }
    return v;
}

// Slice s of query q by one warp (the result in lane 0); re-arms its chunks.
__device__ __forceinline__ ValPart slice_fold(const QueryParams& q, uint32_t s) {
    const int lane = threadIdx.x & 31;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    ValPart v = val_part_rest();
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const uint32_t c = s * kSliceChunks + 2 * lane + k;
        if (c >= q.n_chunks) break;
        const ChunkAcc a = q.acc[c];
        ValPart w = val_part_rest();
        if (a.status) { w.bad = c; w.bad_st = a.status; }
        if (chunk_included(q, a)) {
            w.hi = a.fsum_hi;
            w.lo = a.fsum_lo;
            w.mn = a.fmin;
            w.mx = a.fmax;
            w.cnt = a.count;
        }
        val_part_add(v, w);
        ChunkAcc rest = {};
        rest.dmin = ~0ull;
        rest.fmin = inf;
        rest.fmax = -inf;
        q.acc[c] = rest;
    }
    return val_part_warp(v);
}

__device__ __forceinline__ QueryResult val_part_result(const ValPart& v) {
    QueryResult r;
    r.status = v.bad == 0xffffffffu ? 0u : v.bad_st;
    r.bad_chunk = v.bad;
    r.sum = v.hi + v.lo;
    r.min = v.mn;
    r.max = v.mx;
    r.count = v.cnt;
    return r;
}

// The whole fold of a non-BUFF query by one CTA of kFinThreads threads (the
// batched path: one CTA per query): warps take slices 32 at a time, warp 0
// adds each group into its lanes' running slice sums.
__device__ inline void fold_values_cta(const QueryParams& q, QueryResult* res) {
    __shared__ ValPart parts[kFinThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    constexpr int kWarps = kFinThreads / 32;
    const uint32_t S = value_slices(q.n_chunks);
    ValPart acc = val_part_rest();  // warp 0, lane l: slices l, l + 32, ...
    for (uint32_t g = 0; g < S; g += kWarps) {
        const uint32_t s = g + wid;
        const ValPart p = s < S ? slice_fold(q, s) : val_part_rest();
        if (lane == 0) parts[wid] = p;
        __syncthreads();
        if (wid == 0 && g + lane < S) val_part_add(acc, parts[lane]);
        __syncthreads();
    }
    if (wid == 0) {
        const ValPart r = val_part_warp(acc);
        if (lane == 0) *res = val_part_result(r);
    }
}

// Folds BUFF query q's per-chunk partials in chunk order into *res and
// re-arms q.acc.  A CTA of kFinThreads threads.
__device__ __forceinline__ void finalize_chunks(const QueryParams& q, QueryResult* res) {
    __shared__ unsigned long long sh_u[32];
    __shared__ long long sh_i[32];
    const uint32_t nc = q.n_chunks;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);

    uint32_t bad = 0xffffffffu;
    unsigned long long cnt = 0;
    // integer facts (BUFF)
    long long ssum = 0, smax = LLONG_MIN, smin = LLONG_MAX;
    unsigned long long sabs = 0;
    uint32_t fracmin = 0xffffffffu, fracmax = 0, exact = 1, any = 0;
    // each thread folds a contiguous run of chunks, runs combine in thread order
    const uint32_t per = (nc + kFinThreads - 1) / kFinThreads;
    const uint32_t c0 = min(nc, threadIdx.x * per), c1 = min(nc, c0 + per);
    for (uint32_t c = c0; c < c1; ++c) {
        const ChunkAcc a = q.acc[c];
        if (a.status && bad == 0xffffffffu) bad = c;
        if (!chunk_included(q, a)) continue;
        any = 1;
        cnt += a.count;
        const BuffVal v = buff_value(q, c, a);
        exact &= v.sum_exact;
        ssum += v.sum_fixed;
        const unsigned long long ab = static_cast<unsigned long long>(v.sum_fixed < 0 ? -v.sum_fixed : v.sum_fixed);
        sabs = (sabs + ab < sabs || sabs + ab > (1ull << 62)) ? (1ull << 62) : sabs + ab;
        smax = max(smax, v.max_fixed);
        smin = min(smin, v.min_fixed);
        fracmin = min(fracmin, v.frac);
        fracmax = max(fracmax, v.frac);
    }
    bad = block_reduce<unsigned long long>(bad, [](unsigned long long x, unsigned long long y) { return x < y ? x : y; }, sh_u);
    cnt = block_reduce<unsigned long long>(cnt, [](unsigned long long x, unsigned long long y) { return x + y; }, sh_u);
    any = static_cast<uint32_t>(block_reduce<unsigned long long>(any, [](unsigned long long x, unsigned long long y) { return x | y; }, sh_u));
    QueryResult r;
    r.status = 0;
    r.bad_chunk = static_cast<uint32_t>(bad);
    r.count = cnt;
    ssum = block_reduce<long long>(ssum, [](long long x, long long y) { return x + y; }, sh_i);
    smax = block_reduce<long long>(smax, [](long long x, long long y) { return x > y ? x : y; }, sh_i);
    smin = block_reduce<long long>(smin, [](long long x, long long y) { return x < y ? x : y; }, sh_i);
    sabs = block_reduce<unsigned long long>(sabs, [](unsigned long long x, unsigned long long y) {
        return x + y > (1ull << 62) ? (1ull << 62) : x + y; }, sh_u);
    exact = static_cast<uint32_t>(block_reduce<unsigned long long>(exact, [](unsigned long long x, unsigned long long y) { return x & y; }, sh_u));
    fracmin = static_cast<uint32_t>(block_reduce<unsigned long long>(fracmin, [](unsigned long long x, unsigned long long y) { return x < y ? x : y; }, sh_u));
    fracmax = static_cast<uint32_t>(block_reduce<unsigned long long>(fracmax, [](unsigned long long x, unsigned long long y) { return x > y ? x : y; }, sh_u));
    if (threadIdx.x == 0) {
        if (!any) {
            r.sum = 0.0; r.min = inf; r.max = -inf;
        } else if (fracmin == fracmax) {
            // Every chunk value is integer * 2^-frac: min and max convert once.
            r.max = fold_scale(smax, fracmin);
            r.min = fold_scale(smin, fracmin);
            if (exact && sabs < (1ull << 53)) {
                // Each chunk sum and every prefix of the chunk-ordered fold is
                // an exact multiple of 2^-frac below 2^53 of them, so the
                // reference's sequential f64 fold is exact: it equals the total.
                r.sum = fold_scale(ssum, fracmin);
            } else {
                double s = 0.0;  // the reference's sequential `result += chunk_sum`
                for (uint32_t c = 0; c < nc; ++c) {
                    const ChunkAcc a = q.acc[c];
                    if (chunk_included(q, a)) s += buff_chunk_sum_f64(buff_value(q, c, a), c, q);
                }
                r.sum = s;
            }
        } else {
            double s = 0.0, a1 = inf, b1 = -inf;
            for (uint32_t c = 0; c < nc; ++c) {
                const ChunkAcc a = q.acc[c];
                if (!chunk_included(q, a)) continue;
                const BuffVal v = buff_value(q, c, a);
                s += buff_chunk_sum_f64(v, c, q);
                a1 = fmin(a1, fold_scale(v.min_fixed, v.frac));
                b1 = fmax(b1, fold_scale(v.max_fixed, v.frac));
            }
            r.sum = s; r.min = a1; r.max = b1;
        }
    }
    if (threadIdx.x == 0) {
        if (r.bad_chunk != 0xffffffffu) r.status = q.acc[r.bad_chunk].status;
        *res = r;
    }
    __syncthreads();
    // re-arm the accumulators for the next query
    for (uint32_t c = threadIdx.x; c < nc; c += blockDim.x) {
        ChunkAcc a = {};
        a.dmin = ~0ull;
        a.fmin = inf;
        a.fmax = -inf;
        q.acc[c] = a;
    }
}


}  // namespace
}  // namespace ebi
