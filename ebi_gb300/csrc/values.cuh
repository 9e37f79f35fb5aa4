// values.cuh -- the reference's default operators on decoded f64 values
// (decoder/query.rs:14-154), shared by the codecs that decode to values before
// querying them (RLE, Uncompressed, Gorilla, Chimp, Chimp128).
//
// Per chunk, rows are judged as the default operators do: a row counts when
// it is in the input bitmask (or there is none) and, for a filter, when the
// predicate holds.  The chunk's sum is kept as a double-double (compensated)
// value, min/max with fmin/fmax (NaN-ignoring, as f64::min/max).  Partial
// results are combined in a fixed order, so a query returns the same bits on
// every run and whatever else runs on the GPU.
#pragma once

#include "common.cuh"

namespace ebi {

struct ValAgg {
    double hi, lo;   // double-double sum
    double mn, mx;
    unsigned long long cnt;
};

__device__ __forceinline__ ValAgg val_agg_init() {
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    return ValAgg{0.0, 0.0, inf, -inf, 0};
}

// Adds k copies of v (v * k exactly, through an FMA product split).
__device__ __forceinline__ void val_agg_add(ValAgg& a, double v, uint32_t k) {
    if (!k) return;
    const double kd = static_cast<double>(k);
    const double p = v * kd;
    const double e = fma(v, kd, -p);
    dd_add(a.hi, a.lo, p, e);
    a.mn = fmin(a.mn, v);
    a.mx = fmax(a.mx, v);
    a.cnt += k;
}

__device__ __forceinline__ void val_agg_merge(ValAgg& a, const ValAgg& b) {
    dd_add(a.hi, a.lo, b.hi, b.lo);
    a.mn = fmin(a.mn, b.mn);
    a.mx = fmax(a.mx, b.mx);
    a.cnt += b.cnt;
}

// Block-wide merge in a fixed tree (lane order, then warp order); the result
// is valid in thread 0.  `sh` holds one ValAgg per warp.
__device__ inline ValAgg val_agg_block(ValAgg a, ValAgg* sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        ValAgg b;
        b.hi = __shfl_down_sync(0xffffffffu, a.hi, o);
        b.lo = __shfl_down_sync(0xffffffffu, a.lo, o);
        b.mn = __shfl_down_sync(0xffffffffu, a.mn, o);
        b.mx = __shfl_down_sync(0xffffffffu, a.mx, o);
        b.cnt = __shfl_down_sync(0xffffffffu, a.cnt, o);
        if ((lane & (2 * o - 1)) == 0 && lane + o < 32) val_agg_merge(a, b);
    }
    __syncthreads();
    if (lane == 0) sh[wid] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w) val_agg_merge(a, sh[w]);
    }
    return a;
}

// Adds a chunk's partial into its accumulator (one thread; chunks processed
// by one CTA, so the order is fixed).
__device__ __forceinline__ void val_agg_store(ChunkAcc* acc, const ValAgg& a) {
    double hi = acc->fsum_hi, lo = acc->fsum_lo;
    dd_add(hi, lo, a.hi, a.lo);
    acc->fsum_hi = hi;
    acc->fsum_lo = lo;
    acc->fmin = fmin(acc->fmin, a.mn);
    acc->fmax = fmax(acc->fmax, a.mx);
    acc->count += a.cnt;
}

// Row g of the input bitmask (false past n_records, as RoaringBitmap::contains of a u32 row set).
__device__ __forceinline__ bool mask_row(const uint32_t* m, uint64_t n_records, uint64_t g) {
    return g < n_records && ((m[g >> 5] >> (g & 31)) & 1u);
}

// Exclusive block scan of one u32 per thread (blockDim.x = NT); *total gets the sum.
template <int NT>
__device__ __forceinline__ uint32_t block_excl_scan_u32(uint32_t v, uint32_t* sh, uint32_t* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    __syncthreads();
    if (lane == 31) sh[wid] = inc;
    __syncthreads();
    uint32_t before = 0, t = 0;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) {
        if (w < wid) before += sh[w];
        t += sh[w];
    }
    *total = t;
    return before + inc - v;
}

__device__ __forceinline__ uint32_t range_bits(uint32_t lo, uint32_t hi) {  // bits [lo, hi) of a word, 0 <= lo <= hi <= 32
    const uint32_t a = lo >= 32 ? 0u : (~0u << lo);
    const uint32_t b = hi >= 32 ? ~0u : ((1u << hi) - 1u);
    return a & b;
}

}  // namespace ebi
