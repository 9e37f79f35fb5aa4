// values.cuh -- the reference's default operators on decoded f64 values
// (decoder/query.rs:14-154), shared by the codecs that decode to values before
// querying them (RLE, Uncompressed, Gorilla, Chimp, Chimp128).
//
// Per chunk, rows are decided as the default operators do: a row counts when
// it is in the input bitmask (or there is none) and, for a filter, when the
// predicate holds.  The chunk's sum is compensated, min/max are NaN-ignoring
// (f64::min/max).  Partial results are combined in a fixed order, so a query
// returns the same bits on every run and whatever else runs on the GPU.
#pragma once

#include "common.cuh"

namespace ebi {

// ---- ordered keys ---------------------------------------------------------
// order_key maps f64 bits to an unsigned key whose order is the IEEE total
// order (-NaN < -inf < ... < -0 < +0 < ... < +inf < +NaN).  Predicates, min
// and max compare keys on the integer pipes: GB300's FP64 pipe is a small
// fraction of its integer throughput.
constexpr uint64_t kAbsMask = 0x7fffffffffffffffull;
constexpr uint64_t kSignBit = 0x8000000000000000ull;
__host__ __device__ __forceinline__ constexpr uint64_t order_key(uint64_t b) { return (b >> 63) ? ~b : (b | kSignBit); }
__host__ __device__ __forceinline__ constexpr uint64_t key_bits(uint64_t k) { return (k >> 63) ? (k & ~kSignBit) : ~k; }
__device__ __forceinline__ bool is_nan_bits(uint64_t b) { return (b & kAbsMask) > 0x7ff0000000000000ull; }
constexpr uint64_t kKeyPosInf = order_key(0x7ff0000000000000ull);
constexpr uint64_t kKeyNegInf = order_key(0xfff0000000000000ull);
// Key with -0 and +0 merged (they compare equal in IEEE predicates).
__device__ __forceinline__ uint64_t cmp_key(uint64_t b) { return (b & kAbsMask) ? order_key(b) : kSignBit; }

// A Predicate (decoder/query.rs:396-437) over keys: exactly the f64
// comparisons of RangeImpl::eval / PredicateImpl::eval, NaN included (a NaN
// operand fails every comparison, so NaN rows pass only Ne).
struct KeyPred {
    uint64_t lo, hi;  // cmp_key of the bounds (Eq / Ne: lo = the operand)
    uint32_t kind;    // EBI_PRED_*
    bool lo_on, lo_incl, hi_on, hi_incl, never;
    __device__ __forceinline__ bool pass(uint64_t b) const {
        if (is_nan_bits(b)) return kind == EBI_PRED_NE;
        const uint64_t k = cmp_key(b);
        if (kind != EBI_PRED_RANGE) return ((k == lo) && !never) != (kind == EBI_PRED_NE);
        if (never) return false;
        const bool a = !lo_on || (lo_incl ? k >= lo : k > lo);
        const bool c = !hi_on || (hi_incl ? k <= hi : k < hi);
        return a && c;
    }
};
__device__ __forceinline__ KeyPred key_pred(const ebi_predicate& p) {
    KeyPred kp{};
    kp.kind = static_cast<uint32_t>(p.kind);
    if (p.kind != EBI_PRED_RANGE) {
        const uint64_t b = static_cast<uint64_t>(__double_as_longlong(p.value));
        kp.never = is_nan_bits(b);  // x == NaN is false for every x
        kp.lo = cmp_key(b);
        return kp;
    }
    const uint64_t s = static_cast<uint64_t>(__double_as_longlong(p.start));
    const uint64_t e = static_cast<uint64_t>(__double_as_longlong(p.end));
    kp.lo_on = p.start_kind != EBI_BOUND_NONE;
    kp.hi_on = p.end_kind != EBI_BOUND_NONE;
    kp.lo_incl = p.start_kind == EBI_BOUND_INCLUSIVE;
    kp.hi_incl = p.end_kind == EBI_BOUND_INCLUSIVE;
    kp.never = (kp.lo_on && is_nan_bits(s)) || (kp.hi_on && is_nan_bits(e));
    kp.lo = cmp_key(s);
    kp.hi = cmp_key(e);
    return kp;
}

// ---- per-chunk aggregates --------------------------------------------------
// The sum is compensated (Neumaier: a running sum plus the exact rounding
// error of every addition), min/max are ordered keys with NaN skipped, as
// f64::min / f64::max ignore a NaN operand.  `want` (AGG_* bits) switches off
// what the caller did not ask for; the count is always kept.
struct ValAgg {
    double hi, lo;
    unsigned long long mnk, mxk;
    unsigned long long cnt;
    uint32_t want;
};

__device__ __forceinline__ ValAgg val_agg_init(uint32_t want = AGG_ALL) {
    return ValAgg{0.0, 0.0, kKeyPosInf, kKeyNegInf, 0, want};
}

// hi + lo += v (one FP64 add on the dependency chain through hi).  Once the
// running sum leaves the finite range it carries the plain IEEE sum.
__device__ __forceinline__ void neumaier_add(double& hi, double& lo, double v) {
    const double s = hi + v;
    const uint64_t sb = static_cast<uint64_t>(__double_as_longlong(s));
    if ((sb & kAbsMask) < 0x7ff0000000000000ull) {
        const uint64_t hb = static_cast<uint64_t>(__double_as_longlong(hi)) & kAbsMask;
        const uint64_t vb = static_cast<uint64_t>(__double_as_longlong(v)) & kAbsMask;
        lo += hb >= vb ? (hi - s) + v : (v - s) + hi;
    }
    hi = s;
}
__device__ __forceinline__ double neumaier_value(double hi, double lo) {
    const uint64_t hb = static_cast<uint64_t>(__double_as_longlong(hi));
    return (hb & kAbsMask) < 0x7ff0000000000000ull ? hi + lo : hi;
}

__device__ __forceinline__ void val_agg_minmax(ValAgg& a, uint64_t b) {
    if ((a.want & (AGG_MIN | AGG_MAX)) && !is_nan_bits(b)) {
        const uint64_t k = order_key(b);
        a.mnk = k < a.mnk ? k : a.mnk;
        a.mxk = k > a.mxk ? k : a.mxk;
    }
}

// One value (bits).
__device__ __forceinline__ void val_agg_add1(ValAgg& a, uint64_t b) {
    ++a.cnt;
    val_agg_minmax(a, b);
    if (a.want & AGG_SUM) neumaier_add(a.hi, a.lo, __longlong_as_double(static_cast<long long>(b)));
}

// k copies of v (RLE runs): v * k split exactly into product and FMA error.
__device__ __forceinline__ void val_agg_add(ValAgg& a, double v, uint32_t k) {
    if (!k) return;
    a.cnt += k;
    const uint64_t b = static_cast<uint64_t>(__double_as_longlong(v));
    val_agg_minmax(a, b);
    if (a.want & AGG_SUM) {
        const double kd = static_cast<double>(k);
        // rounded on its own (never fused into the add that follows): every
        // kernel that adds runs gets the same bits, whatever the compiler fuses
        const double p = __dmul_rn(v, kd);
        neumaier_add(a.hi, a.lo, p);
        const uint64_t pb = static_cast<uint64_t>(__double_as_longlong(p));
        if ((pb & kAbsMask) < 0x7ff0000000000000ull) a.lo += fma(v, kd, -p);
    }
}

__device__ __forceinline__ void val_agg_merge(ValAgg& a, const ValAgg& b) {
    if (a.want & AGG_SUM) {
        neumaier_add(a.hi, a.lo, b.hi);
        const uint64_t hb = static_cast<uint64_t>(__double_as_longlong(a.hi));
        if ((hb & kAbsMask) < 0x7ff0000000000000ull) a.lo += b.lo;
    }
    a.mnk = b.mnk < a.mnk ? b.mnk : a.mnk;
    a.mxk = b.mxk > a.mxk ? b.mxk : a.mxk;
    a.cnt += b.cnt;
}

__device__ __forceinline__ ValAgg val_agg_shfl_down(const ValAgg& a, int o) {
    ValAgg b;
    b.hi = __shfl_down_sync(0xffffffffu, a.hi, o);
    b.lo = __shfl_down_sync(0xffffffffu, a.lo, o);
    b.mnk = __shfl_down_sync(0xffffffffu, a.mnk, o);
    b.mxk = __shfl_down_sync(0xffffffffu, a.mxk, o);
    b.cnt = __shfl_down_sync(0xffffffffu, a.cnt, o);
    b.want = a.want;
    return b;
}

// Warp merge in a fixed tree (lane order); the result is in lane 0.
__device__ __forceinline__ ValAgg val_agg_warp(ValAgg a) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const ValAgg b = val_agg_shfl_down(a, o);
        if ((lane & (2 * o - 1)) == 0) val_agg_merge(a, b);
    }
    return a;
}

// Block-wide merge in a fixed tree (lane order, then warp order); the result
// is valid in thread 0.  `sh` holds one ValAgg per warp.
__device__ inline ValAgg val_agg_block(ValAgg a, ValAgg* sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    a = val_agg_warp(a);
    __syncthreads();
    if (lane == 0) sh[wid] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w) val_agg_merge(a, sh[w]);
    }
    return a;
}

// Stores a chunk's result in its accumulator (at rest before: one writer per chunk).
__device__ __forceinline__ void val_agg_store(ChunkAcc* acc, const ValAgg& a) {
    acc->fsum_hi = a.hi;
    acc->fsum_lo = a.lo;
    acc->fmin = __longlong_as_double(static_cast<long long>(key_bits(a.mnk)));
    acc->fmax = __longlong_as_double(static_cast<long long>(key_bits(a.mxk)));
    acc->count = a.cnt;
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
