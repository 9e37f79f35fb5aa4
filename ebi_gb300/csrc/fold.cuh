// fold.cuh -- the reference's per-chunk BUFF results in exact integer form and
// the chunk-ordered f64 fold of Decoder::{sum, min, max} (api/decoder.rs:323-439).
#pragma once

#include <climits>

#include "common.cuh"

namespace ebi {

__device__ __forceinline__ double fold_pow2(int e) {  // 2^e for -1022 <= e <= 1023, exact
    return __longlong_as_double(static_cast<long long>(uint64_t(1023 + e) << 52));
}
// (double)x / 2^frac exactly as `x as f64 / 2.0f64.powi(frac)` rounds it.
__device__ __forceinline__ double fold_scale(long long x, uint32_t frac) {
    const double v = static_cast<double>(x);
    if (frac <= 1022) return __dmul_rn(v, fold_pow2(-static_cast<int>(frac)));
    return v / (frac <= 1023 ? fold_pow2(1023) : __longlong_as_double(0x7ff0000000000000ll));
}

// One BUFF chunk's contribution in exact integer form: every result of the
// reference is (integer) as f64 / 2^frac (buff/sum.rs:116, buff/min_max.rs:273-276).
struct BuffVal {
    long long sum_fixed;  // sum_with_bitmask's integer before the f64 conversion
    long long max_fixed, min_fixed;
    uint32_t frac;
    bool sum_exact;       // the chunk's f64 sum equals sum_fixed * 2^-frac exactly
};

__device__ inline BuffVal buff_value(const QueryParams& q, uint32_t c, const ChunkAcc& a) {
    const BuffChunkInfo ci = q.binfo[c];
    const bool has_mask = q.in_mask != nullptr || q.op == OP_FILTER_AGG;
    BuffVal v;
    v.frac = ci.frac;
    constexpr long long kExact = 1ll << 53;
    if (ci.bits == 0) {
        // base / scale * number_of_records (buff/sum.rs:81-84)
        const __int128 p = static_cast<__int128>(ci.base) * ci.n;
        v.sum_fixed = static_cast<long long>(p);
        v.sum_exact = p < kExact && p > -kExact && ci.base < kExact && ci.base > -kExact && ci.frac <= 1022;
        v.max_fixed = v.min_fixed = ci.base;
    } else {
        v.sum_fixed = static_cast<long long>(a.isum + static_cast<unsigned long long>(ci.base) * a.count);
        v.sum_exact = v.sum_fixed < kExact && v.sum_fixed > -kExact && ci.frac <= 1022;
        v.max_fixed = static_cast<long long>(static_cast<unsigned long long>(ci.base) + a.dmax);
        // min_without_bitmask returns base / scale (buff/min_max.rs:316-341)
        v.min_fixed = has_mask ? static_cast<long long>(static_cast<unsigned long long>(ci.base) + a.dmin) : ci.base;
    }
    return v;
}
__device__ inline double buff_chunk_sum_f64(const BuffVal& v, uint32_t c, const QueryParams& q) {
    const BuffChunkInfo ci = q.binfo[c];
    // rounded on its own: never fused into the reference's `result += chunk` that follows
    if (ci.bits == 0) return __dmul_rn(fold_scale(ci.base, ci.frac), static_cast<double>(ci.n));
    return fold_scale(v.sum_fixed, v.frac);
}

__device__ __forceinline__ bool chunk_included(const QueryParams& q, const ChunkAcc& a) {
    if (a.status) return false;
    return q.op == OP_FILTER_AGG ? a.count > 0 : a.selected != 0;
}


// Sequential fold of every included BUFF chunk, in chunk order, exactly as
// the reference accumulates it (one thread).
__device__ inline void fold_buff_chunks(const QueryParams& q, QueryResult& r) {
    double s = 0.0, mn = r.min, mx = r.max;
    for (uint32_t c = 0; c < q.n_chunks; ++c) {
        const ChunkAcc a = q.acc[c];
        if (!chunk_included(q, a)) continue;
        const BuffVal v = buff_value(q, c, a);
        s += buff_chunk_sum_f64(v, c, q);
        mn = fmin(mn, fold_scale(v.min_fixed, v.frac));
        mx = fmax(mx, fold_scale(v.max_fixed, v.frac));
    }
    r.sum = s;
    r.min = mn;
    r.max = mx;
}

}  // namespace ebi
