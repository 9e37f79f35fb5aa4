// buff_common.cuh -- BUFF helpers shared by the scan and the materialize kernels:
// fixed-point conversion and the predicate compiled into the delta domain.
#pragma once

#include "internal.h"

namespace ebi {
namespace buff {



// into_fixed_representation_with_fractional_part_bits_length
// (compression_common/buff.rs:11-51), with the reference's release-build
// wrapping shift.
__device__ inline int64_t buff_fixed(double value, int32_t frac) {
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

// A row's value, (fixed as f64) / 2^frac (buff/decode.rs:5-17 divides by
// 2.0f64.powi(frac)), assembled on the integer pipes: the f64 conversion
// rounds |fixed| to 53 significant bits, ties to even (IEEE 754
// roundTiesToEven), and dividing by a power of two only lowers the exponent,
// exactly, while the result stays a normal double.  The remaining cases
// (frac > 1022, a subnormal result) take the f64 arithmetic itself.
__device__ __forceinline__ double fixed_to_f64(long long fixed, uint32_t frac, double scale) {
    const unsigned long long u = static_cast<unsigned long long>(fixed);
    const unsigned long long sign = u & 0x8000000000000000ull;
    const unsigned long long m = sign ? 0ull - u : u;
    if (m == 0) return 0.0;
    int e = 63 - __clzll(static_cast<long long>(m));  // m in [2^e, 2^(e+1))
    unsigned long long mant;
    if (e <= 52) {
        mant = m << (52 - e);
    } else {
        const int sh = e - 52;
        mant = m >> sh;
        const unsigned long long rem = m & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (mant & 1ull))) {
            ++mant;
            if (mant >> 53) { mant >>= 1; ++e; }
        }
    }
    if (frac > 1022u || e + 1023 <= static_cast<int>(frac)) return static_cast<double>(fixed) / scale;
    const unsigned long long ex = static_cast<unsigned long long>(e + 1023 - static_cast<int>(frac));
    return __longlong_as_double(static_cast<long long>(sign | (ex << 52) | (mant & 0xfffffffffffffull)));
}

// fixed_to_f64 for a value that fits an int32 with frac <= 1022: exact (at most
// 32 significant bits) and normal, so only the leading-zero count, one shift
// and the exponent remain, in 32-bit arithmetic.
__device__ __forceinline__ double fixed32_to_f64(int32_t fixed, uint32_t frac) {
    const uint32_t s = static_cast<uint32_t>(fixed >> 31);     // 0 or all ones
    const uint32_t m = (static_cast<uint32_t>(fixed) ^ s) - s;  // |fixed|
    const int lz = __clz(static_cast<int>(m));                  // m in [2^(31 - lz), 2^(32 - lz))
    // significand with its leading one at bit 52, plus the biased exponent minus one
    const unsigned long long mant = static_cast<unsigned long long>(m) << (lz + 21);
    const uint32_t hi = static_cast<uint32_t>(mant >> 32) + (static_cast<uint32_t>(1053 - lz - static_cast<int>(frac)) << 20);
    const uint32_t lo = static_cast<uint32_t>(mant);
    return m ? __hiloint2double(static_cast<int>(hi | (s & 0x80000000u)), static_cast<int>(lo)) : 0.0;
}

enum : uint32_t { SIDE_ABSENT = 0, SIDE_ALL = 1, SIDE_NONE = 2, SIDE_CMP = 3 };

// Predicate compiled into the delta domain of one chunk, exactly as the
// reference's in-situ filters decide it.
struct BuffPred {
    uint32_t lmode, rmode, lincl, rincl, emode;
    uint64_t lthr, rthr, etgt;
};

__device__ inline void compile_pred(const ebi_predicate& pr, int64_t base, uint32_t bits, uint32_t frac, bool has_mask,
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


}  // namespace buff
}  // namespace ebi
