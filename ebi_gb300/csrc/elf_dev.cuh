// elf_dev.cuh -- decimal restoration of the Elf / ElfOnChimp readers on the
// device: recover_v_by_beta_star (decoder/chunk_reader/elf.rs:66-81) with the
// helpers of compression_common/elf.rs.
//
// The host builds one table of doubles per device (elf_tables.cu):
//   [kElfP10, +kElfNP10)  10^i, i < kElfNP10    (get_10i_p; inf above)
//   [kElfN10, +kElfNN10)  10^-i, i < kElfNN10   (get_10i_n; 0 above)
//   [kElfSpB, +kElfNSp)   for k = -324 .. 308, the least positive double v
//                         with floor(log10(v)) >= k, log10 being the host C
//                         library's (the function get_sp calls for values
//                         outside [1e-10, 1e9))
// so every step is table lookups, comparisons and correctly rounded IEEE
// multiplies, divisions, floor and ceil: the results are the reference's bits.
#pragma once

#include <cstdint>

namespace ebi {

constexpr uint32_t kElfNP10 = 310;   // 10^309 and up overflow to inf
constexpr uint32_t kElfNN10 = 325;   // 10^-324 and down round to 0
constexpr int32_t kElfSpMin = -324;  // floor(log10) of the least subnormal
constexpr int32_t kElfSpMax = 308;   // floor(log10) of the greatest double
constexpr uint32_t kElfNSp = kElfSpMax - kElfSpMin + 1;
constexpr uint32_t kElfP10 = 0, kElfN10 = kElfNP10, kElfSpB = kElfNP10 + kElfNN10;
constexpr uint32_t kElfTabLen = kElfSpB + kElfNSp;

// Elf record flags (wrapper prefix of decoder/chunk_reader/elf.rs:42-64):
// restore the value with beta*, and a new beta* (low 4 bits) read before it.
constexpr uint8_t kElfRestore = 0x80, kElfBeta = 0x40;

#if defined(__CUDACC__)
// get_sp (elf.rs:115-133) of v = |v'|.
__device__ __forceinline__ int32_t elf_sp(double v, const double* __restrict__ tab) {
    if (v >= 1.0) {
        if (v < 1e9) {
            int32_t k = 0;
            while (k < 8 && v >= tab[kElfP10 + k + 1]) ++k;
            return k;
        }
    } else {
        for (int32_t i = 1; i <= 10; ++i)
            if (v >= tab[kElfN10 + i]) return -i;
    }
    // floor(log10(v)) as i32: NaN -> 0, inf -> i32::MAX, 0 -> i32::MIN
    if (v != v) return 0;
    const uint64_t b = static_cast<uint64_t>(__double_as_longlong(v));
    if (b >= 0x7ff0000000000000ull) return INT32_MAX;
    if (b == 0) return INT32_MIN;
    // binary exponent (subnormals: of the highest set bit), then
    // floor(e2 * log10(2)), which is sp or sp - 1
    const int32_t e2 = (b >> 52) ? static_cast<int32_t>(b >> 52) - 1023 : -1074 + (63 - __clzll(static_cast<long long>(b)));
    int32_t k = (e2 * 78913) >> 18;
    k = k < kElfSpMin ? kElfSpMin : (k > kElfSpMax ? kElfSpMax : k);
#pragma unroll 1
    for (int s = 0; s < 8 && k < kElfSpMax && v >= tab[kElfSpB + (k + 1 - kElfSpMin)]; ++s) ++k;
#pragma unroll 1
    for (int s = 0; s < 8 && k > kElfSpMin && v < tab[kElfSpB + (k - kElfSpMin)]; ++s) --k;
    return k;
}

// recover_v_by_beta_star: v' (the erased value) back to the decimal it
// stands for; beta = the last beta* read (i32::MAX before any).
__device__ __forceinline__ double elf_recover(double vp, int32_t beta, const double* __restrict__ tab) {
    const int32_t sp = elf_sp(fabs(vp), tab);
    if (beta == 0) {
        const uint32_t i = static_cast<uint32_t>(-static_cast<int64_t>(sp) - 1);
        const double r = i < kElfNN10 ? tab[kElfN10 + i] : 0.0;
        return vp < 0.0 ? -r : r;
    }
    // round_up (elf.rs:48-55) at alpha = beta - sp - 1 digits
    const uint32_t alpha = static_cast<uint32_t>(static_cast<int64_t>(beta) - sp - 1);
    const double scale = alpha < kElfNP10 ? tab[kElfP10 + alpha] : __longlong_as_double(0x7ff0000000000000ll);
    const double m = __dmul_rn(vp, scale);
    return vp < 0.0 ? __ddiv_rn(floor(m), scale) : __ddiv_rn(ceil(m), scale);
}
#endif

}  // namespace ebi
