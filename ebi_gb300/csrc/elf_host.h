// elf_host.h -- host-side decimal helpers of the Elf codecs
// (compression_common/elf.rs), shared by the encoder and by the builder of the
// device decimal tables.  Float -> int casts saturate (NaN -> 0) and integer
// arithmetic wraps, as Rust's `as` casts and release-mode arithmetic do.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

namespace ebi {
namespace elf {

inline int32_t sat_i32(double x) {
    if (x != x) return 0;
    if (x >= 2147483647.0) return INT32_MAX;
    if (x <= -2147483648.0) return INT32_MIN;
    return static_cast<int32_t>(x);
}
inline int64_t sat_i64(double x) {
    if (x != x) return 0;
    if (x >= 9223372036854775807.0) return INT64_MAX;
    if (x <= -9223372036854775808.0) return INT64_MIN;
    return static_cast<int64_t>(x);
}
inline uint32_t sat_u32(double x) {
    if (x != x || x <= 0.0) return 0;
    if (x >= 4294967295.0) return UINT32_MAX;
    return static_cast<uint32_t>(x);
}

// get_10i_p / get_10i_n (elf.rs:97-113): 10^i and 10^-i as the nearest double
// (the tables below 21 are exact; above, the decimal string "1.0E{i}" parsed).
inline double pow10_pos(uint32_t i) {
    static const double kP[21] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9, 1e10,
                                  1e11, 1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20};
    if (i < 21) return kP[i];
    char b[32];
    std::snprintf(b, sizeof b, "1.0E%u", i);
    return std::strtod(b, nullptr);
}
inline double pow10_neg(uint32_t i) {
    static const double kN[21] = {1e-0,  1e-1,  1e-2,  1e-3,  1e-4,  1e-5,  1e-6,  1e-7,  1e-8,  1e-9, 1e-10,
                                  1e-11, 1e-12, 1e-13, 1e-14, 1e-15, 1e-16, 1e-17, 1e-18, 1e-19, 1e-20};
    if (i < 21) return kN[i];
    char b[32];
    std::snprintf(b, sizeof b, "1.0E-%u", i);
    return std::strtod(b, nullptr);
}

// get_sp_and_10i_n_flag (elf.rs:135-155): the decimal exponent of v > 0 and
// whether v is exactly 10^sp.  get_sp (elf.rs:115-133) is the same without the flag.
inline int32_t sp_of(double v, bool* exact_pow10) {
    if (exact_pow10) *exact_pow10 = false;
    if (v >= 1.0) {
        double p = 1.0;
        for (int32_t i = 0; i < 9; ++i) {
            p *= 10.0;
            if (v < p) return i;
        }
    } else {
        for (uint32_t i = 1; i < 11; ++i) {
            const double t = pow10_neg(i);
            if (v >= t) {
                if (exact_pow10) *exact_pow10 = v == t;
                return -static_cast<int32_t>(i);
            }
        }
    }
    const double l = std::log10(v);
    if (exact_pow10) *exact_pow10 = l == std::floor(l);
    return sat_i32(std::floor(l));
}

// get_f_alpha (elf.rs:33-39): ceil(alpha * log2(10)).
inline uint32_t f_alpha(uint32_t alpha) {
    static const uint32_t kF[21] = {0, 4, 7, 10, 14, 17, 20, 24, 27, 30, 34, 37, 40, 44, 47, 50, 54, 57, 60, 64, 67};
    if (alpha < 21) return kF[alpha];
    return sat_u32(std::ceil(static_cast<double>(alpha) * 3.32192809488736234787));
}

// get_significant_count (elf.rs:57-95): decimal significant digits of v > 0
// (17 when v needs more than a double's worth).
inline int32_t significant(double v, int32_t sp, int32_t last_beta_star) {
    int32_t i;
    if (last_beta_star != INT32_MAX && last_beta_star != 0) {
        i = last_beta_star - sp - 1;
        if (i < 1) i = 1;
    } else if (last_beta_star == INT32_MAX) {
        i = 17 - sp - 1;
    } else if (sp >= 0) {
        i = 1;
    } else {
        i = -sp;
    }
    double t = v * pow10_pos(static_cast<uint32_t>(i));
    int64_t ti = sat_i64(t);
    while (static_cast<double>(ti) != t) {
        ++i;
        t = v * pow10_pos(static_cast<uint32_t>(i));
        if (std::isinf(t)) return 17;
        ti = sat_i64(t);
    }
    if (t / pow10_pos(static_cast<uint32_t>(i)) != v) return 17;
    while (i > 0 && ti % 10 == 0) {
        --i;
        ti /= 10;
    }
    return sp + i + 1;
}

}  // namespace elf
}  // namespace ebi
