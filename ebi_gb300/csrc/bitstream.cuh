// bitstream.cuh -- big-endian bit reads over the resident file (XOR codecs).
//
// The stream's bit 0 is the most significant bit of the chunk's first byte.
// peek64 returns the 64 stream bits starting at a bit position from three
// 32-bit words; the file's 64 bytes of zero padding keep the over-read of the
// last record inside the allocation.
#pragma once

#include <cstdint>

namespace ebi {

__device__ __forceinline__ uint32_t bswap32(uint32_t x) { return __byte_perm(x, 0, 0x0123); }

// From a big-endian word array (already byte-swapped, e.g. staged in shared memory).
__device__ __forceinline__ uint64_t peek64_be(const uint32_t* w, uint64_t q) {
    const uint64_t i = q >> 5;
    const uint32_t sh = static_cast<uint32_t>(q & 31);
    const uint32_t a = w[i], b = w[i + 1], c = w[i + 2];
    const uint32_t hi = __funnelshift_l(b, a, sh), lo = __funnelshift_l(c, b, sh);
    return (uint64_t(hi) << 32) | lo;
}
// From little-endian file words in global memory.
__device__ __forceinline__ uint64_t peek64_file(const uint32_t* w, uint64_t q) {
    const uint64_t i = q >> 5;
    const uint32_t sh = static_cast<uint32_t>(q & 31);
    const uint32_t a = bswap32(__ldg(w + i)), b = bswap32(__ldg(w + i + 1)), c = bswap32(__ldg(w + i + 2));
    const uint32_t hi = __funnelshift_l(b, a, sh), lo = __funnelshift_l(c, b, sh);
    return (uint64_t(hi) << 32) | lo;
}

}  // namespace ebi
