// xor.cu -- kernel and launchers of the Chimp / Chimp128 / Elf / ElfOnChimp
// chunk pass: one warp per chunk (xor_warp.cuh), several chunks per CTA.
#include "internal.h"
#include "xor_warp.cuh"

namespace ebi {
namespace {

// Warps (= chunks) per CTA and shared memory per warp: 8 KB of stream
// windows, and 2 KB of waiting bitmask words or, for Chimp128, 36 KB of
// rings (whose ext bytes hold the waiting bitmask words during the query
// pass); a CTA holds one Chimp128 warp and five fit an SM.
template <int CODEC>
constexpr int xor_warps() { return CODEC == CODEC_CHIMP128 ? 1 : 4; }
template <int CODEC>
constexpr size_t xor_warp_bytes() { return kWinBytes + (CODEC == CODEC_CHIMP128 ? kRingBytes : kBitBytes); }
template <int CODEC>
constexpr size_t xor_warp_smem() { return size_t(xor_warps<CODEC>()) * xor_warp_bytes<CODEC>(); }
static_assert(kBitBytes <= kRingBytes - kRingValBytes, "a Chimp128 warp's waiting bitmask words fit its ext bytes");

template <int CODEC>
__global__ void __launch_bounds__(xor_warps<CODEC>() * 32)
xor_warp_kernel(const __grid_constant__ QueryParams q, uint32_t chunk_base, uint32_t n_chunks, int mode,
                const unsigned long long* chunk_offsets) {
    extern __shared__ __align__(16) uint8_t smem[];
    const uint32_t w = threadIdx.x >> 5;
    const uint32_t li = blockIdx.x * xor_warps<CODEC>() + w;
    if (li >= n_chunks) return;  // whole warps; the kernel has no block barriers
    uint8_t* mine = smem + size_t(w) * xor_warp_bytes<CODEC>();
    uint64_t* rx = nullptr;
    uint8_t* re = nullptr;
    uint32_t* bits = reinterpret_cast<uint32_t*>(mine + kWinBytes);
    if (CODEC == CODEC_CHIMP128) {
        rx = reinterpret_cast<uint64_t*>(mine + kWinBytes);
        re = reinterpret_cast<uint8_t*>(rx + kLanes * kRingSlots);
        bits = reinterpret_cast<uint32_t*>(re);
    }
    xor_chunk_warp<CODEC, 1>(&q, 1, li, chunk_base + li, mode, chunk_offsets, reinterpret_cast<uint32_t*>(mine), bits,
                             rx, re);
}

template <int CODEC>
cudaError_t launch_codec(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                         const unsigned long long* chunk_offsets, cudaStream_t s) {
    constexpr size_t bytes = xor_warp_smem<CODEC>();
    if (bytes > 48 * 1024) {
        static bool configured = false;  // per process; the attribute is per function
        if (!configured) {
            const cudaError_t e = cudaFuncSetAttribute(xor_warp_kernel<CODEC>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       static_cast<int>(bytes));
            if (e != cudaSuccess) return e;
            configured = true;
        }
    }
    constexpr uint32_t W = xor_warps<CODEC>();
    xor_warp_kernel<CODEC><<<(n_chunks + W - 1) / W, W * 32, bytes, s>>>(q, chunk_begin, n_chunks, mode, chunk_offsets);
    count_launch();
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_xor(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                       const unsigned long long* chunk_offsets, cudaStream_t s) {
    if (n_chunks == 0) return cudaSuccess;
    switch (q.scheme) {
    case EBI_GORILLA: return launch_gorilla(q, chunk_begin, n_chunks, mode, chunk_offsets, s);
    case EBI_CHIMP: return launch_codec<CODEC_CHIMP>(q, chunk_begin, n_chunks, mode, chunk_offsets, s);
    case EBI_CHIMP128: return launch_codec<CODEC_CHIMP128>(q, chunk_begin, n_chunks, mode, chunk_offsets, s);
    case EBI_ELF_ON_CHIMP: return launch_codec<CODEC_ELF_CHIMP>(q, chunk_begin, n_chunks, mode, chunk_offsets, s);
    case EBI_ELF: return launch_codec<CODEC_ELF>(q, chunk_begin, n_chunks, mode, chunk_offsets, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace ebi
