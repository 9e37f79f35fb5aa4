// xor.cu -- kernel and launchers of the Chimp / Chimp128 chunk pass (xor_dev.cuh).
#include "internal.h"
#include "xor_dev.cuh"
#include "xor_lanes.cuh"

namespace ebi {
namespace {

constexpr int kLaneThreads = 32;  // chunks per CTA of the lane-per-chunk kernel

template <int CODEC>
__global__ void __launch_bounds__(kLaneThreads) xor_lanes_kernel(QueryParams q, uint32_t chunk_base, uint32_t n_chunks,
                                                                 int mode, const unsigned long long* chunk_offsets) {
    const uint32_t li = blockIdx.x * kLaneThreads + threadIdx.x;
    if (li < n_chunks) xor_lane_chunk<CODEC>(q, li, chunk_base + li, mode, chunk_offsets);
}

template <int CODEC>
__global__ void __launch_bounds__(kXorThreads, 2) xor_kernel(QueryParams q, uint32_t chunk_base, int mode,
                                                          const unsigned long long* chunk_offsets) {
    xor_chunk<CODEC>(q, blockIdx.x, chunk_base + blockIdx.x, mode, chunk_offsets);
}

template <int CODEC>
cudaError_t launch_codec(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                         const unsigned long long* chunk_offsets, cudaStream_t s) {
    static bool configured = false;  // per process; the attribute is per function
    constexpr size_t bytes = xor_smem_bytes(CODEC);
    if (!configured) {
        const cudaError_t e = cudaFuncSetAttribute(xor_kernel<CODEC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   static_cast<int>(bytes));
        if (e != cudaSuccess) return e;
        configured = true;
    }
    xor_kernel<CODEC><<<n_chunks, kXorThreads, bytes, s>>>(q, chunk_begin, mode, chunk_offsets);
    count_launch();
    return cudaGetLastError();
}

// Chunks per launch from which one thread per chunk beats one CTA per chunk
// (Chimp / Chimp128 chunks of 8,192 values on 152 SMs).
constexpr uint32_t kLanesFromChunks = 1024;

template <int CODEC>
cudaError_t launch_lanes(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                         const unsigned long long* chunk_offsets, cudaStream_t s) {
    xor_lanes_kernel<CODEC><<<(n_chunks + kLaneThreads - 1) / kLaneThreads, kLaneThreads, 0, s>>>(
        q, chunk_begin, n_chunks, mode, chunk_offsets);
    count_launch();
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_xor(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                       const unsigned long long* chunk_offsets, cudaStream_t s) {
    if (n_chunks == 0) return cudaSuccess;
    const bool lanes = n_chunks >= kLanesFromChunks;
    switch (q.scheme) {
    case EBI_GORILLA: return launch_gorilla(q, chunk_begin, n_chunks, mode, chunk_offsets, s);
    case EBI_CHIMP:
        return lanes ? launch_lanes<CODEC_CHIMP>(q, chunk_begin, n_chunks, mode, chunk_offsets, s)
                     : launch_codec<CODEC_CHIMP>(q, chunk_begin, n_chunks, mode, chunk_offsets, s);
    case EBI_CHIMP128:
        return lanes ? launch_lanes<CODEC_CHIMP128>(q, chunk_begin, n_chunks, mode, chunk_offsets, s)
                     : launch_codec<CODEC_CHIMP128>(q, chunk_begin, n_chunks, mode, chunk_offsets, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace ebi
