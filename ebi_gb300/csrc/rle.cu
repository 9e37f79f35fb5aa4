// rle.cu -- kernel and launcher of the RLE chunk pass (rle_dev.cuh).
#include "internal.h"
#include "rle_dev.cuh"

namespace ebi {
namespace {

// Warp w of CTA b: chunk chunk_base + 4b + w (small CTAs spread the chunks
// evenly over the SMs).
constexpr uint32_t kRleWarps = 4;
__global__ void __launch_bounds__(kRleWarps * 32) rle_kernel(QueryParams q, uint32_t chunk_base, uint32_t n_chunks,
                                                             int mode, const unsigned long long* chunk_offsets) {
    __shared__ RleWarpSmem sm[kRleWarps];
    const uint32_t warp = threadIdx.x >> 5, li = blockIdx.x * kRleWarps + warp;
    if (li >= n_chunks) return;
    rle_chunk_warp(q, li, chunk_base + li, mode, chunk_offsets, sm + warp);
}

}  // namespace

cudaError_t launch_rle(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                       const unsigned long long* chunk_offsets, cudaStream_t s) {
    if (n_chunks == 0) return cudaSuccess;
    rle_kernel<<<(n_chunks + kRleWarps - 1) / kRleWarps, kRleWarps * 32, 0, s>>>(q, chunk_begin, n_chunks, mode,
                                                                             chunk_offsets);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ebi
