// rle.cu -- kernel and launcher of the RLE chunk pass (rle_dev.cuh).
#include "internal.h"
#include "rle_dev.cuh"

namespace ebi {
namespace {

__global__ void __launch_bounds__(kRleThreads) rle_kernel(QueryParams q, uint32_t chunk_base, int mode,
                                                          const unsigned long long* chunk_offsets) {
    rle_chunk(q, blockIdx.x, chunk_base + blockIdx.x, mode, chunk_offsets);
}

}  // namespace

cudaError_t launch_rle(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                       const unsigned long long* chunk_offsets, cudaStream_t s) {
    if (n_chunks == 0) return cudaSuccess;
    rle_kernel<<<n_chunks, kRleThreads, 0, s>>>(q, chunk_begin, mode, chunk_offsets);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ebi
