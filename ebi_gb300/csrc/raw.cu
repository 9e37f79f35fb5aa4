// raw.cu -- kernel and launcher of the Uncompressed chunk pass (raw_dev.cuh).
#include "internal.h"
#include "raw_dev.cuh"

namespace ebi {
namespace {

constexpr int kRawThreads = 512;

__global__ void __launch_bounds__(kRawThreads) raw_kernel(QueryParams q, uint32_t chunk_base, int mode,
                                                          const unsigned long long* chunk_offsets) {
    raw_chunk<kRawThreads>(q, blockIdx.x, chunk_base + blockIdx.x, mode, chunk_offsets);
}

}  // namespace

cudaError_t launch_raw(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                       const unsigned long long* chunk_offsets, cudaStream_t s) {
    if (n_chunks == 0) return cudaSuccess;
    raw_kernel<<<n_chunks, kRawThreads, 0, s>>>(q, chunk_begin, mode, chunk_offsets);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ebi
