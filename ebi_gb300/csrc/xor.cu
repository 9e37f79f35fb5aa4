// xor.cu -- kernel and launchers of the Chimp / Chimp128 / Elf / ElfOnChimp chunk pass (xor_dev.cuh).
#include "internal.h"
#include "xor_dev.cuh"

namespace ebi {
namespace {

template <int CODEC>
__global__ void __launch_bounds__(kXorThreads, 2) xor_kernel(QueryParams q, uint32_t chunk_base, int mode,
                                                          const unsigned long long* chunk_offsets) {
    xor_chunk<CODEC>(&q, 1, blockIdx.x, chunk_base + blockIdx.x, mode, chunk_offsets);
}

template <int CODEC>
cudaError_t launch_codec(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                         const unsigned long long* chunk_offsets, cudaStream_t s) {
    constexpr size_t bytes = xor_smem_bytes(CODEC);
    const cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void*>(xor_kernel<CODEC>), bytes);
    if (e != cudaSuccess) return e;
    xor_kernel<CODEC><<<n_chunks, kXorThreads, bytes, s>>>(q, chunk_begin, mode, chunk_offsets);
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
