// xor.cu -- kernel and launchers of the Chimp / Chimp128 / Elf / ElfOnChimp chunk pass (xor_dev.cuh).
#include "internal.h"
#include "xor_dev.cuh"

namespace ebi {
namespace {

template <int CODEC>
__global__ void __launch_bounds__(kXorThreads, 2) xor_kernel(QueryParams q, uint32_t chunk_base, int mode,
                                                          const unsigned long long* chunk_offsets,
                                                          const SegState* segs) {
    xor_chunk<CODEC>(&q, 1, blockIdx.x, chunk_base + blockIdx.x, mode, chunk_offsets, segs);
}

// The control parse of chunk chunk_base + blockIdx.x ahead of the chunk pass:
// the same rounds as the pass's own, but without the pass's shared memory
// (the chunk is read through L1, warmed in L2 first), so that many more
// chunks converge at once than the pass holds.  Chunks the pass decodes in
// order (or rejects) are skipped.
template <int CODEC>
__global__ void __launch_bounds__(kXorThreads, 4) xor_converge_kernel(QueryParams q, uint32_t chunk_base,
                                                                   SegState* segs) {
    __shared__ uint64_t s_in[kXorThreads], s_out[kXorThreads];
    __shared__ uint32_t s_red[kXorThreads / 32];
    const uint32_t li = blockIdx.x, c = chunk_base + li;
    const ChunkDesc cd = q.chunks[c];
    if (cd.flags & kChunkBadGeometry) return;
    const uint64_t B = cd.byte_len * 8;
    if (!((is_elf(CODEC) || B >= 64) && cd.n_rows + 1 < kRcap)) return;  // as xor_chunk's `parallel`
    for (uint64_t a = (cd.byte_off & ~uint64_t(127)) + uint64_t(threadIdx.x) * 128; a < cd.byte_off + cd.byte_len;
         a += uint64_t(kXorThreads) * 128)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(q.file + a));
    const uint32_t* fw = reinterpret_cast<const uint32_t*>(q.file);
    const uint64_t bit0 = cd.byte_off * 8;
    auto peek = [fw, bit0](uint64_t p) { return peek64_file(fw, bit0 + p); };
    PState in;
    uint32_t n, fail, first_fail;
    converge_segments<CODEC>(peek, B, s_in, s_out, s_red, in, n, fail, first_fail);
    segs[uint64_t(li) * kSegsPerChunk + threadIdx.x] = SegState{pack_state(in), n, fail};
}

template <int CODEC>
cudaError_t launch_codec(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                         const unsigned long long* chunk_offsets, cudaStream_t s) {
    constexpr size_t bytes = xor_smem_bytes(CODEC);
    const cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void*>(xor_kernel<CODEC>), bytes);
    if (e != cudaSuccess) return e;
    const SegState* segs = nullptr;
    if (mode == VAL_SCAN && q.segs) {
        xor_converge_kernel<CODEC><<<n_chunks, kXorThreads, 0, s>>>(q, chunk_begin, q.segs);
        count_launch();
        segs = q.segs;
    }
    xor_kernel<CODEC><<<n_chunks, kXorThreads, bytes, s>>>(q, chunk_begin, mode, chunk_offsets, segs);
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
