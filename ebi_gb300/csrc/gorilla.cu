// gorilla.cu -- kernel and launcher of the Gorilla chunk pass (gorilla_dev.cuh):
// one warp per chunk, the chunk staged in shared memory by one bulk copy
// (cp.async.bulk, completed on an mbarrier with a bounded wait); chunks above
// the staging size are read through L1 from the resident file instead.
#include "internal.h"
#include "gorilla_dev.cuh"

namespace ebi {
namespace {

constexpr int kWarpsPerCta = 1;  // one chunk (and its staged bytes) per CTA

__global__ void __launch_bounds__(kWarpsPerCta * 32) gorilla_kernel(QueryParams q, uint32_t chunk_base, uint32_t n_chunks,
                                                                    int mode, const unsigned long long* chunk_offsets) {
    const int lane = threadIdx.x & 31;
    const uint32_t li = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
    if (li >= n_chunks) return;  // whole warps; the kernel has no block barriers
    const uint32_t c = chunk_base + li;
    if (!gorilla_begin(q, li, c, mode, chunk_offsets)) return;
    const ChunkDesc cd = q.chunks[c];
    ChunkAcc* acc = q.acc + c;
    extern __shared__ __align__(16) uint8_t smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
    const uint32_t* stage = reinterpret_cast<const uint32_t*>(smem + 16);
    const uint64_t span = stage_span(cd.byte_off, cd.byte_len);
    if (span <= q.stage_bytes) {
        const uint8_t* src = q.file + (cd.byte_off & ~uint64_t(15));
        if (lane == 0) {
            mbar_init(bar, 1);
            fence_mbar_init();
            mbar_arrive_expect_tx(bar, static_cast<uint32_t>(span));
            bulk_g2s(smem + 16, src, static_cast<uint32_t>(span), bar);
        }
        __syncwarp();
        bool arrived = mbar_wait(bar, 0, q.copy_wait);
        if (!__all_sync(kFull, arrived)) {
            // give the copy a second wait (full limit) before the CTA leaves, then report it
            mbar_wait(bar, 0);
            if (lane == 0) {
                set_status(acc, EBI_E_CUDA);
                if (mode == VAL_COUNT) q.tile_counts[li] = 0;
            }
            return;
        }
        const uint64_t bit0 = (cd.byte_off & 15) * 8;
        walk<1>(&q, 1, 1u, cd, c, li, mode, chunk_offsets,
                [stage, bit0](uint64_t p) { return peek64_le_smem(stage, bit0 + p); });
    } else {
        const uint32_t* fw = reinterpret_cast<const uint32_t*>(q.file);
        const uint64_t bit0 = cd.byte_off * 8;
        walk<1>(&q, 1, 1u, cd, c, li, mode, chunk_offsets, [fw, bit0](uint64_t p) { return peek64_file(fw, bit0 + p); });
    }
}

}  // namespace

uint32_t gorilla_stage_bytes(const ChunkDesc* chunks, uint64_t n) {
    uint64_t mx = 0;
    for (uint64_t i = 0; i < n; ++i) {
        if (chunks[i].flags & kChunkBadGeometry) continue;
        const uint64_t sp = stage_span(chunks[i].byte_off, chunks[i].byte_len);
        if (sp <= kGorillaStageCap && sp > mx) mx = sp;
    }
    return static_cast<uint32_t>(mx);
}

cudaError_t launch_gorilla(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                           const unsigned long long* chunk_offsets, cudaStream_t s) {
    if (n_chunks == 0) return cudaSuccess;
    const uint32_t grid = (n_chunks + kWarpsPerCta - 1) / kWarpsPerCta;
    const size_t smem = q.stage_bytes ? 16 + size_t(q.stage_bytes) : 16;
    const cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void*>(gorilla_kernel), smem);
    if (e != cudaSuccess) return e;
    gorilla_kernel<<<grid, kWarpsPerCta * 32, smem, s>>>(q, chunk_begin, n_chunks, mode, chunk_offsets);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ebi
