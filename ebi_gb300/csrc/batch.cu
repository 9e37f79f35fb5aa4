// batch.cu -- many queries over many columns of mixed codecs in one
// persistent launch.
//
// A batch is a list of work items, each naming a query and a unit of one of
// its columns: an 8,192-row BUFF tile, a whole Uncompressed / RLE / Chimp /
// Chimp128 / Elf / ElfOnChimp chunk, or a group of Gorilla chunks (one per warp).
// A Chimp-family item may name a run of consecutive queries over one column
// (count of them, at most 32): the chunk is decoded once for all of them.  A persistent
// grid of 256-thread CTAs pulls items from a device counter, so columns of
// very different lengths and codecs share the GPU without a launch per
// column; each item runs the same per-chunk device code as the single-column
// kernels and leaves its result in the query's own per-chunk accumulators.
// A second launch folds every query (one CTA per query, chunk order).
#include "internal.h"
#include "buff_tile.cuh"
#include "finalize.cuh"
#include "gorilla_dev.cuh"
#include "raw_dev.cuh"
#include "rle_dev.cuh"
#include "xor_dev.cuh"

namespace ebi {
namespace {

constexpr int kBatchThreads = 256;
static_assert(kBatchThreads == kXorThreads && kBatchThreads == kRleThreads, "codec CTA shapes");

// One function per item kind, kept out of line so that each gets its own
// register allocation (the kernel's is the largest, not the sum of all paths).
__device__ __noinline__ void item_buff_tile(const QueryParams& q, const BatchItem& it, BuffCtx& k, BlockRed& red) {
    const Tile t = q.tiles[it.unit];
    if (threadIdx.x == 0) buff_setup(q, t.chunk, q.in_mask != nullptr, k);
    __syncthreads();
    if (k.ok && k.bits > 32) buff_query_dispatch<unsigned long long>(q, k, t.chunk, it.unit, t.begin, red);
    else buff_query_dispatch<uint32_t>(q, k, t.chunk, it.unit, t.begin, red);
}
__device__ __noinline__ void item_raw(const QueryParams& q, const BatchItem& it) {
    raw_chunk<kBatchThreads>(q, it.unit, it.unit, VAL_SCAN, nullptr);
}
__device__ __noinline__ void item_rle(const QueryParams& q, const BatchItem& it) {
    rle_chunk(q, it.unit, it.unit, VAL_SCAN, nullptr);
}
__device__ __noinline__ void item_gorilla(const QueryParams& q, const BatchItem& it) {
    const uint32_t warp = threadIdx.x >> 5, chunks = it.count & 0xffu;
    const uint32_t nq = it.count >> 8 ? it.count >> 8 : 1u;  // queries it.query .. + nq: one column
    if (warp < chunks) gorilla_chunk_l1<kGorillaShare>(&q, nq, it.unit + warp, it.unit + warp, VAL_SCAN, nullptr);
}
__device__ __noinline__ void item_chimp(const QueryParams& q, const BatchItem& it) {
    xor_chunk<CODEC_CHIMP>(&q, it.count, it.unit, it.unit, VAL_SCAN, nullptr);  // queries it.query .. + count: one column
}
__device__ __noinline__ void item_chimp128(const QueryParams& q, const BatchItem& it) {
    xor_chunk<CODEC_CHIMP128>(&q, it.count, it.unit, it.unit, VAL_SCAN, nullptr);  // queries it.query .. + count: one column
}
__device__ __noinline__ void item_elf_chimp(const QueryParams& q, const BatchItem& it) {
    xor_chunk<CODEC_ELF_CHIMP>(&q, it.count, it.unit, it.unit, VAL_SCAN, nullptr);  // queries it.query .. + count: one column
}
__device__ __noinline__ void item_elf(const QueryParams& q, const BatchItem& it) {
    xor_chunk<CODEC_ELF>(&q, it.count, it.unit, it.unit, VAL_SCAN, nullptr);  // queries it.query .. + count: one column
}

__global__ void __launch_bounds__(kBatchThreads, 2)
batch_kernel(const QueryParams* __restrict__ qp, const BatchItem* __restrict__ items, uint32_t n_items,
             unsigned int* counter) {
    __shared__ uint32_t s_item;
    __shared__ BuffCtx s_k;
    __shared__ BlockRed s_red;
    for (;;) {
        __syncthreads();  // every thread is done with the previous item's shared state
        if (threadIdx.x == 0) s_item = atomicAdd(counter, 1u);
        __syncthreads();
        const uint32_t i = s_item;
        if (i >= n_items) break;
        const BatchItem it = items[i];
        const QueryParams& q = qp[it.query];
        switch (it.kind) {
        case ITEM_BUFF_TILE: item_buff_tile(q, it, s_k, s_red); break;
        case ITEM_RAW: item_raw(q, it); break;
        case ITEM_RLE: item_rle(q, it); break;
        case ITEM_GORILLA: item_gorilla(q, it); break;
        case ITEM_CHIMP: item_chimp(q, it); break;
        case ITEM_CHIMP128: item_chimp128(q, it); break;
        case ITEM_ELF_CHIMP: item_elf_chimp(q, it); break;
        case ITEM_ELF: item_elf(q, it); break;
        default: break;
        }
    }
}

__global__ void __launch_bounds__(kFinThreads) batch_finalize_kernel(const QueryParams* __restrict__ qp,
                                                                     QueryResult* res) {
    finalize_chunks(qp[blockIdx.x], res + blockIdx.x);
}

}  // namespace

size_t batch_smem_bytes() {
    static_assert(xor_smem_bytes(CODEC_CHIMP128) >= xor_smem_bytes(CODEC_ELF), "largest codec body");
    return xor_smem_bytes(CODEC_CHIMP128);
}

void column_items(int scheme, uint64_t n_chunks, uint32_t n_tiles, uint32_t query, std::vector<BatchItem>& out) {
    switch (scheme) {
    case EBI_BUFF:
        for (uint32_t t = 0; t < n_tiles; ++t) out.push_back({query, ITEM_BUFF_TILE, t, 1});
        return;
    case EBI_GORILLA:
        for (uint64_t k = 0; k < n_chunks; k += 8)
            out.push_back({query, ITEM_GORILLA, static_cast<uint32_t>(k),
                           static_cast<uint32_t>(n_chunks - k < 8 ? n_chunks - k : 8)});
        return;
    default: {
        const uint32_t kind = scheme == EBI_UNCOMPRESSED ? ITEM_RAW
                            : scheme == EBI_RLE          ? ITEM_RLE
                            : scheme == EBI_CHIMP        ? ITEM_CHIMP
                            : scheme == EBI_CHIMP128     ? ITEM_CHIMP128
                            : scheme == EBI_ELF_ON_CHIMP ? ITEM_ELF_CHIMP
                                                         : ITEM_ELF;
        for (uint64_t k = 0; k < n_chunks; ++k) out.push_back({query, kind, static_cast<uint32_t>(k), 1});
    }
    }
}

double item_cost(uint32_t kind, uint32_t count) {
    switch (kind) {
    case ITEM_GORILLA: return 40.0 * (count & 0xffu);  // the chunks; queries sharing them cost little more
    case ITEM_ELF: return 35.0;
    case ITEM_ELF_CHIMP: return 35.0;
    case ITEM_CHIMP128: return 30.0;
    case ITEM_CHIMP: return 25.0;
    case ITEM_BUFF_TILE: return 1.0;
    case ITEM_RLE: return 0.5;
    default: return 2.0;
    }
}

cudaError_t prepare_batch_kernel() {
    return cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(batch_smem_bytes()));
}

cudaError_t launch_batch(const QueryParams* d_qp, const BatchItem* d_items, uint32_t n_items, unsigned int* d_counter,
                         uint32_t grid, cudaStream_t s) {
    if (n_items == 0) return cudaSuccess;
    const size_t smem = batch_smem_bytes();
    cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
    batch_kernel<<<grid, kBatchThreads, smem, s>>>(d_qp, d_items, n_items, d_counter);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_batch_finalize(const QueryParams* d_qp, QueryResult* d_res, uint32_t n_queries, cudaStream_t s) {
    if (n_queries == 0) return cudaSuccess;
    batch_finalize_kernel<<<n_queries, kFinThreads, 0, s>>>(d_qp, d_res);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ebi
