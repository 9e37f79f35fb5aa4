// batch.cu -- many queries over many columns of mixed codecs in one
// persistent launch.
//
// A batch is a list of work items, each naming a query and a unit of one of
// its columns: a run of 8,192-row BUFF tiles, a run of Uncompressed / RLE
// chunks, a whole Chimp / Chimp128 / Elf / ElfOnChimp chunk, or a group of
// Gorilla chunks (one warp walks each; eight warps per item).  How many tiles
// or chunks one item covers is the batch's tiling (BatchTiling, per codec
// family and column-size bucket), which the batch's first run tunes.
// A Chimp-family item may name a run of consecutive queries over one column
// (count of them, at most 32): the chunk is decoded once for all of them.  A persistent
// grid of 256-thread CTAs pulls items from a device counter, so columns of
// very different lengths and codecs share the GPU without a launch per
// column; each item runs the same per-chunk device code as the single-column
// kernels and leaves its result in the query's own per-chunk accumulators.
// A second launch folds every query (one CTA per query, chunk order).
#include <algorithm>
#include <vector>

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
static_assert(kBatchThreads == kXorThreads, "codec CTA shapes");

// One function per item kind, kept out of line so that each gets its own
// register allocation (the kernel's is the largest, not the sum of all paths).
// One tile with 32-bit or 64-bit deltas, each out of line with its own
// register allocation (the 64-bit form needs twice the delta registers).
__device__ __noinline__ void buff_tile32(const QueryParams& q, const BuffCtx& k, uint32_t chunk, uint32_t tile,
                                         uint32_t begin, BlockRed& red) {
    buff_query_dispatch<uint32_t>(q, k, chunk, tile, begin, red);
}
__device__ __noinline__ void buff_tile64(const QueryParams& q, const BuffCtx& k, uint32_t chunk, uint32_t tile,
                                         uint32_t begin, BlockRed& red) {
    buff_query_dispatch<unsigned long long>(q, k, chunk, tile, begin, red);
}

// Tiles [unit, unit + count) of one query's column; the chunk context is set
// up again only when the chunk changes.
__device__ __noinline__ void item_buff_tile(const QueryParams& q, const BatchItem& it, BuffCtx& k, BlockRed& red) {
    uint32_t chunk = 0xffffffffu;
    for (uint32_t j = 0; j < it.count; ++j) {
        const uint32_t tile = it.unit + j;
        const Tile t = q.tiles[tile];
        // thread 0 has read the previous tile's block reduction (and every
        // thread is done with k) before any warp writes the next one
        if (j) __syncthreads();
        if (t.chunk != chunk) {
            if (threadIdx.x == 0) buff_setup(q, t.chunk, q.in_mask != nullptr, k);
            __syncthreads();
            chunk = t.chunk;
        }
        if (k.ok && k.bits > 32) buff_tile64(q, k, t.chunk, tile, t.begin, red);
        else buff_tile32(q, k, t.chunk, tile, t.begin, red);
    }
}
__device__ __noinline__ void item_raw(const QueryParams& q, const BatchItem& it) {
    for (uint32_t j = 0; j < it.count; ++j) {
        if (j) __syncthreads();  // the previous chunk is done with shared memory
        raw_chunk<kBatchThreads>(q, it.unit + j, it.unit + j, VAL_SCAN, nullptr);
    }
}
// Chunks [unit, unit + count): warp w takes chunks w, w + 8, ... with its
// share of the dynamic shared memory.
static_assert((kBatchThreads / 32) * sizeof(RleWarpSmem) <= xor_smem_bytes(CODEC_CHIMP128),
              "the batch kernel's dynamic shared memory holds one RLE stage per warp");
__device__ __noinline__ void item_rle(const QueryParams& q, const BatchItem& it) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    RleWarpSmem* sm = reinterpret_cast<RleWarpSmem*>(smem_raw) + (threadIdx.x >> 5);
    for (uint32_t j = threadIdx.x >> 5; j < it.count; j += kBatchThreads / 32)
        rle_chunk_warp(q, it.unit + j, it.unit + j, VAL_SCAN, nullptr, sm);
}
// Chunks [unit, unit + chunks): warp w walks chunks w, w + 8, ...  Up to
// kGorillaShare queries keep their state in registers; more (up to
// kGorillaShareWide) keep it in the warp's share of the dynamic shared memory.
static_assert(kGorillaShareWide <= kSharedSinkQueries, "shared-memory walk state");
static_assert((kBatchThreads / 32) * sizeof(SharedSinkState) <= xor_smem_bytes(CODEC_CHIMP128),
              "the batch kernel's dynamic shared memory holds one walk state per warp");
__device__ __noinline__ void item_gorilla(const QueryParams& q, const BatchItem& it) {
    const uint32_t warp = threadIdx.x >> 5, chunks = it.count & 0xffu;
    const uint32_t nq = it.count >> 8 ? it.count >> 8 : 1u;  // queries it.query .. + nq: one column
    if (nq <= kGorillaShare) {
        for (uint32_t w = warp; w < chunks; w += kBatchThreads / 32)
            gorilla_chunk_l1<kGorillaShare>(&q, nq, it.unit + w, it.unit + w, VAL_SCAN, nullptr);
        return;
    }
    extern __shared__ __align__(16) uint8_t smem_raw[];
    SharedSinkState* st = reinterpret_cast<SharedSinkState*>(smem_raw) + warp;
    for (uint32_t w = warp; w < chunks; w += kBatchThreads / 32) gorilla_chunk_l1_shared(&q, nq, it.unit + w, st);
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
    const QueryParams& q = qp[blockIdx.x];
    if (q.scheme == EBI_BUFF) finalize_chunks(q, res + blockIdx.x);
    else fold_values_cta(q, res + blockIdx.x);
}

}  // namespace

size_t batch_smem_bytes() {
    static_assert(xor_smem_bytes(CODEC_CHIMP128) >= xor_smem_bytes(CODEC_ELF), "largest codec body");
    return xor_smem_bytes(CODEC_CHIMP128);
}

int size_bucket(uint64_t n_records) { return n_records < (1ull << 18) ? 0 : n_records < (1ull << 22) ? 1 : 2; }

BatchTiling default_tiling() {
    BatchTiling t{};
    for (int b = 0; b < kSizeBuckets; ++b) {
        t.buff_tiles[b] = 8;
        t.value_chunks[b] = 8;
        t.gorilla_chunks[b] = 16;
    }
    return t;
}

void column_items(int scheme, uint64_t n_chunks, uint32_t n_tiles, uint64_t n_records, const BatchTiling& tl,
                  uint32_t query, std::vector<BatchItem>& out) {
    const int b = size_bucket(n_records);
    auto clamp = [](uint32_t v, uint32_t hi) { return v < 1 ? 1u : v > hi ? hi : v; };
    switch (scheme) {
    case EBI_BUFF: {
        const uint32_t per = clamp(tl.buff_tiles[b], kMaxItemTiles);
        for (uint32_t t = 0; t < n_tiles; t += per)
            out.push_back({query, ITEM_BUFF_TILE, t, n_tiles - t < per ? n_tiles - t : per});
        return;
    }
    case EBI_GORILLA: {
        const uint64_t per = clamp(tl.gorilla_chunks[b], kMaxGorillaChunks);
        for (uint64_t k = 0; k < n_chunks; k += per)
            out.push_back({query, ITEM_GORILLA, static_cast<uint32_t>(k),
                           static_cast<uint32_t>(n_chunks - k < per ? n_chunks - k : per)});
        return;
    }
    case EBI_UNCOMPRESSED:
    case EBI_RLE: {
        const uint64_t per = clamp(tl.value_chunks[b], kMaxItemTiles);
        const uint32_t kind = scheme == EBI_RLE ? ITEM_RLE : ITEM_RAW;
        for (uint64_t k = 0; k < n_chunks; k += per)
            out.push_back({query, kind, static_cast<uint32_t>(k), static_cast<uint32_t>(n_chunks - k < per ? n_chunks - k : per)});
        return;
    }
    default: {
        const uint32_t kind = scheme == EBI_CHIMP        ? ITEM_CHIMP
                            : scheme == EBI_CHIMP128     ? ITEM_CHIMP128
                            : scheme == EBI_ELF_ON_CHIMP ? ITEM_ELF_CHIMP
                                                         : ITEM_ELF;
        for (uint64_t k = 0; k < n_chunks; ++k) out.push_back({query, kind, static_cast<uint32_t>(k), 1});
    }
    }
}

void shared_column_items(int scheme, uint64_t n_chunks, uint32_t n_tiles, uint64_t n_records, const BatchTiling& t,
                         uint32_t first, uint32_t n, std::vector<BatchItem>& out) {
    const bool chimp = scheme == EBI_CHIMP || scheme == EBI_CHIMP128 || scheme == EBI_ELF_ON_CHIMP || scheme == EBI_ELF;
    const uint32_t end = first + n;
    if (chimp) {
        for (uint32_t q0 = first; q0 < end; q0 += 32) {
            const size_t i0 = out.size();
            column_items(scheme, n_chunks, n_tiles, n_records, t, q0, out);
            for (size_t i = i0; i < out.size(); ++i) out[i].count = std::min<uint32_t>(32, end - q0);
        }
    } else if (scheme == EBI_GORILLA) {
        for (uint32_t q0 = first; q0 < end; q0 += kGorillaShareWide) {
            const size_t i0 = out.size();
            column_items(scheme, n_chunks, n_tiles, n_records, t, q0, out);
            const uint32_t share = std::min<uint32_t>(kGorillaShareWide, end - q0);
            for (size_t i = i0; i < out.size(); ++i) out[i].count |= share << 8;
        }
    } else {
        for (uint32_t qi = first; qi < end; ++qi) column_items(scheme, n_chunks, n_tiles, n_records, t, qi, out);
    }
}

uint64_t column_item_count(int scheme, uint64_t n_chunks, uint32_t n_tiles, uint64_t n_records, const BatchTiling& tl) {
    const int b = size_bucket(n_records);
    auto per = [](uint32_t v, uint32_t hi) -> uint64_t { return v < 1 ? 1u : v > hi ? hi : v; };
    switch (scheme) {
    case EBI_BUFF: return (n_tiles + per(tl.buff_tiles[b], kMaxItemTiles) - 1) / per(tl.buff_tiles[b], kMaxItemTiles);
    case EBI_GORILLA:
        return (n_chunks + per(tl.gorilla_chunks[b], kMaxGorillaChunks) - 1) / per(tl.gorilla_chunks[b], kMaxGorillaChunks);
    case EBI_UNCOMPRESSED:
    case EBI_RLE: return (n_chunks + per(tl.value_chunks[b], kMaxItemTiles) - 1) / per(tl.value_chunks[b], kMaxItemTiles);
    default: return n_chunks;
    }
}

double item_cost(uint32_t kind, uint32_t count) {
    switch (kind) {
    case ITEM_GORILLA: return 40.0 * (count & 0xffu);  // the chunks; queries sharing them cost little more
    case ITEM_ELF: return 35.0;
    case ITEM_ELF_CHIMP: return 35.0;
    case ITEM_CHIMP128: return 30.0;
    case ITEM_CHIMP: return 25.0;
    case ITEM_BUFF_TILE: return 1.0 * count;
    case ITEM_RLE: return 0.5 * count;
    default: return 2.0 * count;
    }
}

void order_by_cost(std::vector<BatchItem>& items) {
    // distinct costs, descending; then a stable counting sort on their rank
    std::vector<double> costs;
    std::vector<uint32_t> rank(items.size());
    for (size_t i = 0; i < items.size(); ++i) {
        const double c = item_cost(items[i].kind, items[i].count);
        size_t r = 0;
        while (r < costs.size() && costs[r] != c) ++r;
        if (r == costs.size()) {
            if (costs.size() == 256) {  // not a handful after all
                std::stable_sort(items.begin(), items.end(), [](const BatchItem& x, const BatchItem& y) {
                    return item_cost(x.kind, x.count) > item_cost(y.kind, y.count);
                });
                return;
            }
            costs.push_back(c);
        }
        rank[i] = static_cast<uint32_t>(r);
    }
    std::vector<uint32_t> order(costs.size());
    for (uint32_t r = 0; r < order.size(); ++r) order[r] = r;
    std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return costs[a] > costs[b]; });
    std::vector<size_t> pos_of(costs.size()), cnt(costs.size(), 0);
    for (uint32_t r : rank) ++cnt[r];
    size_t at = 0;
    for (uint32_t r : order) { pos_of[r] = at; at += cnt[r]; }
    std::vector<BatchItem> out(items.size());
    for (size_t i = 0; i < items.size(); ++i) out[pos_of[rank[i]]++] = items[i];
    items.swap(out);
}

cudaError_t prepare_batch_kernel() {
    return allow_dynamic_smem(reinterpret_cast<const void*>(batch_kernel), batch_smem_bytes());
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
