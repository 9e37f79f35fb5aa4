// rowset.cu -- conversions between a set of u32 row ids (what the reference's
// RoaringBitmap holds and iterates in ascending order) and the engine's dense
// bitmask (ceil(n_records / 64) little-endian u64 words), on the device.
//
//   rows -> mask: every row id sets its bit (duplicates and any order allowed;
//                 ids >= n_records are dropped: no chunk can hold them).
//   mask -> rows: the set rows in ascending order, as RoaringBitmap::iter gives
//                 them: per-block popcounts, an exclusive scan of the block
//                 totals, then each block writes its rows at its offset.
#include <algorithm>

#include "internal.h"

namespace ebi {
namespace {

constexpr int kThreads = 256;
constexpr uint32_t kWordsPerBlock = 8192;  // u32 words of the bitmask per CTA

__global__ void rows_to_mask_kernel(const uint32_t* rows, uint64_t n, uint32_t* mask, uint64_t n_records) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
        const uint32_t r = rows[i];
        if (r < n_records) atomicOr(mask + (r >> 5), 1u << (r & 31));
    }
}

__device__ __forceinline__ uint32_t word_at(const uint32_t* mask, uint64_t w, uint64_t n_words, uint64_t n_records) {
    if (w >= n_words) return 0;
    uint32_t x = mask[w];
    const uint64_t base = w << 5;
    if (n_records - base < 32) x &= (1u << (n_records - base)) - 1u;  // bits past the last row
    return x;
}

// Block b: total set bits of words [b * kWordsPerBlock, (b + 1) * kWordsPerBlock).
__global__ void __launch_bounds__(kThreads) mask_block_counts(const uint32_t* mask, uint64_t n_words, uint64_t n_records,
                                                             unsigned long long* counts) {
    __shared__ unsigned long long red[kThreads / 32];
    const uint64_t w0 = uint64_t(blockIdx.x) * kWordsPerBlock;
    unsigned long long c = 0;
    for (uint32_t k = threadIdx.x; k < kWordsPerBlock; k += kThreads) c += __popc(word_at(mask, w0 + k, n_words, n_records));
    c = warp_sum(c);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int i = 0; i < kThreads / 32; ++i) t += red[i];
        counts[blockIdx.x] = t;
    }
}

// Block b writes the rows of its words at offsets[b] onwards, ascending.
__global__ void __launch_bounds__(kThreads) mask_write_rows(const uint32_t* mask, uint64_t n_words, uint64_t n_records,
                                                           const unsigned long long* offsets, uint32_t* rows,
                                                           uint64_t cap) {
    __shared__ unsigned long long wsum[kThreads / 32];
    __shared__ unsigned long long carry;
    if (threadIdx.x == 0) carry = offsets[blockIdx.x];
    __syncthreads();
    const uint64_t w0 = uint64_t(blockIdx.x) * kWordsPerBlock;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (uint32_t k0 = 0; k0 < kWordsPerBlock; k0 += kThreads) {
        const uint64_t w = w0 + k0 + threadIdx.x;
        const uint32_t x = word_at(mask, w, n_words, n_records);
        const uint32_t c = __popc(x);
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) wsum[wid] = inc;
        __syncthreads();
        unsigned long long before = carry, all = 0;
        for (int i = 0; i < kThreads / 32; ++i) {
            if (i < wid) before += wsum[i];
            all += wsum[i];
        }
        unsigned long long pos = before + inc - c;
        for (uint32_t bits = x; bits; bits &= bits - 1, ++pos)
            if (pos < cap) rows[pos] = static_cast<uint32_t>((w << 5) + __ffs(bits) - 1);
        __syncthreads();
        if (threadIdx.x == 0) carry += all;
        __syncthreads();
    }
}

}  // namespace
}  // namespace ebi

using namespace ebi;

extern "C" {

int ebi_mask_from_rows(const uint32_t* d_rows, uint64_t n_rows, uint64_t n_records, uint64_t* d_mask, void* stream) {
    if ((!d_rows && n_rows) || !d_mask) {
        set_last_error("rows or mask is null");
        return EBI_E_INVALID;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint64_t words = (n_records + 63) / 64;
    cudaError_t e = cudaMemsetAsync(d_mask, 0, (words ? words : 1) * 8, s);
    if (e == cudaSuccess && n_rows) {
        const uint64_t blocks = std::min<uint64_t>((n_rows + kThreads - 1) / kThreads, 4096);
        rows_to_mask_kernel<<<static_cast<uint32_t>(blocks), kThreads, 0, s>>>(d_rows, n_rows,
                                                                            reinterpret_cast<uint32_t*>(d_mask), n_records);
        count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_last_error(std::string("ebi_mask_from_rows: ") + cudaGetErrorString(e));
        return EBI_E_CUDA;
    }
    return EBI_OK;
}

int ebi_rows_from_mask(const uint64_t* d_mask, uint64_t n_records, uint32_t* d_rows, uint64_t cap, uint64_t* n_out,
                       void* stream) {
    if (!d_mask || (!d_rows && cap) || !n_out) {
        set_last_error("mask, rows or n_out is null");
        return EBI_E_INVALID;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint64_t n_words = (n_records + 31) / 32;  // u32 words holding rows
    const uint64_t blocks = (n_words + kWordsPerBlock - 1) / kWordsPerBlock;
    *n_out = 0;
    if (blocks == 0) return EBI_OK;
    unsigned long long* counts = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&counts), (2 * blocks + 1) * sizeof(unsigned long long), s);
    if (e == cudaSuccess) {
        unsigned long long* offsets = counts + blocks;
        const uint32_t* m = reinterpret_cast<const uint32_t*>(d_mask);
        mask_block_counts<<<static_cast<uint32_t>(blocks), kThreads, 0, s>>>(m, n_words, n_records, counts);
        count_launch();
        e = cudaGetLastError();
        if (e == cudaSuccess) e = launch_tile_scan(counts, offsets, static_cast<uint32_t>(blocks), s);
        if (e == cudaSuccess) {
            mask_write_rows<<<static_cast<uint32_t>(blocks), kThreads, 0, s>>>(m, n_words, n_records, offsets, d_rows, cap);
            count_launch();
            e = cudaGetLastError();
        }
        unsigned long long total = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&total, offsets + blocks, 8, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        cudaFreeAsync(counts, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        *n_out = total;
    }
    if (e != cudaSuccess) {
        set_last_error(std::string("ebi_rows_from_mask: ") + cudaGetErrorString(e));
        return EBI_E_CUDA;
    }
    if (*n_out > cap) {
        set_last_error("row buffer smaller than the set rows (n_out holds the number needed)");
        return EBI_E_INVALID;
    }
    return EBI_OK;
}

}  // extern "C"
