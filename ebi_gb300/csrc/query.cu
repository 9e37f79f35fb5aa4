// query.cu -- kernels shared by every codec: chunk selection, tile scans and
// the folds of per-chunk results into the query's result (Decoder's
// `result += chunk`, `result = result.min(chunk)`, `result = result.max(chunk)`,
// api/decoder.rs:323-439; finalize.cuh).
#include <climits>

#include "internal.h"
#include "finalize.cuh"

namespace ebi {
namespace {

__global__ void acc_init_kernel(ChunkAcc* acc, uint32_t n) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        ChunkAcc a = {};
        a.dmin = ~0ull;
        a.fmin = __longlong_as_double(0x7ff0000000000000ll);
        a.fmax = __longlong_as_double(static_cast<long long>(0xfff0000000000000ull));
        acc[c] = a;
    }
}

// acc[c].selected for chunk c = blockIdx.x (grid-stride): the chunk passes
// chunk_id and the input bitmask intersects its rows (api/decoder.rs:258-268).
__global__ void select_chunks_kernel(QueryParams q) {
    __shared__ int any;
    for (uint32_t c = blockIdx.x; c < q.n_chunks; c += gridDim.x) {
        if (threadIdx.x == 0) any = 0;
        __syncthreads();
        const ChunkDesc cd = q.chunks[c];
        const bool id_ok = q.chunk_id < 0 || static_cast<uint64_t>(q.chunk_id) == c;
        if (id_ok) {
            // logical_record_range_u32: rows [row_off, row_off + n_rows)
            for (uint64_t r = uint64_t(threadIdx.x) * 32; r < cd.n_rows && !any; r += uint64_t(blockDim.x) * 32) {
                const uint64_t left = cd.n_rows - r;
                uint32_t w = mask_word(q.in_mask, cd.row_off + r, q.n_records);
                if (left < 32) w &= (1u << left) - 1u;
                if (w) any = 1;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) q.acc[c].selected = static_cast<uint32_t>(id_ok && any);
        __syncthreads();
    }
}

// Exclusive scan of tile counts (one CTA; tiles are few thousands).
__global__ void tile_scan_kernel(const unsigned long long* counts, unsigned long long* offsets, uint32_t n) {
    __shared__ unsigned long long wsum[32];
    __shared__ unsigned long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (uint32_t base = 0; base < n; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const unsigned long long v = i < n ? counts[i] : 0;
        unsigned long long inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) wsum[wid] = inc;
        __syncthreads();
        if (wid == 0) {
            unsigned long long x = lane < static_cast<int>(blockDim.x >> 5) ? wsum[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            wsum[lane] = x;  // inclusive warp prefix
        }
        __syncthreads();
        const unsigned long long before = (wid ? wsum[wid - 1] : 0) + carry;
        if (i < n) offsets[i] = before + inc - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + inc;
        __syncthreads();
    }
    if (threadIdx.x == 0) offsets[n] = carry;
}

__global__ void __launch_bounds__(kFinThreads) finalize_kernel(QueryParams q, QueryResult* res) {
    finalize_chunks(q, res);
}

// The non-BUFF fold over a grid (more than eight slices): warp w of CTA b folds slice 8b + w into
// parts[slice]; the last CTA to finish (a ticket in the counter behind the
// slices) sums the slices into *res and puts the counter back to 0.
constexpr int kSliceWarps = 8;

__global__ void __launch_bounds__(kSliceWarps * 32) fold_values_kernel(QueryParams q, ValPart* parts,
                                                                       QueryResult* res) {
    __shared__ uint32_t last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t S = value_slices(q.n_chunks);
    unsigned int* counter = fold_counters(parts, S);
    const uint32_t s = blockIdx.x * kSliceWarps + wid;
    if (s < S) {
        const ValPart p = slice_fold(q, s);
        if (lane == 0) {
            parts[s] = p;
            __threadfence();
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last || wid) return;
    __threadfence();
    fold_parts_warp(parts, S, res);
    if (lane == 0) *counter = 0;
}

}  // namespace

cudaError_t launch_acc_init(ChunkAcc* acc, uint32_t n, cudaStream_t s) {
    if (!n) return cudaSuccess;
    acc_init_kernel<<<(n + 255) / 256, 256, 0, s>>>(acc, n);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_select_chunks(const QueryParams& q, cudaStream_t s) {
    if (!q.n_chunks) return cudaSuccess;
    const uint32_t grid = q.n_chunks < 4096 ? q.n_chunks : 4096;
    select_chunks_kernel<<<grid, 256, 0, s>>>(q);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_tile_scan(const unsigned long long* counts, unsigned long long* offsets, uint32_t n,
                             cudaStream_t s) {
    tile_scan_kernel<<<1, 1024, 0, s>>>(counts, offsets, n);
    count_launch();
    return cudaGetLastError();
}

// Up to 8 slices: one CTA, a warp per slice, the slices summed through
// shared memory (no global round trips between the two steps).  More slices
// take the grid: one SM folding 32 slices measured slower than four.
constexpr uint32_t kCtaSlices = 8;
__global__ void __launch_bounds__(kCtaSlices * 32) fold_values_cta_kernel(QueryParams q, QueryResult* res) {
    __shared__ ValPart sp[kCtaSlices];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t S = value_slices(q.n_chunks);
    if (static_cast<uint32_t>(wid) < S) {
        const ValPart p = slice_fold(q, wid);
        if (lane == 0) sp[wid] = p;
    }
    __syncthreads();
    if (wid) return;
    const bool have = static_cast<uint32_t>(lane) < S;
    const uint32_t tq = __reduce_max_sync(0xffffffffu, have ? sp[lane].top : 0u);
    ValTotal t = val_total_rest();
    if (have) val_total_add(t, sp[lane], tq);
    t = val_total_warp(t);
    if (lane == 0) *res = val_total_result(t, tq);
}

cudaError_t launch_finalize(const QueryParams& q, QueryResult* res, ValPart* parts, cudaStream_t s) {
    const uint32_t S = value_slices(q.n_chunks);
    if (q.scheme == EBI_BUFF) {
        finalize_kernel<<<1, kFinThreads, 0, s>>>(q, res);
    } else if (S <= kCtaSlices) {
        fold_values_cta_kernel<<<1, S ? S * 32 : 32, 0, s>>>(q, res);
    } else {
        if (!parts) return cudaErrorInvalidValue;
        const uint32_t grid = S ? (S + kSliceWarps - 1) / kSliceWarps : 1;
        fold_values_kernel<<<grid, kSliceWarps * 32, 0, s>>>(q, parts, res);
    }
    count_launch();
    return cudaGetLastError();
}

}  // namespace ebi
