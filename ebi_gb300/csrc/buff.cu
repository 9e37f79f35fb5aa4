// buff.cu -- BUFF (byte-sliced fixed point) chunks decoded and queried in place.
//
// Chunk layout (compressor/buff.rs:234-307): a 20-byte header (base as two
// u32, row count, bit width `bits`, fractional bits `frac`), then bits/8 byte
// planes, most significant first, each one byte per row and XOR 0x80
// (`flip`), then a tail plane of bits%8 bits per row packed LSB-first.  A row
// decodes to (base + delta) as f64 / 2^frac.
//
// Work split: one CTA of 256 threads per tile of 8192 rows; every thread owns
// 32 consecutive rows, reads their 32 bytes of each plane with three aligned
// 16-byte loads realigned in registers (the file sits in HBM unmodified, so
// planes start at arbitrary byte addresses), and forms the 32 deltas.  The
// range / equality predicates are compiled per chunk into the fixed-point
// domain exactly as the reference's in-situ filters decide them
// (buff/filter_cmp.rs:299-451, buff/filter_eq.rs:74-200), including their
// shortcuts.  Sums are exact u64 sums of deltas (buff/sum.rs:60-119); min
// and max are exact via the deltas (buff/min_max.rs).
#include "buff_common.cuh"
#include "buff_tile.cuh"
#include "tma.cuh"
#include "fold.cuh"
#include <climits>

namespace ebi {
namespace {
using namespace buff;

__global__ void __launch_bounds__(kTileThreads) buff_query_kernel(QueryParams q, uint32_t tile_base) {
    __shared__ BuffCtx k;
    __shared__ BlockRed red;
    const Tile t = q.tiles[tile_base + blockIdx.x];
    if (threadIdx.x == 0) buff_setup(q, t.chunk, q.in_mask != nullptr, k);
    __syncthreads();
    if (k.ok && k.bits > 32) buff_query_dispatch<unsigned long long>(q, k, t.chunk, blockIdx.x, t.begin, red);
    else buff_query_dispatch<uint32_t>(q, k, t.chunk, blockIdx.x, t.begin, red);
}

// Materialize pass 1: rows of the bitmask per tile.  A chunk is read (and its
// header errors reported) only when the bitmask selects some of its rows.
__global__ void __launch_bounds__(kTileThreads) buff_count_kernel(QueryParams q, uint32_t tile_base) {
    __shared__ unsigned long long wsum[kTileWarps];
    __shared__ BuffCtx k;
    const Tile t = q.tiles[tile_base + blockIdx.x];
    const ChunkDesc cd = q.chunks[t.chunk];
    const uint32_t r0 = t.begin + threadIdx.x * 32;
    uint32_t cnt = 0;
    if (r0 < cd.n_rows) {
        const uint32_t left = cd.n_rows - r0;
        const uint32_t valid = left >= 32 ? ~0u : ((1u << left) - 1u);
        cnt = __popc(mask_word(q.in_mask, cd.row_off + r0, q.n_records) & valid);
    }
    const unsigned long long w = warp_sum<unsigned long long>(cnt);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = w;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long tot = 0;
        for (int i = 0; i < kTileWarps; ++i) tot += wsum[i];
        q.tile_counts[blockIdx.x] = tot;
        if (tot) buff_setup(q, t.chunk, false, k);
    }
}

// Materialization: the decoded values of the selected rows, in row order.
// Each warp owns 1,024 consecutive rows of the tile and a contiguous run of
// the output.  Its lanes form the deltas of their 32 rows each and put the
// selected ones, compacted, into a padded shared-memory stage (one pad entry
// per 32, so both the per-lane writes and the per-row reads are free of bank
// conflicts); the warp then reads the stage back in output order, turns each
// delta into its double and writes the run as consecutive doubles, 256 bytes
// per store instruction.
constexpr int kMatStage = 32 * 33;  // entries per warp
// stage bytes: 64-bit deltas (WIDE) or 32-bit
constexpr size_t mat_smem(bool wide) { return size_t(kTileWarps) * kMatStage * (wide ? 8 : 4); }

// The warp's run: staged entry j (padded position j + j / 32) becomes output
// wbase + j.  SMALL: every fixed value of the chunk fits an int32.
template <bool SMALL, typename D>
__device__ __forceinline__ void mat_write(const QueryParams& q, const BuffCtx& k, const D* st,
                                          unsigned long long wbase, unsigned int wcount, int lane) {
    const unsigned long long base = static_cast<unsigned long long>(k.base);
    auto value = [&](D delta) -> double {
        if constexpr (SMALL)
            return fixed32_to_f64(static_cast<int32_t>(static_cast<uint32_t>(base) + static_cast<uint32_t>(delta)), k.frac);
        else
            return fixed_to_f64(static_cast<long long>(base + static_cast<unsigned long long>(delta)), k.frac, k.scale);
    };
    if (wcount == 1024 && wbase + 1024 <= q.out_cap) {
        double* o = q.out_vals + wbase + lane;
        const D* sp = st + lane;
#pragma unroll 8
        for (int it = 0; it < 32; ++it) o[32 * it] = value(sp[33 * it]);
        return;
    }
#pragma unroll 4
    for (unsigned int j = lane; j < wcount; j += 32) {
        const unsigned long long pos = wbase + j;
        if (pos < q.out_cap) q.out_vals[pos] = value(st[j + (j >> 5)]);
    }
}

template <int TB, typename D>
__device__ void buff_mat_tile(const QueryParams& q, const BuffCtx& k, uint32_t begin,
                              const unsigned long long* tile_offsets, unsigned long long base_row,
                              unsigned int* warp_tot, unsigned long long* stage) {
    const uint32_t r0 = begin + threadIdx.x * 32;
    const bool has_mask = q.in_mask != nullptr;
    uint32_t sel = 0;
    D d[32];
    if (r0 < k.n && k.ok) {
        const uint32_t left = k.n - r0;
        const uint32_t valid = left >= 32 ? ~0u : ((1u << left) - 1u);
        sel = has_mask ? (mask_word(q.in_mask, k.row_off + r0, q.n_records) & valid) : valid;
        if (sel) load_deltas<TB, D>(k, r0, k.np_load, k.np, k.load_tail, d);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned int wcount, off;
    unsigned long long wbase;
    if (has_mask) {
        // block-exclusive prefix of the per-thread counts (has_mask is the same for the whole block)
        const unsigned int cnt = __popc(sel);
        unsigned int inc = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned int y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) warp_tot[wid] = inc;
        __syncthreads();
        wcount = __shfl_sync(0xffffffffu, inc, 31);
        if (wcount == 0) return;  // warp-uniform
        unsigned int before = 0;
        for (int w = 0; w < wid; ++w) before += warp_tot[w];
        wbase = tile_offsets[blockIdx.x] + before;
        off = inc - cnt;
    } else {
        // every row of the warp's 1,024 inside the chunk, in order: lanes before
        // the last holding rows are full
        const uint32_t w0 = begin + uint32_t(wid) * 1024u;
        wcount = k.ok && w0 < k.n ? (k.n - w0 < 1024u ? k.n - w0 : 1024u) : 0u;
        if (wcount == 0) return;  // warp-uniform
        wbase = k.row_off + w0 - base_row;
        off = uint32_t(lane) * 32u;
    }
    D* st = reinterpret_cast<D*>(stage) + wid * kMatStage;
    if (sel == ~0u && off == uint32_t(lane) * 32u) {
        // a full lane at its own place: rows lane*32 + i go to entries lane*33 + i
        D* p = st + lane * 33;
#pragma unroll
        for (int i = 0; i < 32; ++i) p[i] = d[i];
    } else {
#pragma unroll
        for (int i = 0; i < 32; ++i) {
            if ((sel >> i) & 1u) {
                st[off + (off >> 5)] = d[i];
                ++off;
            }
        }
    }
    __syncwarp();
    if (k.fits32 && sizeof(D) == 4) mat_write<true, D>(q, k, st, wbase, wcount, lane);
    else mat_write<false, D>(q, k, st, wbase, wcount, lane);
}

template <typename D>
__device__ void buff_mat_dispatch(const QueryParams& q, const BuffCtx& k, uint32_t begin,
                                  const unsigned long long* offs, unsigned long long base_row, unsigned int* wt,
                                  unsigned long long* st) {
    switch (k.ok ? k.tb : 0) {
        case 0: buff_mat_tile<0, D>(q, k, begin, offs, base_row, wt, st); break;
        case 1: buff_mat_tile<1, D>(q, k, begin, offs, base_row, wt, st); break;
        case 2: buff_mat_tile<2, D>(q, k, begin, offs, base_row, wt, st); break;
        case 3: buff_mat_tile<3, D>(q, k, begin, offs, base_row, wt, st); break;
        case 4: buff_mat_tile<4, D>(q, k, begin, offs, base_row, wt, st); break;
        case 5: buff_mat_tile<5, D>(q, k, begin, offs, base_row, wt, st); break;
        case 6: buff_mat_tile<6, D>(q, k, begin, offs, base_row, wt, st); break;
        default: buff_mat_tile<7, D>(q, k, begin, offs, base_row, wt, st); break;
    }
}

// WIDE: some readable chunk of the column is more than 32 bits wide (64-bit
// deltas); the narrow build stages 32-bit deltas (33 KB a CTA) and fits four
// CTAs per SM.
// quiet: no chunk the pass reads can raise, so the chunks' accumulators are
// left untouched and no fold follows.
template <bool WIDE>
__global__ void __launch_bounds__(kTileThreads, WIDE ? 2 : 4) buff_materialize_kernel(
    QueryParams q, uint32_t tile_base, const unsigned long long* tile_offsets, unsigned long long base_row,
    bool quiet) {
    extern __shared__ unsigned long long mat_stage[];
    __shared__ BuffCtx k;
    __shared__ unsigned int warp_tot[kTileWarps];
    const uint32_t tile = tile_base + blockIdx.x;
    const Tile t = q.tiles[tile];
    if (threadIdx.x == 0) {
        // with a bitmask, tiles without selected rows were counted as 0 and
        // their chunk may be unselected: only tiles that select rows read
        buff_setup(q, t.chunk, false, k, !quiet);
        if (q.in_mask && tile_offsets[blockIdx.x + 1] == tile_offsets[blockIdx.x]) k.ok = 0;
    }
    __syncthreads();
    if constexpr (WIDE) {
        if (k.ok && k.bits > 32) {
            buff_mat_dispatch<unsigned long long>(q, k, t.begin, tile_offsets, base_row, warp_tot, mat_stage);
            return;
        }
    }
    buff_mat_dispatch<uint32_t>(q, k, t.begin, tile_offsets, base_row, warp_tot, mat_stage);
}


}  // namespace

TileMap buff_tiles(const std::vector<ChunkDesc>& chunks) {
    TileMap m;
    m.first_tile.reserve(chunks.size() + 1);
    for (uint32_t c = 0; c < chunks.size(); ++c) {
        m.first_tile.push_back(static_cast<uint32_t>(m.tiles.size()));
        const uint32_t n = chunks[c].n_rows;
        uint32_t b = 0;
        do { m.tiles.push_back(Tile{c, b}); b += kBuffTileRows; } while (b < n);
    }
    m.first_tile.push_back(static_cast<uint32_t>(m.tiles.size()));
    return m;
}

cudaError_t launch_buff_query(const QueryParams& q, uint32_t tile_begin, uint32_t n_tiles, cudaStream_t s) {
    if (n_tiles == 0) return cudaSuccess;
    buff_query_kernel<<<n_tiles, kTileThreads, 0, s>>>(q, tile_begin);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_buff_count(const QueryParams& q, uint32_t tile_begin, uint32_t n_tiles, cudaStream_t s) {
    if (n_tiles == 0) return cudaSuccess;
    buff_count_kernel<<<n_tiles, kTileThreads, 0, s>>>(q, tile_begin);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_buff_materialize(const QueryParams& q, uint32_t tile_begin, uint32_t n_tiles,
                                    const unsigned long long* tile_offsets, uint64_t base_row, bool wide,
                                    bool quiet, cudaStream_t s) {
    if (n_tiles == 0) return cudaSuccess;
    const void* fn = wide ? reinterpret_cast<const void*>(buff_materialize_kernel<true>)
                          : reinterpret_cast<const void*>(buff_materialize_kernel<false>);
    const size_t smem = mat_smem(wide);
    const cudaError_t e = allow_dynamic_smem(fn, smem);
    if (e != cudaSuccess) return e;
    if (wide) buff_materialize_kernel<true><<<n_tiles, kTileThreads, smem, s>>>(q, tile_begin, tile_offsets, base_row, quiet);
    else buff_materialize_kernel<false><<<n_tiles, kTileThreads, smem, s>>>(q, tile_begin, tile_offsets, base_row, quiet);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ebi
