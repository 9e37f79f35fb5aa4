// raw_dev.cuh -- Uncompressed chunks: n_rows little-endian f64 values
// (compressor/uncompressed.rs; decoder/chunk_reader/uncompressed.rs).  The
// reader takes exactly number_of_records values and fails with an IO error
// when the chunk is shorter.
//
// One CTA per chunk steps through the chunk blockDim rows at a time: every
// warp reads 32 consecutive values (coalesced; realigned from two aligned words
// when the chunk does not start on an 8-byte boundary) and forms its bitmask
// word with a ballot.  Each thread accumulates its rows in row order and the
// block merges in a fixed tree, so results do not depend on scheduling.
#pragma once

#include "values.cuh"

namespace ebi {
namespace {


__device__ __forceinline__ uint64_t raw_bits(const uint64_t* w, uint32_t sh, uint64_t r) {
    const uint64_t a = w[r];
    return sh ? (a >> sh) | (w[r + 1] << (64 - sh)) : a;
}

// One Uncompressed chunk c by a CTA of kThreads threads; li indexes the
// pass's per-chunk counts / offsets.
template <int kThreads>
__device__ __forceinline__ void raw_chunk(const QueryParams& q, uint32_t li, uint32_t c, int mode,
                                          const unsigned long long* chunk_offsets) {
    __shared__ ValAgg sh_agg[kThreads / 32];
    __shared__ uint32_t sh_scan[kThreads / 32];
    __shared__ int s_ok;
    const ChunkDesc cd = q.chunks[c];
    ChunkAcc* acc = q.acc + c;
    const bool has_mask = q.in_mask != nullptr;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        int ok = 1;
        if (mode == VAL_SCAN) {
            ok = has_mask ? acc->selected != 0 : (q.chunk_id < 0 || static_cast<uint64_t>(q.chunk_id) == c);
            if (ok && !has_mask) acc->selected = 1;
        } else if (mode == VAL_MATERIALIZE) {
            ok = chunk_offsets[li + 1] != chunk_offsets[li];
        }
        // (count pass: a chunk without bitmask rows contributes nothing and raises nothing)
        if (ok && mode != VAL_COUNT && ((cd.flags & kChunkBadGeometry) || uint64_t(cd.n_rows) * 8 > cd.byte_len)) {
            set_status(acc, EBI_E_IO);
            ok = 0;
        }
        s_ok = ok;
    }
    zero_chunk_words(q, cd, c);
    __syncthreads();
    if (!s_ok) {
        if (mode == VAL_COUNT && threadIdx.x == 0) q.tile_counts[li] = 0;
        return;
    }
    const bool readable = !(cd.flags & kChunkBadGeometry) && uint64_t(cd.n_rows) * 8 <= cd.byte_len;
    const uintptr_t addr = reinterpret_cast<uintptr_t>(q.file + cd.byte_off);
    const uint64_t* words = reinterpret_cast<const uint64_t*>(addr & ~uintptr_t(7));
    const uint32_t sh = static_cast<uint32_t>(addr & 7) * 8;
    const bool pred_on = q.pred_on != 0;
    const bool store = mode == VAL_SCAN && pred_on && q.out_mask != nullptr;
    const KeyPred kp = key_pred(q.pred);
    ValAgg agg = val_agg_init(q.op == OP_FILTER_AGG || q.op == OP_AGG ? q.agg : 0u);
    unsigned long long pos = mode == VAL_MATERIALIZE ? chunk_offsets[li] : 0;
    uint32_t count_in_mask = 0;  // count pass over an unreadable chunk: rows the bitmask selects
    for (uint64_t r0 = 0; r0 < cd.n_rows; r0 += kThreads) {
        const uint64_t r = r0 + threadIdx.x;
        const uint64_t g = cd.row_off + r;
        const bool in = r < cd.n_rows && (!has_mask || mask_row(q.in_mask, q.n_records, g));
        if (!readable) {  // block-uniform: only a count pass gets here with an unreadable chunk
            count_in_mask += in;
            continue;
        }
        const uint64_t vb = in ? raw_bits(words, sh, r) : 0;
        const bool pass = in && (!pred_on || kp.pass(vb));
        if (mode == VAL_MATERIALIZE) {
            uint32_t total;
            const uint32_t before = block_excl_scan_u32<kThreads>(pass, sh_scan, &total);
            if (pass && pos + before < q.out_cap) q.out_vals[pos + before] = __longlong_as_double(static_cast<long long>(vb));
            pos += total;
            continue;
        }
        if (store) {
            // rows [g - lane, g - lane + 32): chunks start on any row, so OR into a zeroed mask
            const uint32_t word = __ballot_sync(0xffffffffu, pass && g < q.n_records);
            if (lane == 0 && word) store_mask_word(q.out_mask, g, word, true);
        }
        if (pass) val_agg_add1(agg, vb);
    }
    if (mode == VAL_MATERIALIZE) return;
    const ValAgg a = val_agg_block(agg, sh_agg);
    if (mode == VAL_COUNT) {
        const uint32_t unread = __syncthreads_count(count_in_mask != 0);
        if (threadIdx.x == 0) {
            q.tile_counts[li] = readable ? a.cnt : 0;
            // the Decoder reads the chunk (no bitmask, or one that meets its rows) and fails
            if (!readable && (!has_mask || unread)) set_status(acc, EBI_E_IO);
        }
        return;
    }
    if (threadIdx.x == 0) val_agg_store(acc, a);
}

}  // namespace
}  // namespace ebi
