// rle_dev.cuh -- RLE chunks (compressor/run_length.rs:49-117): a u64 field count,
// then packed 9-byte fields (u8 run length, f64 little-endian value).  The
// reader expands every run in order (decoder/chunk_reader/run_length.rs:68-91);
// row i of the chunk is global row logical_offset + i, and the default
// operators (decoder/query.rs:14-154) run over the expanded rows.
//
// One CTA per chunk walks its fields in batches of 1024 (4 per thread): a
// block scan of the run lengths gives every field's first row; each field
// then evaluates the predicate once for its whole run and sets the run's
// bitmask bits with at most ceil(255 / 32) + 1 word operations.
#pragma once

#include "values.cuh"

namespace ebi {
namespace {

constexpr int kRleThreads = 256;
constexpr int kRlePer = 4;

__device__ __forceinline__ double field_value(const uint8_t* f) {
    return __longlong_as_double(static_cast<long long>(load_u64_unaligned(f + 1)));
}

// One RLE chunk c by a CTA of kRleThreads threads; li indexes the pass's
// per-chunk counts / offsets.
__device__ __forceinline__ void rle_chunk(const QueryParams& q, uint32_t li, uint32_t c, int mode,
                                          const unsigned long long* chunk_offsets) {
    constexpr int kThreads = kRleThreads;
    __shared__ uint32_t sh_scan[kThreads / 32];
    __shared__ ValAgg sh_agg[kThreads / 32];
    __shared__ int s_ok;
    const ChunkDesc cd = q.chunks[c];
    const bool has_mask = q.in_mask != nullptr;
    ChunkAcc* acc = q.acc + c;
    if (threadIdx.x == 0) {
        int ok = 1;
        if (mode == VAL_SCAN) {
            ok = has_mask ? acc->selected != 0 : (q.chunk_id < 0 || static_cast<uint64_t>(q.chunk_id) == c);
            if (ok && !has_mask) acc->selected = 1;
        } else if (mode == VAL_MATERIALIZE) {
            ok = chunk_offsets[li + 1] != chunk_offsets[li];
        } else if (has_mask) {
            // the Decoder reads a chunk only when the bitmask meets its rows
            uint32_t any = 0;
            for (uint64_t r = 0; r < cd.n_rows && !any; r += 32) {
                uint32_t w = mask_word(q.in_mask, cd.row_off + r, q.n_records);
                if (cd.n_rows - r < 32) w &= (1u << (cd.n_rows - r)) - 1u;
                any = w;
            }
            ok = any != 0;
        }
        if (ok) {
            if (cd.flags & kChunkBadGeometry) { set_status(acc, EBI_E_IO); ok = 0; }
            else if (cd.byte_len < 8) { set_status(acc, EBI_E_IO); ok = 0; }
            else if (load_u64_unaligned(q.file + cd.byte_off) > (cd.byte_len - 8) / 9) {
                set_status(acc, EBI_E_IO);  // read_exact past the chunk
                ok = 0;
            }
        }
        s_ok = ok;
        if (mode == VAL_COUNT && !ok) q.tile_counts[li] = 0;
    }
    zero_chunk_words(q, cd, c);
    __syncthreads();
    if (!s_ok) return;
    const uint8_t* base = q.file + cd.byte_off;
    const uint64_t nf = load_u64_unaligned(base);
    const uint8_t* fields = base + 8;
    const bool pred_on = q.pred_on != 0;
    const bool store = mode == VAL_SCAN && pred_on && q.out_mask;
    const KeyPred kp = key_pred(q.pred);
    ValAgg agg = val_agg_init(q.op == OP_FILTER_AGG || q.op == OP_AGG ? q.agg : 0u);
    unsigned long long out_pos = mode == VAL_MATERIALIZE ? chunk_offsets[li] : 0;
    uint64_t carry_row = 0;
    for (uint64_t b0 = 0; b0 < nf; b0 += (kRleThreads * kRlePer)) {
        const uint64_t f0 = b0 + uint64_t(threadIdx.x) * kRlePer;
        uint32_t run[kRlePer];
        double val[kRlePer];
        uint32_t rows = 0;
#pragma unroll
        for (int k = 0; k < kRlePer; ++k) {
            const bool in = f0 + k < nf;
            run[k] = in ? fields[9 * (f0 + k)] : 0u;
            val[k] = in ? field_value(fields + 9 * (f0 + k)) : 0.0;
            rows += run[k];
        }
        uint32_t total;
        const uint32_t first = block_excl_scan_u32<kThreads>(rows, sh_scan, &total);
        uint64_t r = carry_row + first;  // chunk row of this thread's first field
        uint32_t sel_rows[kRlePer];
#pragma unroll
        for (int k = 0; k < kRlePer; ++k) {
            const uint64_t g0 = cd.row_off + r;  // global rows [g0, g0 + run)
            const bool pass = !pred_on || kp.pass(static_cast<uint64_t>(__double_as_longlong(val[k])));
            uint32_t n_sel = 0;
            if (run[k] && pass) {
                if (!has_mask) n_sel = run[k];
                if (has_mask || store) {
                    for (uint64_t g = g0; g < g0 + run[k];) {
                        const uint64_t w = g >> 5;
                        const uint64_t wend = (w + 1) << 5;
                        const uint64_t stop = g0 + run[k] < wend ? g0 + run[k] : wend;
                        uint32_t bits = range_bits(static_cast<uint32_t>(g & 31), static_cast<uint32_t>(stop - (w << 5)));
                        // rows at or past n_records are never in a bitmask
                        if ((w << 5) >= q.n_records) bits = 0;
                        else if (q.n_records - (w << 5) < 32) bits &= (1u << (q.n_records - (w << 5))) - 1u;
                        if (has_mask) {
                            if (bits) bits &= q.in_mask[w];
                            n_sel += __popc(bits);
                        }
                        if (store && bits) atomicOr(&q.out_mask[w], bits);
                        g = wend;
                    }
                }
            }
            sel_rows[k] = n_sel;
            if (mode == VAL_SCAN) val_agg_add(agg, val[k], n_sel);
            else agg.cnt += n_sel;
            r += run[k];
        }
        if (mode == VAL_MATERIALIZE) {
            uint32_t mine = 0;
#pragma unroll
            for (int k = 0; k < kRlePer; ++k) mine += sel_rows[k];
            uint32_t btotal;
            const uint32_t before = block_excl_scan_u32<kThreads>(mine, sh_scan, &btotal);
            unsigned long long pos = out_pos + before;
#pragma unroll
            for (int k = 0; k < kRlePer; ++k) {
                for (uint32_t i = 0; i < sel_rows[k]; ++i, ++pos)
                    if (pos < q.out_cap) q.out_vals[pos] = val[k];
            }
            out_pos += btotal;
        }
        carry_row += total;
        __syncthreads();
    }
    if (mode == VAL_MATERIALIZE) return;
    const ValAgg a = val_agg_block(agg, sh_agg);
    if (threadIdx.x != 0) return;
    if (mode == VAL_COUNT) q.tile_counts[li] = a.cnt;
    else val_agg_store(acc, a);
}

}  // namespace
}  // namespace ebi
