// rle_dev.cuh -- RLE chunks (compressor/run_length.rs:49-117): a u64 field count,
// then packed 9-byte fields (u8 run length, f64 little-endian value).  The
// reader expands every run in order (decoder/chunk_reader/run_length.rs:68-91);
// row i of the chunk is global row logical_offset + i, and the default
// operators (decoder/query.rs:14-154) run over the expanded rows.
//
// One warp per chunk (rle_chunk_warp); the field bytes of each step are
// staged in shared memory by coalesced 16-byte loads first (9-byte fields read
// in place would touch ~18 sectors per warp load).
#pragma once

#include "values.cuh"

namespace ebi {
namespace {

constexpr int kRlePer = 6;
constexpr uint32_t kRleStep = 32 * kRlePer;  // fields per warp step
constexpr uint32_t kRleWords = 256;          // bitmap words per warp: chunks up to 8,192 rows

// A warp's shared memory: the chunk's bitmap and one step's field bytes (the
// 16-byte words that cover them, plus slack for the last value's second word).
struct RleWarpSmem {
    uint32_t bits[kRleWords];
    alignas(16) uint8_t stage[(kRleStep * 9 + 30) / 16 * 16 + 16];
};

// One RLE chunk c by one warp; li indexes the pass's per-chunk counts /
// offsets.  Fields go 32 * kRlePer at a time (kRlePer consecutive fields per
// lane): a warp scan of the run lengths gives every field's first row; each
// field evaluates the predicate once for its run and sets the run's bitmask
// bits with at most ceil(255 / 32) + 1 word operations, into the warp's
// bitmap in shared memory (kRleWords words) when the chunk owns its words
// (q.own_words) and fits, which then go out as whole words; else into the
// output by atomicOr.  A warp per chunk keeps every step on shuffles: no
// CTA barrier, and as many chunks in flight as warps fit.
__device__ __forceinline__ void rle_chunk_warp(const QueryParams& q, uint32_t li, uint32_t c, int mode,
                                               const unsigned long long* chunk_offsets, RleWarpSmem* sm) {
    const int lane = threadIdx.x & 31;
    const ChunkDesc cd = q.chunks[c];
    const bool has_mask = q.in_mask != nullptr;
    ChunkAcc* acc = q.acc + c;
    int ok = 1;
    if (lane == 0) {
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
        if (mode == VAL_COUNT && !ok) q.tile_counts[li] = 0;
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    const bool pred_on = q.pred_on != 0;
    const bool store = mode == VAL_SCAN && pred_on && q.out_mask;
    // the chunk's words of the output bitmask (the last chunk's run to the mask's end)
    const uint64_t mend = ((q.n_records + 63) >> 6) * 2;
    const uint64_t gw0 = min(cd.row_off >> 5, mend);
    const uint64_t gw1 = c + 1 == q.n_chunks ? mend : min((cd.row_off + cd.n_rows + 31) >> 5, mend);
    uint32_t* sbits = sm->bits;
    const bool local = ok && store && q.own_words && gw1 - gw0 <= kRleWords;
    if (q.zero_out && !local) {
        for (uint64_t w = gw0 + lane; w < gw1; w += 32) q.out_mask[w] = 0u;
        __syncwarp();  // before this warp's ORs into the same words
    }
    if (!ok) return;
    if (local) {
        for (uint32_t w = lane; w < kRleWords; w += 32) sbits[w] = 0u;
        __syncwarp();
    }
    const uint8_t* base = q.file + cd.byte_off;
    const uint64_t nf = load_u64_unaligned(base);
    const uint8_t* fields = base + 8;
    const KeyPred kp = key_pred(q.pred);
    ValAgg agg = val_agg_init(q.op == OP_FILTER_AGG || q.op == OP_AGG ? q.agg : 0u);
    unsigned long long out_pos = mode == VAL_MATERIALIZE ? chunk_offsets[li] : 0;
    uint64_t carry_row = 0;
    // Without an input bitmask, a chunk that owns its words marks only where
    // the predicate's outcome changes: a toggle bit at the first row of every
    // run whose outcome differs from the last non-empty run before it (and at
    // the end of the chunk's rows if the last one passes); a prefix XOR over
    // the words then gives the bitmask.
    const bool toggles = local && !has_mask;
    uint32_t prev_pass = 0;  // outcome of the last non-empty run so far (warp-uniform)
    for (uint64_t b0 = 0; b0 < nf; b0 += kRleStep) {
        // the step's fields [b0, b0 + kRleStep) into shared memory (the file
        // allocation is 16-byte aligned and padded past its end)
        const uint8_t* s0 = fields + 9 * b0;
        const uint64_t nb = 9 * min(uint64_t(kRleStep), nf - b0);
        const uint8_t* a0 = reinterpret_cast<const uint8_t*>(reinterpret_cast<uintptr_t>(s0) & ~uintptr_t(15));
        const uint32_t skew = static_cast<uint32_t>(s0 - a0);
        const uint32_t n16 = static_cast<uint32_t>((skew + nb + 15) >> 4);
        __syncwarp();  // the previous step's fields are read
        for (uint32_t i = lane; i < n16; i += 32)
            reinterpret_cast<uint4*>(sm->stage)[i] = ldg16(a0 + 16 * i);
        __syncwarp();
        const uint64_t f0 = b0 + uint64_t(lane) * kRlePer;
        uint32_t run[kRlePer];
        double val[kRlePer];
        uint32_t rows = 0;
#pragma unroll
        for (int k = 0; k < kRlePer; ++k) {
            const bool in = f0 + k < nf;
            const uint32_t o = skew + 9 * (lane * kRlePer + k);  // the field's byte in the stage
            run[k] = in ? sm->stage[o] : 0u;
            uint64_t vb = 0;
            if (in) {
                const uint32_t p = o + 1, sh = (p & 7) * 8;
                const uint64_t* w = reinterpret_cast<const uint64_t*>(sm->stage + (p & ~7u));
                vb = sh ? (w[0] >> sh) | (w[1] << (64 - sh)) : w[0];
            }
            val[k] = __longlong_as_double(static_cast<long long>(vb));
            rows += run[k];
        }
        uint32_t incl = rows;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        uint64_t r = carry_row + (incl - rows);  // chunk row of this lane's first field
        uint32_t sel_rows[kRlePer];
        uint32_t e = prev_pass;  // toggles: the outcome before this lane's first field
        if (toggles) {
            // last non-empty run among this lane's fields, then among the lanes before it
            uint32_t hv = 0;  // bit 1: a non-empty run, bit 0: its outcome
#pragma unroll
            for (int k = 0; k < kRlePer; ++k)
                if (run[k]) hv = 2u | (!pred_on || kp.pass(static_cast<uint64_t>(__double_as_longlong(val[k]))) ? 1u : 0u);
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, hv, o);
                if (lane >= o && !(hv & 2u)) hv = y;
            }
            const uint32_t before = __shfl_up_sync(0xffffffffu, hv, 1);
            if (lane > 0 && (before & 2u)) e = before & 1u;
            const uint32_t last = __shfl_sync(0xffffffffu, hv, 31);
            if (last & 2u) prev_pass = last & 1u;
        }
#pragma unroll
        for (int k = 0; k < kRlePer; ++k) {
            const uint64_t g0 = cd.row_off + r;  // global rows [g0, g0 + run)
            const bool pass = !pred_on || kp.pass(static_cast<uint64_t>(__double_as_longlong(val[k])));
            uint32_t n_sel = 0;
            if (toggles && run[k]) {
                if ((pass ? 1u : 0u) != e && r < 32u * kRleWords)
                    atomicXor(&sbits[r >> 5], 1u << (r & 31));
                e = pass ? 1u : 0u;
            }
            if (run[k] && pass) {
                if (!has_mask) n_sel = run[k];
                if (has_mask || (store && !toggles)) {
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
                        if (store && bits) {
                            // a chunk that owns its words decodes no row past them
                            if (local && w >= gw0 && w - gw0 < kRleWords) atomicOr(&sbits[w - gw0], bits);
                            else atomicOr(&q.out_mask[w], bits);
                        }
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
            uint32_t mi = mine;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, mi, o);
                if (lane >= o) mi += y;
            }
            unsigned long long pos = out_pos + (mi - mine);
#pragma unroll
            for (int k = 0; k < kRlePer; ++k) {
                for (uint32_t i = 0; i < sel_rows[k]; ++i, ++pos)
                    if (pos < q.out_cap) q.out_vals[pos] = val[k];
            }
            out_pos += __shfl_sync(0xffffffffu, mi, 31);
        }
        carry_row += total;
    }
    if (toggles) {
        // the last run's outcome ends at the chunk's last decoded row
        if (lane == 0 && prev_pass && carry_row < 32u * kRleWords)
            atomicXor(&sbits[carry_row >> 5], 1u << (carry_row & 31));
        __syncwarp();
        // prefix XOR: lane l takes words [8l, 8l + 8), the carry in is the
        // parity of every toggle in the words before them
        uint32_t x[kRleWords / 32], par = 0;
#pragma unroll
        for (int j = 0; j < int(kRleWords / 32); ++j) {
            x[j] = sbits[(kRleWords / 32) * lane + j];
            par ^= __popc(x[j]) & 1u;
        }
        uint32_t pi = par;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, pi, o);
            if (lane >= o) pi ^= y;
        }
        uint32_t carry = pi ^ par;
        __syncwarp();
#pragma unroll
        for (int j = 0; j < int(kRleWords / 32); ++j) {
            uint32_t y = x[j];
            y ^= y << 1;
            y ^= y << 2;
            y ^= y << 4;
            y ^= y << 8;
            y ^= y << 16;
            sbits[(kRleWords / 32) * lane + j] = carry ? ~y : y;
            carry ^= __popc(x[j]) & 1u;
        }
    }
    if (local) {
        __syncwarp();
        for (uint64_t w = gw0 + lane; w < gw1; w += 32) q.out_mask[w] = sbits[w - gw0];
    }
    if (mode == VAL_MATERIALIZE) return;
    const ValAgg a = val_agg_warp(agg);
    if (lane != 0) return;
    if (mode == VAL_COUNT) q.tile_counts[li] = a.cnt;
    else val_agg_store(acc, a);
}

}  // namespace
}  // namespace ebi
