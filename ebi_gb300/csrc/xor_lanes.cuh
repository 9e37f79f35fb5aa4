// xor_lanes.cuh -- Gorilla, Chimp and Chimp128 chunks decoded one chunk per
// thread, for launches with many chunks (batches, long columns).
//
// Each thread walks its chunk's stream exactly as the reader does
// (decoder/chunk_reader/{gorilla,chimp,chimp_n}.rs): the next record's header
// and payload are read from a three-word window over the big-endian stream,
// and the record's length, window and payload are formed with selects rather
// than branches, so the 32 threads of a warp (32 different chunks) stay
// converged.  Chimp128's ring of the last 128 values is a per-thread array in
// local memory; its slot is the record index mod 128, the same for every
// thread of a warp that decodes in lockstep.  Values go straight to the query
// (NaN end marker, bitmask words, compensated sums, materialize positions).
//
// Compared with the segment-parallel decode (xor_dev.cuh), one record costs a
// few dozen instructions instead of several hundred, but a chunk takes 8,192
// dependent steps: the better choice when there are enough chunks to fill the
// GPU's threads.
#pragma once

#include "bitstream.cuh"
#include "values.cuh"
#include "xor_parse.cuh"

namespace ebi {
namespace {

using namespace xorp;

__device__ __forceinline__ uint64_t be64(const uint64_t* w, uint64_t i) {
    const uint64_t x = __ldg(w + i);
    return (uint64_t(bswap32(static_cast<uint32_t>(x))) << 32) | bswap32(static_cast<uint32_t>(x >> 32));
}

// Bits [base, base + 192) of the file as three big-endian words.
struct BitWindow {
    const uint64_t* f;
    uint64_t w;  // word index of W0
    uint64_t W0, W1, W2;
    __device__ __forceinline__ void init(const uint64_t* file, uint64_t abs_bit) {
        f = file;
        w = abs_bit >> 6;
        W0 = be64(f, w);
        W1 = be64(f, w + 1);
        W2 = be64(f, w + 2);
    }
    // 64 bits at absolute bit a, w * 64 <= a < w * 64 + 128.
    __device__ __forceinline__ uint64_t peek(uint64_t a) const {
        const uint32_t sh = static_cast<uint32_t>(a - (w << 6));
        const uint64_t hi = sh < 64 ? W0 : W1, lo = sh < 64 ? W1 : W2;
        const uint32_t s = sh & 63;
        return s ? (hi << s) | (lo >> (64 - s)) : hi;
    }
    // Moves the window so that it starts at the word of absolute bit a (a >= w * 64).
    __device__ __forceinline__ void advance(uint64_t a) {
        const uint64_t nw = a >> 6;
        if (nw == w) return;
        if (nw == w + 1) {
            W0 = W1;
            W1 = W2;
            W2 = be64(f, nw + 2);
        } else if (nw == w + 2) {
            W0 = W2;
            W1 = be64(f, nw + 1);
            W2 = be64(f, nw + 2);
        } else {
            W0 = be64(f, nw);
            W1 = be64(f, nw + 1);
            W2 = be64(f, nw + 2);
        }
        w = nw;
    }
};

// Per-thread query over one chunk's values, in row order.
struct LaneSink {
    const QueryParams* q;
    KeyPred kp;
    ValAgg agg;
    uint64_t row_off;
    unsigned long long pos;
    uint64_t word_idx;
    uint32_t word;
    int mode;
    bool has_mask, pred_on, store;
    __device__ __forceinline__ void flush() {
        if (word) atomicOr(&q->out_mask[word_idx], word);
        word = 0;
    }
    __device__ __forceinline__ void row(uint64_t i, uint64_t vb) {
        const uint64_t g = row_off + i;
        const bool in = !has_mask || mask_row(q->in_mask, q->n_records, g);
        const bool pass = in && (!pred_on || kp.pass(vb));
        if (!pass) return;
        if (mode == VAL_MATERIALIZE) {
            if (pos < q->out_cap) q->out_vals[pos] = __longlong_as_double(static_cast<long long>(vb));
            ++pos;
            return;
        }
        if (mode == VAL_COUNT) { ++agg.cnt; return; }
        if (store && g < q->n_records) {
            if ((g >> 5) != word_idx) { flush(); word_idx = g >> 5; }
            word |= 1u << (g & 31);
        }
        val_agg_add1(agg, vb);
    }
};

// Decodes chunk c of q in this thread and runs the pass `mode` over it; li
// indexes the pass's per-chunk counts / offsets.
template <int CODEC>
__device__ __noinline__ void xor_lane_chunk(const QueryParams& q, uint32_t li, uint32_t c, int mode,
                                            const unsigned long long* chunk_offsets) {
    const ChunkDesc cd = q.chunks[c];
    ChunkAcc* acc = q.acc + c;
    const bool has_mask = q.in_mask != nullptr;
    bool ok = true;
    if (mode == VAL_SCAN) {
        ok = has_mask ? acc->selected != 0 : (q.chunk_id < 0 || static_cast<uint64_t>(q.chunk_id) == c);
        if (ok && !has_mask) acc->selected = 1;
    } else if (mode == VAL_MATERIALIZE) {
        ok = chunk_offsets[li + 1] != chunk_offsets[li];
    } else if (has_mask) {
        uint32_t any = 0;
        for (uint64_t r = 0; r < cd.n_rows && !any; r += 32) {
            uint32_t w = mask_word(q.in_mask, cd.row_off + r, q.n_records);
            if (cd.n_rows - r < 32) w &= (1u << (cd.n_rows - r)) - 1u;
            any = w;
        }
        ok = any != 0;
    }
    if (ok && (cd.flags & kChunkBadGeometry)) {
        set_status(acc, EBI_E_IO);
        ok = false;
    }
    if (!ok) {
        if (mode == VAL_COUNT) q.tile_counts[li] = 0;
        return;
    }
    LaneSink sink{&q, key_pred(q.pred), val_agg_init(q.op == OP_FILTER_AGG || q.op == OP_AGG ? q.agg : 0u), cd.row_off,
                  mode == VAL_MATERIALIZE ? chunk_offsets[li] : 0ull, 0, 0, mode, has_mask, q.pred_on != 0,
                  mode == VAL_SCAN && q.pred_on && q.out_mask != nullptr};
    const uint64_t B = cd.byte_len * 8;
    const uint64_t a0 = cd.byte_off * 8;  // absolute bit of the chunk's first bit
    uint32_t status = 0;
    uint64_t ring[CODEC == CODEC_CHIMP128 ? 128 : 1];
    if (B < 64) {
        status = EBI_E_UNEXPECTED_END;
    } else {
        BitWindow win;
        win.init(reinterpret_cast<const uint64_t*>(q.file), a0);
        uint64_t v = win.peek(a0);
        uint64_t p = 64;
        uint32_t lead = CODEC == CODEC_GORILLA ? 0u : kNoLead, trail = 0;
        if (CODEC == CODEC_CHIMP128) {
#pragma unroll 1
            for (int k = 0; k < 128; ++k) ring[k] = 0;
            ring[0] = v;
        }
        bool check = true;
        for (uint64_t i = 0;; ++i) {
            if (check && v == kNanBits) break;
            sink.row(i, v);
            win.advance(a0 + p);
            const uint64_t x = win.peek(a0 + p);
            uint32_t hdr, n, shift, e = 0, slot = 0;
            bool from_ring = false;
            if (CODEC == CODEC_GORILLA) {
                const uint32_t b0 = static_cast<uint32_t>(x >> 63), b1 = static_cast<uint32_t>(x >> 62) & 1u;
                const uint32_t l = static_cast<uint32_t>(x >> 57) & 31u, sg = (static_cast<uint32_t>(x >> 51) & 63u) + 1;
                const bool nw = b0 && b1;
                hdr = !b0 ? 1u : (nw ? 13u : 2u);
                n = !b0 ? 0u : (nw ? sg : 64 - lead - trail);
                if (p + 1 > B || (b0 && p + 2 > B) || (nw && p + 13 > B)) e = EBI_E_UNEXPECTED_END;
                else if (nw && l + sg > 64) e = EBI_E_CORRUPT;
                if (nw && !e) { lead = l; trail = 64 - l - sg; }
                shift = trail;
                check = true;
            } else {
                const uint32_t flag = static_cast<uint32_t>(x >> 62);
                constexpr uint32_t hdr1 = CODEC == CODEC_CHIMP128 ? 16u : 9u;
                const uint32_t t1 = static_cast<uint32_t>(x >> (62 - hdr1)) & ((1u << hdr1) - 1u);
                const uint32_t lead1 = lead_decode((t1 >> 6) & 7u);
                const uint32_t sig1 = (t1 & 63u) ? (t1 & 63u) : 64u;
                const uint32_t lead3 = lead_decode(static_cast<uint32_t>(x >> 59) & 7u);
                hdr = flag == 0 ? (CODEC == CODEC_CHIMP128 ? 9u : 2u) : flag == 1 ? 2 + hdr1 : flag == 2 ? 2u : 5u;
                n = flag == 0 ? 0u : flag == 1 ? sig1 : flag == 2 ? 64u - (lead > 64 ? 0u : lead) : 64u - lead3;
                shift = flag == 1 ? 64 - sig1 - lead1 : 0u;
                if (p + 2 > B || (flag != 2 && p + hdr > B)) e = EBI_E_UNEXPECTED_END;
                else if ((flag == 1 && sig1 + lead1 > 64) || (flag == 2 && lead > 64)) e = EBI_E_CORRUPT;
                if (!e) lead = flag == 1 ? lead1 : flag == 3 ? lead3 : lead;
                if (CODEC == CODEC_CHIMP128) {
                    from_ring = flag <= 1;
                    slot = flag == 0 ? static_cast<uint32_t>(x >> 55) & 127u : (t1 >> 9) & 127u;
                    check = flag != 0;
                }
            }
            if (!e && p + hdr + n > B) e = EBI_E_UNEXPECTED_END;
            if (e) {
                status = e;
                break;
            }
            const uint64_t pay = n ? (win.peek(a0 + p + hdr) >> (64 - n)) : 0;
            const uint64_t base = (CODEC == CODEC_CHIMP128 && from_ring) ? ring[slot] : v;
            v = base ^ (pay << shift);
            if (CODEC == CODEC_CHIMP128) ring[(i + 1) & 127] = v;
            p += hdr + n;
        }
    }
    if (status) {
        set_status(acc, status);
        if (mode == VAL_COUNT) q.tile_counts[li] = 0;
        return;
    }
    if (mode == VAL_MATERIALIZE) return;
    if (mode == VAL_COUNT) { q.tile_counts[li] = sink.agg.cnt; return; }
    if (sink.store) sink.flush();
    val_agg_store(acc, sink.agg);
}

}  // namespace
}  // namespace ebi
