// gorilla_dev.cuh -- Gorilla chunks decoded and queried by one warp per chunk.
//
// Format (decoder/chunk_reader/gorilla.rs:90-157; encoder compressor/gorilla.rs:118-190):
// 64 raw bits, then per value '0' (repeat), '10' + payload in the inherited
// window (significant bits = 64 - lead - trail), or '11' + 5-bit leading +
// 6-bit (significant - 1) + payload.  The stream ends at the first value
// equal to f64::NAN's bits; a read past the chunk raises UnexpectedEndOfChunk.
//
// The warp follows the stream exactly, several records per step:
//   * a '0' run: the count of leading zero bits at the cursor is the number of
//     consecutive repeats (up to 32 per step);
//   * a '10' run: with the window fixed, records sit at a fixed stride of
//     2 + significant bits.  Lane i checks that record i of the stride still
//     starts with '10' and fits in the chunk; the ballot's leading ones say how
//     many records are confirmed, each lane extracts its payload and a
//     warp-shuffle prefix XOR (seeded with the previous value) gives the values;
//   * a '11' record (new window) is one step.
// On the bench series over 99 % of the records are '10' in a handful of
// windows, so an 8,192-value chunk takes a few hundred warp steps.  Each
// step's values go straight to the query: NaN end check, bitmask ballot,
// per-lane compensated sums, materialize positions from the ballot.
//
// Every step's read depends on the previous step's position, so the chunk is
// first brought into shared memory by one bulk copy (cp.async.bulk, completed
// on an mbarrier with a bounded wait); chunks above the staging size are read
// through L1 from the resident file instead.
#pragma once

#include "bitstream.cuh"
#include "tma.cuh"
#include "values.cuh"

namespace ebi {
namespace {

constexpr uint32_t kFull = 0xffffffffu;

// 64 stream bits from little-endian words in shared memory.
__device__ __forceinline__ uint64_t peek64_le_smem(const uint32_t* w, uint64_t q) {
    const uint32_t i = static_cast<uint32_t>(q >> 5);
    const uint32_t sh = static_cast<uint32_t>(q & 31);
    const uint32_t a = bswap32(w[i]), b = bswap32(w[i + 1]), c = bswap32(w[i + 2]);
    const uint32_t hi = __funnelshift_l(b, a, sh), lo = __funnelshift_l(c, b, sh);
    return (uint64_t(hi) << 32) | lo;
}

// Bytes [byte_off & ~15, end) staged for a chunk: 16-byte aligned both ends
// (bulk-copy rule) and 16 bytes past the chunk for the last read's over-read.
__host__ __device__ __forceinline__ uint64_t stage_span(uint64_t byte_off, uint64_t byte_len) {
    return ((byte_off + byte_len + 15) & ~uint64_t(15)) + 16 - (byte_off & ~uint64_t(15));
}

// Decodes chunk cd and runs the query over its values (one warp).
// The walk of one chunk for up to MaxQ queries over the same column at once
// (qs[0 .. nq), those with bit j of okm set): the stream is parsed once and
// each emitted run of values goes through every query's bitmask, predicate
// and aggregates.  Materialize and count passes take one query.
template <int MaxQ, typename Peek>
__device__ __forceinline__ void walk(const QueryParams* qs, uint32_t nq, uint32_t okm, const ChunkDesc& cd, uint32_t c,
                                     uint32_t li, int mode, const unsigned long long* chunk_offsets, Peek peek) {
    const int lane = threadIdx.x & 31;
    const uint64_t B = cd.byte_len * 8;
    KeyPred kp[MaxQ];
    ValAgg agg[MaxQ];
#pragma unroll
    for (int j = 0; j < MaxQ; ++j) {
        const QueryParams& q = qs[j < static_cast<int>(nq) ? j : 0];
        kp[j] = key_pred(q.pred);
        agg[j] = val_agg_init(q.op == OP_FILTER_AGG || q.op == OP_AGG ? q.agg : 0u);
    }
    unsigned long long out_pos = mode == VAL_MATERIALIZE ? chunk_offsets[li] : 0ull;
    uint64_t idx = 0;  // chunk row of the next value

    // Lanes [0, k) hold the values (bits) of rows idx + lane.  Applies the end
    // marker and the queries; returns true when the stream ended here.
    auto emit = [&](uint32_t k, uint64_t vbits) -> bool {
        const uint32_t nanm = __ballot_sync(kFull, static_cast<uint32_t>(lane) < k && vbits == kNanBits);
        bool ended = false;
        if (nanm) {
            k = __ffs(nanm) - 1;
            ended = true;
        }
        const uint64_t g = cd.row_off + idx + lane;
#pragma unroll
        for (int j = 0; j < MaxQ; ++j) {
            if (j >= static_cast<int>(nq) || !((okm >> j) & 1u)) continue;  // the same for every lane
            const QueryParams& q = qs[j];
            const bool pred_on = q.pred_on != 0;
            const bool in = static_cast<uint32_t>(lane) < k && (!q.in_mask || mask_row(q.in_mask, q.n_records, g));
            const bool pass = in && (!pred_on || kp[j].pass(vbits));
            if (mode == VAL_MATERIALIZE) {
                const uint32_t bal = __ballot_sync(kFull, pass);
                if (pass) {
                    const unsigned long long pos = out_pos + __popc(bal & ((1u << lane) - 1u));
                    if (pos < q.out_cap) q.out_vals[pos] = __longlong_as_double(static_cast<long long>(vbits));
                }
                out_pos += __popc(bal);
            } else {
                if (mode == VAL_SCAN && pred_on && q.out_mask != nullptr) {
                    const uint32_t word = __ballot_sync(kFull, pass && g < q.n_records);
                    if (lane == 0 && word) store_mask_word(q.out_mask, cd.row_off + idx, word, true);
                }
                if (pass) {
                    if (mode == VAL_COUNT) ++agg[j].cnt;
                    else val_agg_add1(agg[j], vbits);
                }
            }
        }
        idx += k;
        return ended;
    };

    uint32_t status = 0;
    if (B < 64) {
        status = EBI_E_UNEXPECTED_END;
    } else {
        uint64_t carry = peek(0);  // the previous value
        uint64_t p = 64;
        uint32_t lead = 0, trail = 0;
        bool done = emit(1, carry);
        while (!done) {
            if (p + 1 > B) { status = EBI_E_UNEXPECTED_END; break; }
            const uint64_t x = peek(p);
            if (!(x >> 63)) {
                // '0' run: one repeat per zero bit inside the chunk
                uint64_t z = x ? static_cast<uint64_t>(__clzll(static_cast<long long>(x))) : 64;
                if (z > B - p) z = B - p;
                const uint32_t k = z < 32 ? static_cast<uint32_t>(z) : 32u;
                done = emit(k, carry);
                p += k;
                continue;
            }
            if (p + 2 > B) { status = EBI_E_UNEXPECTED_END; break; }
            if (!((x >> 62) & 1)) {
                // '10' run at stride 2 + sig
                const uint32_t sig = 64 - lead - trail;  // 1..64
                const uint64_t L = 2 + sig;
                const uint64_t qi = p + static_cast<uint64_t>(lane) * L;
                bool fits = qi + L <= B;
                uint64_t y = 0;
                if (fits) {
                    y = peek(qi);
                    fits = (y >> 62) == 2;
                }
                const uint32_t m = __ballot_sync(kFull, fits);
                const uint32_t k = ~m ? static_cast<uint32_t>(__ffs(~m) - 1) : 32u;
                if (k == 0) { status = EBI_E_UNEXPECTED_END; break; }  // the record at p does not fit
                uint64_t d = 0;
                if (static_cast<uint32_t>(lane) < k) {
                    const uint64_t w = sig <= 62 ? (y << 2) : peek(qi + 2);
                    d = (w >> (64 - sig)) << trail;
                }
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint64_t t = __shfl_up_sync(kFull, d, o);
                    if (lane >= o) d ^= t;
                }
                const uint64_t v = carry ^ d;
                carry = __shfl_sync(kFull, v, k - 1);
                p += k * L;
                done = emit(k, v);
                continue;
            }
            // '11': a new window
            if (p + 13 > B) { status = EBI_E_UNEXPECTED_END; break; }
            const uint32_t l = static_cast<uint32_t>(x >> 57) & 31u;
            const uint32_t sg = (static_cast<uint32_t>(x >> 51) & 63u) + 1;
            if (l + sg > 64) { status = EBI_E_CORRUPT; break; }
            if (p + 13 + sg > B) { status = EBI_E_UNEXPECTED_END; break; }
            lead = l;
            trail = 64 - l - sg;
            carry ^= (peek(p + 13) >> (64 - sg)) << trail;
            p += 13 + sg;
            done = emit(1, carry);
        }
    }
    if (status) {
        if (lane == 0) {
            for (uint32_t j = 0; j < nq; ++j)
                if ((okm >> j) & 1u) set_status(qs[j].acc + c, status);
            if (mode == VAL_COUNT) qs[0].tile_counts[li] = 0;
        }
        return;
    }
    if (mode == VAL_MATERIALIZE) return;
#pragma unroll
    for (int j = 0; j < MaxQ; ++j) {
        if (j >= static_cast<int>(nq) || !((okm >> j) & 1u)) continue;  // the same for every lane
        const ValAgg a = val_agg_warp(agg[j]);
        if (lane != 0) continue;
        if (mode == VAL_COUNT) qs[j].tile_counts[li] = a.cnt;
        else val_agg_store(qs[j].acc + c, a);
    }
}

// Chunk selection and geometry checks of one Gorilla chunk (warp-uniform
// result): false when the pass skips the chunk.
__device__ __forceinline__ bool gorilla_begin(const QueryParams& q, uint32_t li, uint32_t c, int mode,
                                              const unsigned long long* chunk_offsets) {
    const int lane = threadIdx.x & 31;
    const ChunkDesc cd = q.chunks[c];
    ChunkAcc* acc = q.acc + c;
    const bool has_mask = q.in_mask != nullptr;

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
        if (ok && (cd.flags & kChunkBadGeometry)) {
            set_status(acc, EBI_E_IO);
            ok = 0;
        }
        if (!ok && mode == VAL_COUNT) q.tile_counts[li] = 0;
    }
    return __shfl_sync(kFull, ok, 0) != 0;

}

// One Gorilla chunk by one warp for nq <= MaxQ queries over the same column
// (qs[0 .. nq)), reading the stream through L1 (no staging).
template <int MaxQ>
__device__ __forceinline__ void gorilla_chunk_l1(const QueryParams* qs, uint32_t nq, uint32_t li, uint32_t c, int mode,
                                                 const unsigned long long* chunk_offsets) {
    uint32_t okm = 0;
    for (uint32_t j = 0; j < nq; ++j)  // the same for every lane
        if (gorilla_begin(qs[j], li, c, mode, chunk_offsets)) okm |= 1u << j;
    if (!okm) return;
    const ChunkDesc cd = qs[0].chunks[c];
    const uint32_t* fw = reinterpret_cast<const uint32_t*>(qs[0].file);
    const uint64_t bit0 = cd.byte_off * 8;
    walk<MaxQ>(qs, nq, okm, cd, c, li, mode, chunk_offsets,
               [fw, bit0](uint64_t p) { return peek64_file(fw, bit0 + p); });
}

}  // namespace
}  // namespace ebi
