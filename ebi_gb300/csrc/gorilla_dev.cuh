// gorilla_dev.cuh -- Gorilla chunks parsed by one warp per chunk and queried.
//
// Format (decoder/chunk_reader/gorilla.rs:90-157; encoder compressor/gorilla.rs:118-190):
// 64 raw bits, then per value '0' (repeat), '10' + payload in the inherited
// window (significant bits = 64 - lead - trail), or '11' + 5-bit leading +
// 6-bit (significant - 1) + payload.  The stream ends at the first value
// equal to f64::NAN's bits; a read past the chunk raises UnexpectedEndOfChunk.
//
// The warp follows the stream exactly, several records per step:
//   * a '0' run: the count of leading zero bits at the cursor is the number of
//     consecutive repeats (up to 32 per step); the step's remaining lanes
//     check the '10' records that follow, as below;
//   * a '10' run: with the window fixed, records sit at a fixed stride of
//     2 + significant bits.  Lane i checks that record i of the stride still
//     starts with '10' and fits in the chunk; the ballot's leading ones say how
//     many records are confirmed, each lane extracts its payload and a
//     warp-shuffle prefix XOR (seeded with the previous value) gives the values;
//   * a '11' record (new window) opens a step: lane 0 takes it and lanes 1..31
//     check the '10' records that follow it in the new window, as above.
// On the bench series over 98 % of the records are '10', so an 8,192-value
// chunk takes a few hundred warp steps.  The parse (parse_stream) cuts each
// step at the NaN end marker and hands it to a query sink: value i of the step
// to lane i, which runs the bitmask ballot, the per-lane compensated sums,
// min / max, or the materialize positions.  WalkSink keeps up to a few queries'
// state in registers, SharedSink up to 8 in shared memory; both, and the
// single-column pass that feeds a sink from another warp, see the same steps,
// so every path gives the same per-lane sums and the same results.
//
// Every step's read depends on the previous step's position, so the
// single-column pass first brings the chunk into shared memory by one bulk
// copy (cp.async.bulk, completed on an mbarrier with a bounded wait); chunks
// above the staging size, and the batched walk, read through L1 from the
// resident file instead.
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

// The query side of a chunk walk: up to MaxQ queries over the same column
// (qs[0 .. nq), those with bit j of okm set), each with its predicate and
// per-lane running aggregates in registers.  Each emitted run of values (lanes
// [0, k) hold chunk rows idx .. idx + k - 1) goes through every query's
// bitmask, predicate and aggregates.  Materialize and count passes take one
// query.  Part splits the work between two sinks fed the same steps: 0 does
// everything; 1 everything but the compensated sums; 2 only the sums.
enum : int { kPartAll = 0, kPartNoSum = 1, kPartSum = 2 };
template <int MaxQ, int Part = kPartAll>
struct WalkSink {
    const QueryParams* qs;
    uint32_t nq, okm;
    int mode;
    uint64_t row_off;
    KeyPred kp[MaxQ];
    ValAgg agg[MaxQ];
    unsigned long long out_pos;
    uint64_t idx;  // chunk row of the next value

    __device__ __forceinline__ void init(const QueryParams* qs_, uint32_t nq_, uint32_t okm_, const ChunkDesc& cd,
                                         uint32_t li, int mode_, const unsigned long long* chunk_offsets) {
        qs = qs_;
        nq = nq_;
        okm = okm_;
        mode = mode_;
        row_off = cd.row_off;
#pragma unroll
        for (int j = 0; j < MaxQ; ++j) {
            const QueryParams& q = qs[j < static_cast<int>(nq) ? j : 0];
            kp[j] = key_pred(q.pred);
            agg[j] = val_agg_init(q.op == OP_FILTER_AGG || q.op == OP_AGG ? q.agg : 0u);
        }
        out_pos = mode == VAL_MATERIALIZE ? chunk_offsets[li] : 0ull;
        idx = 0;
    }

    __device__ __forceinline__ void apply(uint32_t k, uint64_t vbits) {
        const int lane = threadIdx.x & 31;
        const uint64_t g = row_off + idx + lane;
#pragma unroll
        for (int j = 0; j < MaxQ; ++j) {
            if (j >= static_cast<int>(nq) || !((okm >> j) & 1u)) continue;  // the same for every lane
            const QueryParams& q = qs[j];
            const bool pred_on = q.pred_on != 0;
            const bool in = static_cast<uint32_t>(lane) < k && (!q.in_mask || mask_row(q.in_mask, q.n_records, g));
            const bool pass = in && (!pred_on || kp[j].pass(vbits));
            if (Part == kPartSum) {
                if (mode == VAL_SCAN && pass && (agg[j].want & AGG_SUM))
                    neumaier_add(agg[j].hi, agg[j].lo, __longlong_as_double(static_cast<long long>(vbits)));
                continue;
            }
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
                    if (lane == 0 && word) store_mask_word(q.out_mask, row_off + idx, word, true);
                }
                if (pass) {
                    if (mode == VAL_COUNT) {
                        ++agg[j].cnt;
                    } else if (Part == kPartNoSum) {
                        ++agg[j].cnt;
                        val_agg_minmax(agg[j], vbits);
                    } else {
                        val_agg_add1(agg[j], vbits);
                    }
                }
            }
        }
        idx += k;
    }

    __device__ __forceinline__ void fail(uint32_t c, uint32_t li, uint32_t status) {
        if ((threadIdx.x & 31) == 0) {
            for (uint32_t j = 0; j < nq; ++j)
                if ((okm >> j) & 1u) set_status(qs[j].acc + c, status);
            if (mode == VAL_COUNT) qs[0].tile_counts[li] = 0;
        }
    }

    __device__ __forceinline__ void finish(uint32_t c, uint32_t li) {
        const int lane = threadIdx.x & 31;
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
};

// WalkSink with its per-query state in shared memory instead of registers, so
// that one walk serves up to kSharedSinkQueries queries (a batch item's share
// of the CTA's dynamic shared memory per warp).  Every lane runs the same
// aggregate updates in the same order as WalkSink's (value i of a step to lane
// i), so results are identical.  Scan passes only (no count / materialize).
constexpr uint32_t kSharedSinkQueries = 8;
struct SharedSinkState {
    KeyPred kp[kSharedSinkQueries];
    uint32_t want[kSharedSinkQueries];
    double hi[kSharedSinkQueries][32], lo[kSharedSinkQueries][32];
    unsigned long long mnk[kSharedSinkQueries][32], mxk[kSharedSinkQueries][32], cnt[kSharedSinkQueries][32];
};

struct SharedSink {
    const QueryParams* qs;
    uint32_t nq, okm;
    uint64_t row_off;
    uint64_t idx;
    SharedSinkState* st;

    __device__ __forceinline__ void init(const QueryParams* qs_, uint32_t nq_, uint32_t okm_, const ChunkDesc& cd,
                                         SharedSinkState* st_) {
        const int lane = threadIdx.x & 31;
        qs = qs_;
        nq = nq_;
        okm = okm_;
        row_off = cd.row_off;
        idx = 0;
        st = st_;
        for (uint32_t j = 0; j < nq; ++j) {
            const QueryParams& q = qs[j];
            const ValAgg a = val_agg_init(q.op == OP_FILTER_AGG || q.op == OP_AGG ? q.agg : 0u);
            if (lane == 0) {
                st->kp[j] = key_pred(q.pred);
                st->want[j] = a.want;
            }
            st->hi[j][lane] = a.hi;
            st->lo[j][lane] = a.lo;
            st->mnk[j][lane] = a.mnk;
            st->mxk[j][lane] = a.mxk;
            st->cnt[j][lane] = a.cnt;
        }
        __syncwarp();
    }

    __device__ __forceinline__ void apply(uint32_t k, uint64_t vbits) {
        const int lane = threadIdx.x & 31;
        const uint64_t g = row_off + idx + lane;
        for (uint32_t j = 0; j < nq; ++j) {
            if (!((okm >> j) & 1u)) continue;  // the same for every lane
            const QueryParams& q = qs[j];
            const bool pred_on = q.pred_on != 0;
            const bool in = static_cast<uint32_t>(lane) < k && (!q.in_mask || mask_row(q.in_mask, q.n_records, g));
            const bool pass = in && (!pred_on || st->kp[j].pass(vbits));
            if (pred_on && q.out_mask != nullptr) {
                const uint32_t word = __ballot_sync(kFull, pass && g < q.n_records);
                if (lane == 0 && word) store_mask_word(q.out_mask, row_off + idx, word, true);
            }
            if (pass) {
                ValAgg a{st->hi[j][lane], st->lo[j][lane], st->mnk[j][lane], st->mxk[j][lane], st->cnt[j][lane],
                         st->want[j]};
                val_agg_add1(a, vbits);
                st->hi[j][lane] = a.hi;
                st->lo[j][lane] = a.lo;
                st->mnk[j][lane] = a.mnk;
                st->mxk[j][lane] = a.mxk;
                st->cnt[j][lane] = a.cnt;
            }
        }
        idx += k;
    }

    __device__ __forceinline__ void fail(uint32_t c, uint32_t status) {
        if ((threadIdx.x & 31) == 0)
            for (uint32_t j = 0; j < nq; ++j)
                if ((okm >> j) & 1u) set_status(qs[j].acc + c, status);
    }

    __device__ __forceinline__ void finish(uint32_t c) {
        const int lane = threadIdx.x & 31;
        for (uint32_t j = 0; j < nq; ++j) {
            if (!((okm >> j) & 1u)) continue;  // the same for every lane
            ValAgg a{st->hi[j][lane], st->lo[j][lane], st->mnk[j][lane], st->mxk[j][lane], st->cnt[j][lane], st->want[j]};
            a = val_agg_warp(a);
            if (lane == 0) val_agg_store(qs[j].acc + c, a);
        }
    }
};

// The parse side of a chunk walk (one warp): follows the stream of B bits and
// calls emit(k, vbits) for each step's values, lanes [0, k) holding them (the
// end marker already cut off: k may be 0 on the last step).  Returns 0 when
// the stream ended at its marker, else the chunk's error status.
template <typename Peek, typename Emit>
__device__ __forceinline__ uint32_t parse_stream(uint64_t B, Peek peek, Emit emit) {
    const int lane = threadIdx.x & 31;
    // applies the end marker to a step: true when the stream ended in it
    auto step = [&](uint32_t k, uint64_t vbits) -> bool {
        const uint32_t nanm = __ballot_sync(kFull, static_cast<uint32_t>(lane) < k && vbits == kNanBits);
        const bool ended = nanm != 0;
        emit(ended ? static_cast<uint32_t>(__ffs(nanm) - 1) : k, vbits);
        return ended;
    };
    if (B < 64) return EBI_E_UNEXPECTED_END;
    uint64_t carry = peek(0);  // the previous value
    uint64_t p = 64;
    uint32_t lead = 0, trail = 0;
    if (step(1, carry)) return 0;
    for (;;) {
        if (p + 1 > B) return EBI_E_UNEXPECTED_END;
        const uint64_t x = peek(p);
        uint32_t first;  // lanes before it hold a value already (repeats, or this step's '11' record)
        uint64_t d = 0;  // each lane's XOR delta against the previous value
        uint64_t p0;     // the run's first record
        if (!(x >> 63)) {
            // '0' run: one repeat (delta 0) per zero bit inside the chunk, then in
            // the same step the '10' run that may follow it
            uint64_t z = x ? static_cast<uint64_t>(__clzll(static_cast<long long>(x))) : 64;
            if (z > B - p) z = B - p;
            first = z < 32 ? static_cast<uint32_t>(z) : 32u;
            p0 = p + first;
        } else if (p + 2 > B) {
            return EBI_E_UNEXPECTED_END;
        } else if (!((x >> 62) & 1)) {
            first = 0;
            p0 = p;
        } else {
            // '11': a new window, then in the same step the '10' run that follows it
            if (p + 13 > B) return EBI_E_UNEXPECTED_END;
            const uint32_t l = static_cast<uint32_t>(x >> 57) & 31u;
            const uint32_t sg = (static_cast<uint32_t>(x >> 51) & 63u) + 1;
            if (l + sg > 64) return EBI_E_CORRUPT;
            if (p + 13 + sg > B) return EBI_E_UNEXPECTED_END;
            lead = l;
            trail = 64 - l - sg;
            if (lane == 0) d = (peek(p + 13) >> (64 - sg)) << trail;
            first = 1;
            p0 = p + 13 + sg;
        }
        // '10' records at stride 2 + sig from p0, one per lane from lane `first`
        const uint32_t sig = 64 - lead - trail;  // 1..64
        const uint64_t L = 2 + sig;
        const uint64_t qi = p0 + static_cast<uint64_t>(static_cast<uint32_t>(lane) - first) * L;
        bool fits = static_cast<uint32_t>(lane) < first;
        uint64_t y = 0;
        if (!fits && qi + L <= B) {
            y = peek(qi);
            fits = (y >> 62) == 2;
        }
        const uint32_t m = __ballot_sync(kFull, fits);
        const uint32_t k = ~m ? static_cast<uint32_t>(__ffs(~m) - 1) : 32u;
        if (k == 0) return EBI_E_UNEXPECTED_END;  // the '10' record at p does not fit
        if (static_cast<uint32_t>(lane) >= first && static_cast<uint32_t>(lane) < k) {
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
        p = p0 + (k - first) * L;
        if (step(k, v)) return 0;
    }
}

// Decodes chunk cd and runs up to MaxQ queries over its values (one warp: the
// walk parses the stream once and applies each step to every query).
template <int MaxQ, typename Peek>
__device__ __forceinline__ void walk(const QueryParams* qs, uint32_t nq, uint32_t okm, const ChunkDesc& cd, uint32_t c,
                                     uint32_t li, int mode, const unsigned long long* chunk_offsets, Peek peek) {
    WalkSink<MaxQ> sink;
    sink.init(qs, nq, okm, cd, li, mode, chunk_offsets);
    const uint32_t status = parse_stream(cd.byte_len * 8, peek, [&](uint32_t k, uint64_t v) { sink.apply(k, v); });
    if (status) sink.fail(c, li, status);
    else sink.finish(c, li);
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

// One Gorilla chunk by one warp for nq <= kSharedSinkQueries scan queries over
// the same column, their state in `st` (this warp's shared memory).
__device__ __forceinline__ void gorilla_chunk_l1_shared(const QueryParams* qs, uint32_t nq, uint32_t c,
                                                        SharedSinkState* st) {
    uint32_t okm = 0;
    for (uint32_t j = 0; j < nq; ++j)  // the same for every lane
        if (gorilla_begin(qs[j], c, c, VAL_SCAN, nullptr)) okm |= 1u << j;
    if (!okm) return;
    const ChunkDesc cd = qs[0].chunks[c];
    const uint32_t* fw = reinterpret_cast<const uint32_t*>(qs[0].file);
    const uint64_t bit0 = cd.byte_off * 8;
    SharedSink sink;
    sink.init(qs, nq, okm, cd, st);
    const uint32_t status = parse_stream(cd.byte_len * 8, [fw, bit0](uint64_t p) { return peek64_file(fw, bit0 + p); },
                                         [&](uint32_t k, uint64_t v) { sink.apply(k, v); });
    if (status) sink.fail(c, status);
    else sink.finish(c);
}

}  // namespace
}  // namespace ebi
