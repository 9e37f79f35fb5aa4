// xor_warp.cuh -- Chimp, Chimp128, Elf and ElfOnChimp chunks decoded and
// queried by ONE WARP per chunk (the lane steps of xor_lanes.h).
//
// Formats (big-endian bit order, MSB of the first byte first):
//   Chimp     decoder/chunk_reader/chimp.rs:58-124: 2-bit flags; '01' carries
//             a 3-bit leading code (LEADING_REPR) and 6 significant bits.
//   Chimp128  decoder/chunk_reader/chimp_n.rs:160-285: as Chimp, but '00' and
//             '01' name one of the last 128 values by a 7-bit ring index.
//   Elf       decoder/chunk_reader/elf.rs: per value a wrapper prefix ('0'
//             restore, '10' as is, '11' + 4-bit beta* and restore) and an
//             ElfXor record; ElfOnChimp: the same prefix over Chimp records.
// A stream ends at the first value equal to f64::NAN's bits (Chimp128: not
// for a '00' copy); a read past the chunk raises UnexpectedEndOfChunk first.
//
// The warp's lanes each take one 32nd of the chunk's bits:
//   1. segment parse until no lane's start differs from its predecessor's
//      end (one or two re-parse rounds: a misaligned parse falls into step
//      within a few dozen records, a segment holds a few hundred; a re-parse
//      stops where it meets its previous path);
//   2. Chimp / Elf: XOR of each lane's deltas and a warp scan; Chimp128: each
//      lane's records in (X, e) form and the lanes' last-128 maps composed in
//      lane order into the values of the 128 records before every lane;
//   3. the query pass: each lane walks its records with their true values and
//      stops at the end marker.  Its bitmask words wait in shared memory
//      until a warp vote has found the chunk's end marker; lanes past it drop
//      what they found.  (A lane with more rows than the buffer holds makes
//      the warp find the end marker in a pass of its own first.)
// Every lane reads its stretch of the chunk from a 256-byte window in shared
// memory that cp.async fills ahead of it: under SIMT a read that missed
// on-chip memory would stall all 32 lanes, and with 32 independent streams
// some lane would miss on almost every step.  Chimp128's rings (36 KB per
// warp) live in shared memory too.  A warp handles up to MaxQ queries of one
// column per query pass; more queries take more passes over the chunk.
#pragma once

#include <type_traits>

#include "bitstream.cuh"
#include "elf_dev.cuh"
#include "values.cuh"
#include "xor_lanes.h"

namespace ebi {
namespace {

using namespace xorp;

constexpr uint32_t kWAll = 0xffffffffu;
constexpr uint32_t kWinBytes = 32 * 256;        // a warp's stream windows
constexpr uint32_t kBitCap = 512;               // rows per lane whose bitmask words wait in shared memory
constexpr uint32_t kBitWords = kBitCap / 32 + 1;
constexpr uint32_t kBitBytes = kBitWords * 32 * 4;  // a warp's waiting bitmask words (per query of a pass)

// A lane's window on the file: 4 blocks of 64 bytes in shared memory, counted
// from the 64-byte block that holds the chunk's first byte, filled by
// cp.async up to 3 blocks ahead of the reader; a jump outside (the next
// pass) starts it again.  Layout: 8-byte unit u (0..31) of lane l at byte
// 8 (u * 32 + l), so a warp-wide 8-byte read of one unit per lane is the
// minimum two wavefronts whatever the units.  P: position type.
template <typename P>
struct LaneWin {
    using S = typename std::conditional<sizeof(P) == 4, int32_t, int64_t>::type;
    uint32_t* sm;         // the warp's windows
    const uint8_t* blk0;  // the file's 64-byte block holding the chunk's first byte
    uint64_t units;       // 8-byte units from blk0 inside the file's allocation (no copy reads past them)
    P rel0;               // bits from blk0 to the chunk's first bit
    S next, done;         // blocks [next - 4, next) requested; those below done have arrived
    uint32_t lane;

    __device__ __forceinline__ void request(S b) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint64_t u = static_cast<uint64_t>(b) * 8 + k;
            if (u < units) {
                const uint32_t dst =
                    static_cast<uint32_t>(__cvta_generic_to_shared(sm + 2 * ((u & 31) * 32 + lane)));
                asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst), "l"(blk0 + u * 8) : "memory");
            }
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    __device__ __forceinline__ static void wait_pending(S n) {  // at most n of the lane's groups in flight
        if (n <= 0) asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        else if (n == 1) asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        else if (n == 2) asm volatile("cp.async.wait_group 2;\n" ::: "memory");
        else asm volatile("cp.async.wait_group 3;\n" ::: "memory");
    }
    // Words [wd, wd + 3] (and the blocks that hold them) in the window.
    __device__ __forceinline__ void ensure(P wd) {
        const S cur = static_cast<S>(wd >> 4), need = static_cast<S>((wd + 3) >> 4);
        if (need >= done || cur < next - 4) {
            if (cur >= next || cur < next - 4) {  // outside the window: start it at cur
                wait_pending(0);
                next = cur;
                done = cur;
            }
            while (next <= cur + 3) request(next++);
            const S pend = next - 1 - need;  // newer blocks may stay in flight
            wait_pending(pend);
            done = next - (pend > 3 ? 3 : pend);
        }
    }
    __device__ __forceinline__ uint2 unit(uint32_t u) const {
        return *reinterpret_cast<const uint2*>(sm + 2 * ((u & 31u) * 32 + lane));
    }
    // The 64 stream bits at chunk bit p, and the 32 after them in y.
    __device__ __forceinline__ uint64_t peek2(P p, uint32_t& y) {
        const P r = rel0 + p;
        const P wd = r >> 5;
        ensure(wd);
        const uint32_t u0 = static_cast<uint32_t>(wd >> 1);
        const uint2 a = unit(u0), b = unit(u0 + 1), c = unit(u0 + 2);
        const bool odd = (wd & 1) != 0;
        const uint32_t w0 = bswap32(odd ? a.y : a.x), w1 = bswap32(odd ? b.x : a.y);
        const uint32_t w2 = bswap32(odd ? b.y : b.x), w3 = bswap32(odd ? c.x : b.y);
        const uint32_t sh = static_cast<uint32_t>(r & 31);
        y = __funnelshift_l(w3, w2, sh);
        return (uint64_t(__funnelshift_l(w1, w0, sh)) << 32) | __funnelshift_l(w2, w1, sh);
    }
    __device__ __forceinline__ uint64_t peek(P p) {
        uint32_t y;
        return peek2(p, y);
    }
    // Leaves none of the lane's copies in flight (before the windows' memory is reused).
    __device__ __forceinline__ static void drain() { wait_pending(0); }
};

__device__ __forceinline__ uint32_t warp_excl_sum(uint32_t v, uint32_t* total) {
    const int lane = threadIdx.x & 31;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kWAll, inc, o);
        if (lane >= o) inc += y;
    }
    *total = __shfl_sync(kWAll, inc, 31);
    return inc - v;
}

// One query's state in a query pass: predicate, aggregates, the cached input
// bitmask word and the output bitmask word being built.
struct WQuery {
    KeyPred kp;
    ValAgg agg;
    uint64_t mw_idx, ow_idx;
    uint32_t mw, ow;
    bool on, has_mask, pred_on, store;
};

// The query pass's sink: every (row, value) of the lane through the queries.
// Bitmask words go to shared memory (bits: word k of query q's buffer at
// bits[(q * kBitWords + k) * 32 + lane], k counted from the lane's first
// row's word w0) or, with bits == nullptr, straight to the output.
template <int CODEC, int MaxQ>
struct WSink {
    const QueryParams* qs;
    WQuery w[MaxQ];
    const double* dec_tab;
    uint32_t* bits;
    uint64_t row0, w0;  // global row of the lane's first record, and its bitmask word
    int mode;           // VAL_SCAN, VAL_COUNT, or VAL_MATERIALIZE (count when !write)
    bool write;         // VAL_MATERIALIZE: write values at pos
    unsigned long long pos;
    __device__ __forceinline__ void flush_bits(int k) {
        WQuery& Q = w[k];
        if (Q.ow_idx == ~0ull) return;
        const uint32_t lane = threadIdx.x & 31;
        if (bits) bits[(k * kBitWords + static_cast<uint32_t>(Q.ow_idx - w0)) * 32 + lane] = Q.ow;
        else if (Q.ow) atomicOr(&qs[k].out_mask[Q.ow_idx], Q.ow);
        Q.ow = 0;
    }
    __device__ __forceinline__ void operator()(uint32_t j, uint64_t v, uint8_t meta, int32_t beta) {
        uint64_t out = v;
        if (is_elf(CODEC) && (meta & kElfRestore))
            out = static_cast<uint64_t>(
                __double_as_longlong(elf_recover(__longlong_as_double(static_cast<long long>(v)), beta, dec_tab)));
        const uint64_t g = row0 + j;
#pragma unroll
        for (int k = 0; k < MaxQ; ++k) {
            WQuery& Q = w[k];
            if (!Q.on) continue;
            const QueryParams& q = qs[k];
            bool in = true;
            if (Q.has_mask) {
                if ((g >> 5) != Q.mw_idx) {
                    Q.mw_idx = g >> 5;
                    Q.mw = g < q.n_records ? q.in_mask[Q.mw_idx] : 0u;
                }
                in = g < q.n_records && ((Q.mw >> (g & 31)) & 1u);
            }
            const bool pass = in && (!Q.pred_on || Q.kp.pass(out));
            if (Q.store && g < q.n_records) {
                if ((g >> 5) != Q.ow_idx) {
                    flush_bits(k);
                    Q.ow_idx = g >> 5;
                }
                Q.ow |= static_cast<uint32_t>(pass) << (g & 31);
            }
            if (!pass) continue;
            if (mode == VAL_MATERIALIZE) {
                if (write && pos < q.out_cap) q.out_vals[pos] = __longlong_as_double(static_cast<long long>(out));
                ++pos;
                continue;
            }
            if (mode == VAL_COUNT) { ++Q.agg.cnt; continue; }
            val_agg_add1(Q.agg, out);
        }
    }
};

// The body of xor_chunk_warp for positions of type P (see there).
template <int CODEC, int MaxQ, typename P>
__device__ __forceinline__ void xor_chunk_warp_p(const QueryParams* qs, uint32_t nq, uint32_t okm, uint32_t li,
                                                 uint32_t c, int mode, const unsigned long long* chunk_offsets,
                                                 uint32_t* win, uint32_t* bitbuf, uint64_t* ring_x, uint8_t* ring_e) {
    const QueryParams& q = qs[0];
    const int lane = threadIdx.x & 31;
    const ChunkDesc cd = q.chunks[c];
    constexpr bool kElf = is_elf(CODEC);
    constexpr bool kRing = CODEC == CODEC_CHIMP128;
    const P B = static_cast<P>(cd.byte_len * 8);
    auto fail_chunk = [&](uint32_t status) {
        if (lane == 0)
            for (uint32_t k = 0; k < nq; ++k) {
                if (!((okm >> k) & 1u)) continue;
                set_status(qs[k].acc + c, status);
                if (mode == VAL_COUNT) qs[k].tile_counts[li] = 0;
            }
    };
    const uint64_t blk = cd.byte_off & ~uint64_t(63);
    LaneWin<P> pk{win, q.file + blk, (q.file_bytes - blk) / 8, static_cast<P>((cd.byte_off & 63) * 8),
                  -8, -8, static_cast<uint32_t>(lane)};

    // ---- 1. segment parse ---------------------------------------------------
    P beg, end, thr[kCps];
    lane_segment<P>(B, CODEC, lane, beg, end, thr);
    LaneParse<P> L;
    L.in = lane == 0 ? PStateT<P>{static_cast<P>(first_bits(CODEC)), start_win(CODEC)} : PStateT<P>{beg, 0u};
    lane_parse<CODEC>(pk, B, end, lane == kLanes - 1, thr, L, false, L);
    for (int round = 0; round < kLanes; ++round) {
        // (pos, win) of the predecessor's end; a position fits 48 bits
        const uint64_t mine = static_cast<uint64_t>(L.out.pos) | (static_cast<uint64_t>(L.out.win) << 48);
        const uint64_t prev = __shfl_up_sync(kWAll, mine, 1);
        const bool stale =
            lane > 0 && (static_cast<uint64_t>(L.in.pos) | (static_cast<uint64_t>(L.in.win) << 48)) != prev;
        if (!__any_sync(kWAll, stale)) break;
        if (stale) {
            const LaneParse<P> old = L;
            L.in = PStateT<P>{static_cast<P>(prev & ((1ull << 48) - 1)), static_cast<uint32_t>(prev >> 48)};
            lane_parse<CODEC>(pk, B, end, lane == kLanes - 1, thr, L, true, old);
        }
    }
    const uint32_t ff = static_cast<uint32_t>(__ffs(__ballot_sync(kWAll, L.fail != 0))) - 1u;  // first failing lane
    const uint32_t fail_status = __shfl_sync(kWAll, L.fail, ff & 31u);
    const bool head = !kElf && lane == 0;
    const uint32_t cnt = (static_cast<uint32_t>(lane) > ff ? 0u : L.n) + (head ? 1u : 0u);
    uint32_t total;
    const uint32_t off = warp_excl_sum(cnt, &total);

    // ---- 2. where each lane's value chain starts ------------------------------
    uint64_t prefix = 0;
    int32_t beta_in = INT32_MAX;
    if constexpr (!kRing) {
        uint64_t x;
        uint32_t bl;
        lane_xor_total<CODEC>(pk, B, L.in, cnt - (head ? 1u : 0u), head, x, bl);
        uint64_t inc = x;
        uint32_t key = bl != 0xffu ? ((static_cast<uint32_t>(lane) + 1u) << 8) | bl : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(kWAll, inc, o);
            const uint32_t ky = __shfl_up_sync(kWAll, key, o);
            if (lane >= o) {
                inc ^= y;
                key = max(key, ky);
            }
        }
        prefix = inc ^ x;
        uint32_t kx = __shfl_up_sync(kWAll, key, 1);
        if (lane == 0) kx = 0;
        if (kx) beta_in = static_cast<int32_t>(kx & 0xffu);
    } else {
        // ring 0 = the zero values before the chunk; lane l < 31 leaves its records'
        // (X, e) forms in ring l + 1 (lane 31's are needed by no one)
        for (uint32_t k = lane; k < kRingSlots; k += 32) RingView{ring_x, ring_e, 0}.put(k, 0);
        if (lane < kLanes - 1) lane_syms(pk, B, L.in, cnt, head, off, RingView{ring_x, ring_e, uint32_t(lane) + 1u});
        __syncwarp();
        for (uint32_t l = 0; l + 1 < kLanes; ++l) {  // ring l + 1 becomes T_l from T_{l-1} in ring l
            const RingView dst{ring_x, ring_e, l + 1}, src{ring_x, ring_e, l};
            for (uint32_t k = lane; k < kRingSlots; k += 32) compose_slot(dst, src, k);
            __syncwarp();
        }
    }

    // ---- 3. value passes ------------------------------------------------------
    // Value pass p reads Chimp128 lane l's starting values from ring (l - p) mod 32
    // and leaves the lane's own last 128 there; lane 0's ring is zeroed first.
    int pass = 0;
    auto walk = [&](uint32_t lim, auto& sink) -> uint32_t {
        if constexpr (kRing) {
            if (pass > 0) {
                const RingView z{ring_x, ring_e, static_cast<uint32_t>(kLanes - pass) & (kLanes - 1)};
                for (uint32_t k = lane; k < kRingSlots; k += 32) z.put(k, 0);
                __syncwarp();
            }
            const RingView rv{ring_x, ring_e, static_cast<uint32_t>(lane - pass) & (kLanes - 1)};
            const uint32_t r = lane_values<CODEC>(pk, B, L.in, lim, head, off, prefix, beta_in, &rv, sink);
            __syncwarp();
            ++pass;
            return r;
        } else {
            ++pass;
            return lane_values<CODEC>(pk, B, L.in, lim, head, off, prefix, beta_in,
                                      static_cast<const RingView*>(nullptr), sink);
        }
    };
    auto none = [](uint32_t, uint64_t, uint8_t, int32_t) {};

    uint32_t lim = cnt;  // records this lane walks
    bool known = false;  // the end marker is found and lim stops before it
    auto find_end = [&](uint32_t nan_j) -> bool {  // false: the chunk has no end marker before its failure
        const uint32_t m = __ballot_sync(kWAll, nan_j < cnt);
        if (!m) return false;
        const uint32_t ls = static_cast<uint32_t>(__ffs(m)) - 1u;
        const uint32_t e = __shfl_sync(kWAll, off + nan_j, ls);
        lim = e > off ? min(e - off, cnt) : 0u;
        known = true;
        return true;
    };
    auto fail_end = [&]() {
        LaneWin<P>::drain();
        fail_chunk(fail_status ? fail_status : EBI_E_UNEXPECTED_END);
    };
    const uint64_t row0 = cd.row_off + off;
    if (mode == VAL_MATERIALIZE) {  // one query: end marker, count, scan, write
        if (!find_end(walk(cnt, none))) { fail_end(); return; }
        const WQuery w0{key_pred(q.pred), val_agg_init(0u), ~0ull, ~0ull, 0u, 0u, true, q.in_mask != nullptr,
                        q.pred_on != 0, false};
        WSink<CODEC, 1> sink{qs, {w0}, q.dec_tab, nullptr, row0, row0 >> 5, VAL_MATERIALIZE, false, 0ull};
        walk(lim, sink);
        uint32_t tot;
        const uint32_t before = warp_excl_sum(static_cast<uint32_t>(sink.pos), &tot);
        WSink<CODEC, 1> wr{qs, {w0}, q.dec_tab, nullptr, row0, row0 >> 5, VAL_MATERIALIZE, true,
                           chunk_offsets[li] + before};
        walk(lim, wr);
        LaneWin<P>::drain();
        return;
    }
    bool stores = false;
    if (mode == VAL_SCAN)
        for (uint32_t k = 0; k < nq; ++k)
            if (((okm >> k) & 1u) && qs[k].pred_on && qs[k].out_mask) stores = true;
    // bitmask words wait in shared memory while every lane's rows fit its buffer
    const bool buffered = __all_sync(kWAll, stores && bitbuf != nullptr && cnt <= kBitCap);
    if (stores && !buffered) {
        if (!find_end(walk(cnt, none))) { fail_end(); return; }
    }
    for (uint32_t k0 = 0; k0 < nq; k0 += MaxQ) {
        if (!((okm >> k0) & ((MaxQ >= 32) ? kWAll : ((1u << MaxQ) - 1u)))) continue;
        WSink<CODEC, MaxQ> sink;
        sink.qs = qs + k0;
        sink.dec_tab = q.dec_tab;
        sink.bits = buffered ? bitbuf : nullptr;
        sink.row0 = row0;
        sink.w0 = row0 >> 5;
        sink.mode = mode;
        sink.write = false;
        sink.pos = 0;
#pragma unroll
        for (int k = 0; k < MaxQ; ++k) {
            const uint32_t qi = k0 + k;
            const bool on = qi < nq && ((okm >> qi) & 1u);
            const QueryParams& qk = qs[on ? qi : 0];
            sink.w[k] = WQuery{key_pred(qk.pred),
                               val_agg_init(qk.op == OP_FILTER_AGG || qk.op == OP_AGG ? qk.agg : 0u), ~0ull, ~0ull,
                               0u, 0u, on, qk.in_mask != nullptr, qk.pred_on != 0,
                               on && mode == VAL_SCAN && qk.pred_on && qk.out_mask != nullptr};
        }
        const uint32_t nan_j = walk(lim, sink);
        const bool was_known = known;
        if (!known && !find_end(nan_j)) { fail_end(); return; }
        // lanes past the end marker found rows that do not exist
        const bool drop = !was_known && lim == 0 && cnt != 0;
#pragma unroll
        for (int k = 0; k < MaxQ; ++k) {
            if (!sink.w[k].on) continue;  // the same for every lane
            if (sink.w[k].store) {
                const uint64_t last_w = sink.w[k].ow_idx;
                sink.flush_bits(k);
                if (buffered && !drop && last_w != ~0ull) {
                    // this lane's waiting words, from its first row to its last: all before the end marker
                    const uint32_t nw = static_cast<uint32_t>(last_w - sink.w0) + 1u;
                    for (uint32_t i = 0; i < nw; ++i) {
                        const uint32_t word = bitbuf[(k * kBitWords + i) * 32 + lane];
                        if (word) atomicOr(&qs[k0 + k].out_mask[sink.w0 + i], word);
                    }
                }
            }
            if (drop) sink.w[k].agg = val_agg_init(sink.w[k].agg.want);
            const ValAgg a = val_agg_warp(sink.w[k].agg);
            if (lane == 0) {
                if (mode == VAL_COUNT) qs[k0 + k].tile_counts[li] = a.cnt;
                else val_agg_store(qs[k0 + k].acc + c, a);
            }
        }
        __syncwarp();  // the waiting words are read before the next pass writes them
    }
    LaneWin<P>::drain();
}

// One Chimp-family chunk c by one warp for the queries qs[0, nq) over the
// same column (nq <= 32; materialize and count passes take one); li indexes
// the pass's per-chunk counts / offsets.  Shared memory of the warp: win
// (kWinBytes, stream windows), bitbuf (MaxQ * kBitBytes of waiting bitmask
// words, or nullptr: bitmask words go straight out after a pass that finds
// the end marker), ring_x / ring_e (Chimp128: kRingBytes of rings).
template <int CODEC, int MaxQ>
__device__ __forceinline__ void xor_chunk_warp(const QueryParams* qs, uint32_t nq, uint32_t li, uint32_t c, int mode,
                                               const unsigned long long* chunk_offsets, uint32_t* win,
                                               uint32_t* bitbuf, uint64_t* ring_x, uint8_t* ring_e) {
    const QueryParams& q = qs[0];  // the column (file, chunk table, tables) of every query
    const int lane = threadIdx.x & 31;
    const ChunkDesc cd = q.chunks[c];
    uint32_t okm = 0;  // bit k: query k reads the chunk
    if (lane == 0) {
        for (uint32_t k = 0; k < nq; ++k) {
            const QueryParams& qk = qs[k];
            ChunkAcc* ak = qk.acc + c;
            const bool hm = qk.in_mask != nullptr;
            int ok = 1;
            if (mode == VAL_SCAN) {
                ok = hm ? ak->selected != 0 : (qk.chunk_id < 0 || static_cast<uint64_t>(qk.chunk_id) == c);
                if (ok && !hm) ak->selected = 1;
            } else if (mode == VAL_MATERIALIZE) {
                ok = chunk_offsets[li + 1] != chunk_offsets[li];
            } else if (hm) {
                // the Decoder reads a chunk only when the bitmask meets its rows
                uint32_t any = 0;
                for (uint64_t r = 0; r < cd.n_rows && !any; r += 32) {
                    uint32_t w = mask_word(qk.in_mask, cd.row_off + r, qk.n_records);
                    if (cd.n_rows - r < 32) w &= (1u << (cd.n_rows - r)) - 1u;
                    any = w;
                }
                ok = any != 0;
            }
            if (ok && (cd.flags & kChunkBadGeometry)) { set_status(ak, EBI_E_IO); ok = 0; }
            if (!ok && mode == VAL_COUNT) qk.tile_counts[li] = 0;
            if (ok) okm |= 1u << k;
        }
    }
    okm = __shfl_sync(kWAll, okm, 0);
    if (!okm) return;
    if (!is_elf(CODEC) && cd.byte_len * 8 < 64) {
        if (lane == 0)
            for (uint32_t k = 0; k < nq; ++k) {
                if (!((okm >> k) & 1u)) continue;
                set_status(qs[k].acc + c, EBI_E_UNEXPECTED_END);
                if (mode == VAL_COUNT) qs[k].tile_counts[li] = 0;
            }
        return;
    }
    if (cd.byte_len < (1ull << 28))  // under 2^31 bits: 32-bit positions
        xor_chunk_warp_p<CODEC, MaxQ, uint32_t>(qs, nq, okm, li, c, mode, chunk_offsets, win, bitbuf, ring_x, ring_e);
    else
        xor_chunk_warp_p<CODEC, MaxQ, uint64_t>(qs, nq, okm, li, c, mode, chunk_offsets, win, bitbuf, ring_x, ring_e);
}

}  // namespace
}  // namespace ebi
