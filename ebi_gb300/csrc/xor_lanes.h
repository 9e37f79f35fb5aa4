// xor_lanes.h -- the per-lane steps of the warp-per-chunk XOR decode
// (Chimp, Chimp128, Elf, ElfOnChimp), host and device alike.
//
// A chunk's bits after its first value are cut into kLanes segments, one per
// lane of a warp.  Every step below is what ONE lane does between two warp
// exchanges (shuffles, votes, scans); xor_warp.cuh runs them on the device
// with warp intrinsics, and a host emulation runs them lane after lane
// (tests/xor_lanes_emu.cpp), checking the split against the sequential
// reader.
//
//   1. lane_parse: parse the records that start in the lane's segment from a
//      start state (the true one for lane 0, a guess for the others).  A lane
//      whose start differs from its predecessor's end parses again from that
//      end; once no lane is stale, every segment equals the sequential parse
//      up to the first failing segment.  A re-parse stops as soon as it meets
//      its previous path at a checkpoint (the first record boundary at or
//      past a fixed bit position of the segment, same window, no failure on
//      either path before it): from there on the two parses are the same.
//   2. lane_xor_total (Chimp, Elf, ElfOnChimp): the XOR of the lane's record
//      deltas, and the lane's last Elf beta*; a warp scan of these gives
//      every lane the value chain and beta* its records start with.
//      lane_syms (Chimp128): every record value is
//      value(ring slot or previous record) ^ delta, the slot naming one of the
//      last 128 records.  The lane resolves its records against its own
//      records where it can and leaves the rest as (X, e): value = X ^
//      value(external record e), e one of the 128 records before the lane.
//      Composing the lanes' last-128 maps in lane order (one shared-memory
//      pass per lane, 128 entries each) gives every lane the true values of
//      the 128 records before it (T).
//   3. lane_values: the lane's records in order with their true values (the
//      chain seeded from step 2, Chimp128 from a ring holding T), stopping at
//      the first value equal to f64::NAN's bits (Chimp128: not for a '00'
//      copy), each value handed to a sink (the query).
//
// Positions are bits from the chunk's start, of type P: uint32_t for chunks
// under 2^31 bits (all the engine's usual chunks), uint64_t above.  Chimp and
// Chimp128 records are decoded branch-free (chimp_rec: the same instructions
// whatever the record's flag, so the lanes of a warp do not split), the Elf
// codecs through parse_rec of xor_parse.cuh.  The bit source is an object pk
// with pk.peek(p) (the 64 stream bits at p) and pk.peek2(p, y) (the same, and
// the 32 bits after them in y).
#pragma once

#include <cstdint>

#include "xor_parse.cuh"

namespace ebi {
namespace xorp {

constexpr int kLanes = 32;
constexpr int kCps = 3;                      // checkpoints per segment
constexpr uint8_t kExtNone = 0x80;           // Chimp128 sym: value has no external part
constexpr uint32_t kRingSlots = 128;

template <typename P>
XOR_HD constexpr P no_pos() { return ~P(0); }  // checkpoint not reached (or reached after a failure)

// Bits before the first record each lane parses: the first value's 64 raw
// bits (the Elf codecs parse their first record like any other).
XOR_HD constexpr uint64_t first_bits(int codec) { return is_elf(codec) ? 0 : 64; }
XOR_HD constexpr uint32_t start_win(int codec) {
    return codec == CODEC_GORILLA ? 0u : codec == CODEC_ELF ? kNoWin : kNoLead;
}

template <typename P>
struct Cp {
    P pos;         // no_pos: not recorded
    uint32_t win;
    uint32_t n;    // records counted before it
};

template <typename P>
struct LaneParse {
    PStateT<P> in, out;
    uint32_t n;     // records before the first failure
    uint32_t fail;  // first failure (0: none)
    Cp<P> cp[kCps];
};

// The lane's segment [beg, end) and its checkpoint positions.
template <typename P>
XOR_HD void lane_segment(P B, int codec, int lane, P& beg, P& end, P (&thr)[kCps]) {
    const P first = static_cast<P>(first_bits(codec));
    const P span = B > first ? B - first : 0;
    const P seg = (span + kLanes - 1) / kLanes;
    beg = first + seg * static_cast<P>(lane);
    if (beg > B) beg = B;
    end = first + seg * static_cast<P>(lane + 1);
    if (lane == kLanes - 1 || end > B) end = B;
#pragma unroll
    for (int k = 0; k < kCps; ++k) thr[k] = beg + (seg * static_cast<P>(k + 1)) / (kCps + 1);
}

// One Chimp / Chimp128 record at s.pos (decoder/chunk_reader/chimp.rs:58-124,
// chimp_n.rs:160-285) from x, the 64 stream bits there, and y, the 32 bits
// after them; the same results and errors as parse_rec, with the same
// instructions for every flag.
template <int CODEC, typename P>
XOR_HD uint32_t chimp_rec(uint64_t x, uint32_t y, P B, PStateT<P>& s, Rec& r) {
    constexpr bool k128 = CODEC == CODEC_CHIMP128;
    constexpr uint32_t H1 = k128 ? 16u : 9u;  // '01' header bits after the flag
    const P p = s.pos;
    const uint32_t flag = static_cast<uint32_t>(x >> 62);
    const uint32_t t1 = static_cast<uint32_t>(x >> (62 - H1)) & ((1u << H1) - 1u);
    const uint32_t lead1 = lead_decode((t1 >> 6) & 7u);
    const uint32_t sig1 = (t1 & 63u) ? (t1 & 63u) : 64u;
    const uint32_t lead3 = lead_decode(static_cast<uint32_t>(x >> 59) & 7u);
    const uint32_t hdr = flag == 0 ? (k128 ? 9u : 2u) : flag == 1 ? 2u + H1 : flag == 2 ? 2u : 5u;
    const uint32_t lead = flag == 1 ? lead1 : flag == 3 ? lead3 : s.win;
    const uint32_t nb = flag == 0 ? 0u : flag == 1 ? sig1 : 64u - (lead < 64u ? lead : 64u);  // payload bits
    const bool corrupt = (flag == 1 && sig1 + lead1 > 64) || (flag == 2 && s.win > 64);
    const uint32_t err = p + 2 > B || p + hdr > B ? EBI_E_UNEXPECTED_END
                       : corrupt                  ? EBI_E_CORRUPT
                       : p + hdr + nb > B         ? EBI_E_UNEXPECTED_END
                                                  : 0u;
    const uint64_t top = (x << hdr) | (static_cast<uint64_t>(y) >> (32 - hdr));  // the bits after the header
    const uint64_t pay = nb ? (top >> (64 - nb)) : 0ull;
    const uint32_t trail = flag == 1 && !corrupt ? 64u - sig1 - lead1 : 0u;
    r.delta = pay << trail;
    r.ring = k128 && flag == 0 ? static_cast<uint32_t>(x >> 55) & 127u : k128 && flag == 1 ? t1 >> 9 : kRefPrev;
    r.nan_ok = !(k128 && flag == 0);  // chimp_n.rs: the '00' copy is not checked against NaN
    r.meta = 0;
    if (!err) {
        s.win = flag == 1 ? lead1 : flag == 3 ? lead3 : s.win;
        s.pos = p + hdr + nb;
    }
    return err;
}

// One record with its delta.
template <int CODEC, typename Pk, typename P>
XOR_HD uint32_t lane_rec(Pk& pk, P B, PStateT<P>& s, Rec& r) {
    if (CODEC == CODEC_CHIMP || CODEC == CODEC_CHIMP128) {
        uint32_t y;
        const uint64_t x = pk.peek2(s.pos, y);
        return chimp_rec<CODEC>(x, y, B, s, r);
    }
    auto peek = [&pk](P q) { return pk.peek(q); };
    return parse_rec<CODEC>(peek, B, s, r);
}

// Parses the records that start in [L.in.pos, end): counts those before the
// first failure and, past a failure, steps one bit and goes on (a failing
// segment is the true end of the stream or a misaligned start; parse_segment
// of xor_parse.cuh has the same rule).  Records the checkpoints.  With
// has_old (old = the lane's previous parse of the segment) the parse stops
// where it meets old's path and takes the rest of old's result.
template <int CODEC, typename Pk, typename P>
XOR_HD void lane_parse(Pk& pk, P B, P end, bool last, const P (&thr)[kCps], LaneParse<P>& L, bool has_old,
                       const LaneParse<P>& old) {
    PStateT<P> s = L.in;
    uint32_t n = 0, f = 0;
    int k = 0;        // next checkpoint
    P nt = thr[0];    // its position (the per-record test reads a register)
    int met = -1;     // checkpoint where the parse met old's path
#pragma unroll
    for (int i = 0; i < kCps; ++i) L.cp[i].pos = no_pos<P>();
    while (s.pos < end) {
        if (s.pos >= nt) {
            // checkpoints k.. at or below s.pos (static indices after unrolling)
#pragma unroll
            for (int i = 0; i < kCps; ++i) {
                if (met >= 0 || i < k || s.pos < thr[i]) continue;
                if (!f) {
                    L.cp[i].pos = s.pos;
                    L.cp[i].win = s.win;
                    L.cp[i].n = n;
                    if (has_old && old.cp[i].pos == s.pos && old.cp[i].win == s.win) met = i;
                }
                k = i + 1;
            }
            if (met >= 0) break;
            nt = no_pos<P>();
#pragma unroll
            for (int i = kCps - 1; i >= 0; --i)
                if (i >= k) nt = thr[i];
        }
        Rec r;
        const uint32_t e = lane_rec<CODEC>(pk, B, s, r);
        if (e) {
            if (!f) f = e;
            s.pos += 1;
            continue;
        }
        if (!f) ++n;
    }
    if (met >= 0) {
        // same state as old at checkpoint `met`: the rest is old's parse, its counts shifted by d
        uint32_t d = 0;
#pragma unroll
        for (int i = 0; i < kCps; ++i)
            if (i == met) d = n - old.cp[i].n;
#pragma unroll
        for (int j = 0; j < kCps; ++j) {
            if (j <= met) continue;
            L.cp[j].pos = old.cp[j].pos;
            L.cp[j].win = old.cp[j].win;
            L.cp[j].n = old.cp[j].n + d;
        }
        L.n = old.n + d;
        L.fail = old.fail;
        L.out = old.out;
        return;
    }
    if (last && !f) f = EBI_E_UNEXPECTED_END;
    L.n = n;
    L.fail = f;
    L.out = s;
}

// XOR of the deltas of the lane's n records from s (after `head`, the
// chunk's raw first value, for lane 0 of the non-Elf codecs), and the beta*
// of its last Elf record that sets one (0xff: none).
template <int CODEC, typename Pk, typename P>
XOR_HD void lane_xor_total(Pk& pk, P B, PStateT<P> s, uint32_t n, bool head, uint64_t& x, uint32_t& beta_last) {
    x = head ? pk.peek(0) : 0;
    beta_last = 0xffu;
    for (uint32_t j = 0; j < n; ++j) {
        Rec r;
        lane_rec<CODEC>(pk, B, s, r);  // succeeds: these records precede the chunk's first failure
        x ^= r.delta;
        if (is_elf(CODEC) && (r.meta & kElfBeta)) beta_last = r.meta & 15u;
    }
}

// Ring r (of a warp's kLanes rings, 128 slots each) in the interleaved
// layout: slot s of ring r is element s * kLanes + ((r + s) % kLanes) of the
// u64 array x and of the byte array e.  Lanes reading different rings at one
// slot, and one ring at the 32 slots lane + 32 i, both hit distinct banks.
struct RingView {
    uint64_t* x;
    uint8_t* e;
    uint32_t r;
    XOR_HD uint32_t at(uint32_t s) const { return s * kLanes + ((r + s) & (kLanes - 1)); }
    XOR_HD uint64_t get(uint32_t s) const { return x[at(s)]; }
    XOR_HD void put(uint32_t s, uint64_t v) const { x[at(s)] = v; }
    XOR_HD uint8_t ext(uint32_t s) const { return e[at(s)]; }
    XOR_HD void put_ext(uint32_t s, uint8_t v) const { e[at(s)] = v; }
};
constexpr uint32_t kRingValBytes = kLanes * kRingSlots * 8;           // a warp's ring values
constexpr uint32_t kRingBytes = kRingValBytes + kLanes * kRingSlots;  // and their ext bytes

// Chimp128: the (X, e) form of the lane's records (its first record is the
// chunk's record `off`), left in `ring` for its last 128 records: slot
// i % 128 holds record i's value as X ^ T[e] (T: values of the 128 records
// before the lane; e = kExtNone when the value is X alone).
template <typename Pk, typename P>
XOR_HD void lane_syms(Pk& pk, P B, PStateT<P> s, uint32_t cnt, bool head, uint32_t off, const RingView& ring) {
    for (uint32_t k = 0; k < kRingSlots; ++k) {
        ring.put(k, 0);
        ring.put_ext(k, static_cast<uint8_t>(k));
    }
    for (uint32_t j = 0; j < cnt; ++j) {
        const uint32_t i = off + j;
        uint64_t x;
        uint8_t e;
        if (head && j == 0) {
            x = pk.peek(0);
            e = kExtNone;
        } else {
            Rec r;
            lane_rec<CODEC_CHIMP128>(pk, B, s, r);
            const uint32_t src = r.ring == kRefPrev ? ((i - 1) & (kRingSlots - 1)) : r.ring;
            x = r.delta ^ ring.get(src);
            e = ring.ext(src);
        }
        ring.put(i & (kRingSlots - 1), x);
        ring.put_ext(i & (kRingSlots - 1), e);
    }
}

// One slot of one composition step: `dst` holds lane l's (X, e) forms and
// becomes T_l; `src` holds T_{l-1}.
XOR_HD void compose_slot(const RingView& dst, const RingView& src, uint32_t k) {
    const uint8_t e = dst.ext(k);
    dst.put(k, dst.get(k) ^ ((e & kExtNone) ? 0ull : src.get(e)));
}

// The lane's records with their values, in order.  The value chain starts at
// v (prefix XOR codecs; lane 0 of the non-Elf codecs starts with its head,
// the raw first value) or, for Chimp128, from `ring` holding T (updated as
// the records go, so that it ends holding the lane's own T).  Elf records
// flagged kElfRestore reach the sink with their erased value and the beta*
// in force (the sink restores).  Stops at the first end marker; returns its
// index among the lane's records (cnt when none of them is one).
// sink(j, bits, meta, beta) takes record j's value.
template <int CODEC, typename Pk, typename P, typename Sink>
XOR_HD uint32_t lane_values(Pk& pk, P B, PStateT<P> s, uint32_t cnt, bool head, uint32_t off, uint64_t v,
                            int32_t beta, const RingView* ring, Sink& sink) {
    uint64_t prev = 0;
    if (CODEC == CODEC_CHIMP128 && cnt) prev = off ? ring->get((off - 1) & (kRingSlots - 1)) : 0;
    for (uint32_t j = 0; j < cnt; ++j) {
        bool nan_ok = true;
        uint8_t meta = 0;
        if (head && j == 0) {
            v = pk.peek(0);
        } else {
            Rec r;
            lane_rec<CODEC>(pk, B, s, r);
            if (CODEC == CODEC_CHIMP128) {
                const uint64_t rv = ring->get(r.ring & (kRingSlots - 1));  // read for every record: no branch
                v = (r.ring == kRefPrev ? prev : rv) ^ r.delta;
                nan_ok = r.nan_ok;
            } else {
                v ^= r.delta;
            }
            meta = r.meta;
        }
        if (CODEC == CODEC_CHIMP128) {
            ring->put((off + j) & (kRingSlots - 1), v);
            prev = v;
        }
        if (nan_ok && v == 0x7ff8000000000000ull) return j;
        if (is_elf(CODEC) && (meta & kElfBeta)) beta = meta & 15;
        sink(j, v, meta, beta);
    }
    return cnt;
}

}  // namespace xorp
}  // namespace ebi
