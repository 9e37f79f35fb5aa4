// xor_parse.cuh -- record parser of the Gorilla, Chimp, Chimp128, Elf and ElfOnChimp bitstreams,
// shared by the decode kernel (xor.cu) and host-side checks of its segment
// algorithm.  Host and device functions alike: the bit source is a functor
// that returns the 64 stream bits starting at a bit position.
#pragma once

#include <cstdint>

#include "../../include/ebi_gpu.h"
#include "elf_dev.cuh"

#if defined(__CUDACC__)
#define XOR_HD __host__ __device__ __forceinline__
#else
#define XOR_HD inline
#endif

namespace ebi {
namespace xorp {

constexpr uint32_t kNoRef = 0xffffu;     // Chimp128: value refers to an unset ring slot (0.0 bits)
constexpr uint32_t kNoLead = 0xffu;      // Chimp: no leading-zero count stored yet

enum : uint32_t {
    CODEC_GORILLA = EBI_GORILLA,
    CODEC_CHIMP = EBI_CHIMP,
    CODEC_CHIMP128 = EBI_CHIMP128,
    CODEC_ELF_CHIMP = EBI_ELF_ON_CHIMP,
    CODEC_ELF = EBI_ELF,
};
// Elf codecs: every record (the first included) is a wrapper prefix and a
// record of the inner XOR stream; the first record starts at bit 0.
XOR_HD constexpr bool is_elf(int codec) { return codec == CODEC_ELF || codec == CODEC_ELF_CHIMP; }
constexpr uint32_t kNoWin = 0xffffu;  // ElfXor: leading and trailing counts not stored yet

// LEADING_REPR decode table [0, 8, 12, 16, 18, 20, 22, 24] (decoder/chunk_reader/chimp.rs), 5 bits per entry.
XOR_HD uint32_t lead_decode(uint32_t t) {
    constexpr uint64_t kTable = (0ull << 0) | (8ull << 5) | (12ull << 10) | (16ull << 15) | (18ull << 20) |
                                (20ull << 25) | (22ull << 30) | (24ull << 35);
    return static_cast<uint32_t>(kTable >> (5 * t)) & 31u;
}

// Parser state: bit position in the chunk and the inherited window
// (Gorilla: lead | trail << 8; Chimp/Chimp128/ElfOnChimp: stored leading zeros
// or kNoLead; Elf: lead | trail << 8, kNoWin before any).
struct PState {
    uint64_t pos;
    uint32_t win;
};
XOR_HD uint64_t pack_state(PState s) { return s.pos | (uint64_t(s.win) << 48); }
XOR_HD PState unpack_state(uint64_t v) { return PState{v & ((1ull << 48) - 1), static_cast<uint32_t>(v >> 48)}; }

// One decoded record: the value is value(ref) ^ delta, where ref is the
// previous record (kRefPrev) or, for Chimp128's '00'/'01', a ring slot.
constexpr uint32_t kRefPrev = 0xffffffffu;
struct Rec {
    uint64_t delta;
    uint32_t ring;  // ring slot (Chimp128 '00'/'01') or kRefPrev
    bool nan_ok;    // the reader checks this value against the NaN end marker
    uint8_t meta;   // Elf: kElfRestore | kElfBeta | beta* of the wrapper prefix
};

// payload of n <= 64 bits at q (0 for n == 0)
template <typename Peek>
XOR_HD uint64_t take_bits(Peek peek, uint64_t q, uint32_t n) {
    return n ? peek(q) >> (64 - n) : 0;
}

// One Elf / ElfOnChimp record at s.pos (decoder/chunk_reader/elf.rs):
// the wrapper prefix '0' (restore with the current beta*), '10' (as is) or
// '11' + 4-bit beta* (restore), then the inner record -- at bit 0 the inner
// stream's first value (ElfXor read_first :121-141: 7-bit trailing zeros
// and the bits above the lowest set one; Chimp: 64 raw bits), else an
// ElfXor record (decompress_float_inner :143-221) or a Chimp record.
template <int CODEC, typename Peek>
XOR_HD uint32_t parse_elf(Peek peek, uint64_t B, PState& s, Rec& r);

// Parses one record at s.pos; returns 0 or the error the reader raises there
// (EBI_E_UNEXPECTED_END for a read past the chunk, EBI_E_CORRUPT for a
// window the reader's u8/u32 arithmetic cannot represent).  B = chunk bits.
template <int CODEC, typename Peek>
XOR_HD uint32_t parse_rec(Peek peek, uint64_t B, PState& s, Rec& r) {
    const uint64_t p = s.pos;
    r.ring = kRefPrev;
    r.nan_ok = true;
    r.meta = 0;
    if (is_elf(CODEC)) {
        return parse_elf<CODEC>(peek, B, s, r);
    } else if (CODEC == CODEC_GORILLA) {
        if (p + 1 > B) return EBI_E_UNEXPECTED_END;
        const uint64_t x = peek(p);
        if (!(x >> 63)) { s.pos = p + 1; r.delta = 0; return 0; }
        if (p + 2 > B) return EBI_E_UNEXPECTED_END;
        uint32_t lead = s.win & 0xffu, trail = s.win >> 8, n;
        uint64_t q;
        if (!((x >> 62) & 1)) {
            n = 64 - lead - trail;
            q = p + 2;
        } else {
            if (p + 13 > B) return EBI_E_UNEXPECTED_END;
            const uint32_t l = static_cast<uint32_t>(x >> 57) & 31u, sg = (static_cast<uint32_t>(x >> 51) & 63u) + 1;
            if (l + sg > 64) return EBI_E_CORRUPT;
            lead = l;
            trail = 64 - l - sg;
            n = sg;
            q = p + 13;
        }
        if (q + n > B) return EBI_E_UNEXPECTED_END;
        r.delta = (peek(q) >> (64 - n)) << trail;
        s.win = lead | (trail << 8);
        s.pos = q + n;
        return 0;
    } else {
        // Chimp / Chimp128, without branches on the flag: the lanes of a warp
        // parse different records, and a branch per flag would run every
        // lane through all four paths.  Every field is computed for every
        // flag and selected; the reader's error checks, in its order, run only
        // when one of them fails.
        if (p + 2 > B) return EBI_E_UNEXPECTED_END;
        // the record's first 128 bits in two reads that do not wait on each
        // other (a record is at most 2 + 16 + 64 bits); the second only when
        // the chunk goes on past the first
        const uint64_t x = peek(p);
        const uint64_t x2 = p + 64 < B ? peek(p + 64) : 0ull;
        const uint32_t flag = static_cast<uint32_t>(x >> 62);
        constexpr uint32_t hdr = CODEC == CODEC_CHIMP128 ? 16u : 9u;  // '01' header after the flag
        const uint32_t t = static_cast<uint32_t>(x >> (62 - hdr)) & ((1u << hdr) - 1u);
        const uint32_t lead1 = lead_decode((t >> 6) & 7u), lead3 = lead_decode(static_cast<uint32_t>(x >> 59) & 7u);
        const uint32_t sig1 = (t & 63u) ? (t & 63u) : 64u;
        const uint32_t lead = flag == 1 ? lead1 : flag == 3 ? lead3 : s.win;  // '00' and '10' keep the stored count
        const uint32_t hl = flag == 0 ? (CODEC == CODEC_CHIMP128 ? 9u : 2u) : flag == 1 ? 2u + hdr : flag == 2 ? 2u : 5u;
        const uint32_t n = flag == 0 ? 0u : flag == 1 ? sig1 : 64u - (lead > 64u ? 64u : lead);
        const uint64_t q = p + hl;
        const bool bad = (flag == 2 && s.win > 64u) || (flag == 1 && sig1 + lead1 > 64u) || q + n > B;
        if (bad) {
            if (flag == 0) return EBI_E_UNEXPECTED_END;  // p + 9 (Chimp128) past the chunk
            if (flag == 1) {
                if (p + 2 + hdr > B) return EBI_E_UNEXPECTED_END;
                if (sig1 + lead1 > 64u) return EBI_E_CORRUPT;
                return EBI_E_UNEXPECTED_END;
            }
            if (flag == 3) return EBI_E_UNEXPECTED_END;  // p + 5 or the payload past the chunk
            if (s.win > 64u) return EBI_E_CORRUPT;        // '10' before any leading count was stored
            return EBI_E_UNEXPECTED_END;
        }
        const uint32_t trail = flag == 1 ? 64u - sig1 - lead1 : 0u;
        const uint64_t y = (x << hl) | (x2 >> (64u - hl));  // the 64 bits at q (hl is 2..18)
        r.delta = (n == 64u ? y : n ? (y >> (64u - n)) : 0ull) << trail;
        if (CODEC == CODEC_CHIMP128) {
            r.ring = flag == 0 ? static_cast<uint32_t>(x >> 55) & 127u : flag == 1 ? (t >> 9) & 127u : kRefPrev;
            r.nan_ok = flag != 0;  // chimp_n.rs: the '00' copy is not checked against NaN
        }
        s.win = lead;
        s.pos = q + n;
        return 0;
    }
}

template <int CODEC, typename Peek>
XOR_HD uint32_t parse_elf(Peek peek, uint64_t B, PState& s, Rec& r) {
    const uint64_t p0 = s.pos;
    if (p0 + 1 > B) return EBI_E_UNEXPECTED_END;
    const uint64_t x = peek(p0);
    uint64_t p;
    if (!(x >> 63)) {
        r.meta = kElfRestore;
        p = p0 + 1;
    } else {
        if (p0 + 2 > B) return EBI_E_UNEXPECTED_END;
        if (!((x >> 62) & 1)) {
            r.meta = 0;
            p = p0 + 2;
        } else {
            if (p0 + 6 > B) return EBI_E_UNEXPECTED_END;
            r.meta = static_cast<uint8_t>(kElfRestore | kElfBeta | ((x >> 58) & 15u));
            p = p0 + 6;
        }
    }
    if (p0 == 0) {  // the first value of the inner stream
        if (CODEC == CODEC_ELF_CHIMP) {
            if (p + 64 > B) return EBI_E_UNEXPECTED_END;
            r.delta = peek(p);
            s.pos = p + 64;
            s.win = kNoLead;
            return 0;
        }
        if (p + 7 > B) return EBI_E_UNEXPECTED_END;
        const uint32_t tz = static_cast<uint32_t>(peek(p) >> 57);
        s.win = kNoWin;
        if (tz >= 64) {
            r.delta = 0;
            s.pos = p + 7;
            return 0;
        }
        const uint32_t n = 63 - tz;
        if (p + 7 + n > B) return EBI_E_UNEXPECTED_END;
        r.delta = ((take_bits(peek, p + 7, n) << 1) | 1u) << tz;
        s.pos = p + 7 + n;
        return 0;
    }
    if (CODEC == CODEC_ELF_CHIMP) {
        const uint8_t meta = r.meta;
        s.pos = p;
        const uint32_t e = parse_rec<CODEC_CHIMP>(peek, B, s, r);
        r.meta = meta;
        return e;
    }
    if (p + 2 > B) return EBI_E_UNEXPECTED_END;
    const uint64_t y = peek(p);
    const uint32_t flag = static_cast<uint32_t>(y >> 62);
    if (flag == 1) {  // '01': the previous value again
        r.delta = 0;
        s.pos = p + 2;
        return 0;
    }
    if (flag == 0) {  // '00': payload in the stored window
        const uint32_t lead = s.win & 0xffu, trail = s.win >> 8;
        if (lead > 64 || trail > 64 || lead + trail > 64) return EBI_E_CORRUPT;
        const uint32_t n = 64 - lead - trail;
        if (p + 2 + n > B) return EBI_E_UNEXPECTED_END;
        r.delta = n ? take_bits(peek, p + 2, n) << trail : 0;
        s.pos = p + 2 + n;
        return 0;
    }
    // '10': 3-bit leading code + 4-bit center; '11': 3-bit leading code + 6-bit center
    const uint32_t hb = flag == 3 ? 9u : 7u, cb = flag == 3 ? 6u : 4u;
    if (p + 2 + hb > B) return EBI_E_UNEXPECTED_END;
    const uint32_t lc = static_cast<uint32_t>(y >> (62 - hb)) & ((1u << hb) - 1u);
    const uint32_t lead = lead_decode(lc >> cb);
    uint32_t center = lc & ((1u << cb) - 1u);
    if (center == 0) center = 1u << cb;
    if (lead + center > 64) return EBI_E_CORRUPT;
    const uint32_t trail = 64 - lead - center;
    const uint64_t q = p + 2 + hb;
    if (flag == 2 && center == 1) {
        r.delta = 1ull << trail;
        s.pos = q;
    } else {
        if (q + center - 1 > B) return EBI_E_UNEXPECTED_END;
        r.delta = ((take_bits(peek, q, center - 1) << 1) | 1u) << trail;
        s.pos = q + center - 1;
    }
    s.win = lead | (trail << 8);
    return 0;
}

// Length-only step of one Chimp / Chimp128 record (the convergence rounds of
// the segment parse need positions and windows, not payloads): selects
// instead of branches, one 64-bit read.  Same errors as parse_rec.
template <int CODEC, typename Peek>
XOR_HD uint32_t step_len(Peek peek, uint64_t B, PState& s) {
    const uint64_t p = s.pos;
    if (p + 2 > B) return EBI_E_UNEXPECTED_END;
    const uint64_t x = peek(p);
    const uint32_t flag = static_cast<uint32_t>(x >> 62);
    constexpr uint32_t hdr1 = CODEC == CODEC_CHIMP128 ? 16u : 9u;  // '01' header after the flag
    const uint32_t t1 = static_cast<uint32_t>(x >> (62 - hdr1)) & ((1u << hdr1) - 1u);
    const uint32_t lead1 = lead_decode((t1 >> 6) & 7u);
    const uint32_t sig1 = (t1 & 63u) ? (t1 & 63u) : 64u;
    const uint32_t lead3 = lead_decode(static_cast<uint32_t>(x >> 59) & 7u);
    const uint32_t lead = s.win;
    // header bits (flag included) and total length per flag
    const uint32_t hdr = flag == 0 ? (CODEC == CODEC_CHIMP128 ? 9u : 2u) : flag == 1 ? 2 + hdr1 : flag == 2 ? 2u : 5u;
    const uint32_t body = flag == 0 ? 0u : flag == 1 ? sig1 : flag == 2 ? 64u - (lead > 64 ? 0u : lead) : 64u - lead3;
    const bool corrupt = (flag == 1 && sig1 + lead1 > 64) || (flag == 2 && lead > 64);
    if (flag != 2 && p + hdr > B) return EBI_E_UNEXPECTED_END;
    if (corrupt) return EBI_E_CORRUPT;
    if (p + hdr + body > B) return EBI_E_UNEXPECTED_END;
    s.win = flag == 1 ? lead1 : flag == 3 ? lead3 : lead;
    s.pos = p + hdr + body;
    return 0;
}

// Parses the records that start in [s.pos, end).  Counts the records before
// the first failure (*fail = its error) and, when it fails, steps one bit and
// goes on: a failing segment is either the true end of the stream or a
// misaligned guess, and a misaligned parse should keep looking for the true
// record boundaries.  The last segment fails at the end of the stream.
template <int CODEC, typename Peek>
XOR_HD PState parse_segment(Peek peek, uint64_t B, PState s, uint64_t end, bool last, uint32_t* n_out,
                            uint32_t* fail) {
    uint32_t n = 0, f = 0;
    while (s.pos < end) {
        uint32_t e;
        if (CODEC == CODEC_GORILLA || is_elf(CODEC)) {
            Rec r;
            e = parse_rec<CODEC>(peek, B, s, r);
        } else {
            e = step_len<CODEC>(peek, B, s);
        }
        if (e) {
            if (!f) f = e;
            s.pos += 1;
            continue;
        }
        n += f ? 0u : 1u;
    }
    if (last && !f) f = EBI_E_UNEXPECTED_END;
    *n_out = n;
    *fail = f;
    return s;
}

// Ring slot -> record index: the latest record j < i with j % 128 == slot, or
// kNoRef when the slot was never written (the ring starts zeroed).
XOR_HD uint32_t ring_ref(uint32_t i, uint32_t slot) {
    const int32_t j = static_cast<int32_t>(i) - 1 - static_cast<int32_t>((i - 1u - slot) & 127u);
    return j < 0 ? kNoRef : static_cast<uint32_t>(j);
}


}  // namespace xorp
}  // namespace ebi
