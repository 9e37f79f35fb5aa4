// Host emulation of the warp-per-chunk XOR decode (ebi_gb300/csrc/xor_lanes.h,
// driven as ebi_gb300/csrc/xor_warp.cuh drives it on the device), lane after
// lane, against the sequential reader built from the same record parser.
// Test infrastructure: compiled and loaded by tests/test_xor_lanes_emu.py.
//
//   warp    the 32-lane algorithm: segment parse rounds, chain starts (XOR
//           scan / Chimp128 ring composition), the end-marker pass and the
//           value pass (rings rotated as on the device), plus the
//           single-pass variant (end marker found by the query pass);
//   serial  the reader's own loop (one record after another, parse_rec).
// Both return the decoded stream up to its end marker as (value bits, Elf
// record flags, beta* in force) triples, or the chunk's error.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "xor_lanes.h"

using namespace ebi::xorp;

namespace {

struct Peek {
    const uint8_t* b;  // padded by at least 16 bytes
    uint64_t operator()(uint64_t p) const {
        const uint64_t byte = p >> 3;
        const uint32_t sh = static_cast<uint32_t>(p & 7);
        uint64_t hi = 0;
        for (int i = 0; i < 8; ++i) hi = (hi << 8) | b[byte + i];
        const uint64_t nx = b[byte + 8];
        return sh ? (hi << sh) | (nx >> (8 - sh)) : hi;
    }
    // the bit source of xor_lanes.h
    uint64_t peek(uint64_t p) const { return (*this)(p); }
    uint64_t peek2(uint64_t p, uint32_t& y) const {
        y = static_cast<uint32_t>((*this)(p + 64) >> 32);
        return (*this)(p);
    }
};

struct Out {
    uint64_t* v;
    uint8_t* meta;
    int32_t* beta;
    uint64_t cap, n;
    void push(uint64_t x, uint8_t m, int32_t b) {
        if (n < cap) {
            v[n] = x;
            meta[n] = m;
            beta[n] = b;
        }
        ++n;
    }
};

template <int CODEC>
uint32_t serial(const Peek& peek, uint64_t B, Out& out) {
    if (is_elf(CODEC)) {
        PState s{0, start_win(CODEC)};
        uint64_t v = 0;
        int32_t beta = INT32_MAX;
        for (;;) {
            Rec r;
            const uint32_t e = parse_rec<CODEC>(peek, B, s, r);
            if (e) return e;
            v ^= r.delta;
            if (v == 0x7ff8000000000000ull) return 0;
            if (r.meta & ebi::kElfBeta) beta = r.meta & 15;
            out.push(v, r.meta, beta);
        }
    }
    if (B < 64) return EBI_E_UNEXPECTED_END;
    uint64_t v = peek(0);
    PState s{64, start_win(CODEC)};
    uint64_t ring[128] = {0};
    uint32_t cur = 0;
    ring[0] = v;
    bool check = true;
    for (;;) {
        if (check && v == 0x7ff8000000000000ull) return 0;
        out.push(v, 0, INT32_MAX);
        Rec r;
        const uint32_t e = parse_rec<CODEC>(peek, B, s, r);
        if (e) return e;
        if (CODEC == CODEC_CHIMP128) {
            v = (r.ring == kRefPrev ? v : ring[r.ring]) ^ r.delta;
            cur = (cur + 1) & 127u;
            ring[cur] = v;
        } else {
            v ^= r.delta;
        }
        check = r.nan_ok;
    }
}

struct Rows {
    std::vector<uint64_t> v;
    std::vector<uint8_t> m;
    std::vector<int32_t> b;
};

template <int CODEC, typename P>
uint32_t warp(const Peek& peek_in, uint64_t B64, Out& out, bool single_pass, uint32_t* rounds_out) {
    Peek pk = peek_in;
    const P B = static_cast<P>(B64);
    constexpr bool kElf = is_elf(CODEC);
    constexpr bool kRing = CODEC == CODEC_CHIMP128;
    if (!kElf && B64 < 64) return EBI_E_UNEXPECTED_END;
    LaneParse<P> L[kLanes];
    P beg[kLanes], end[kLanes], thr[kLanes][kCps];
    for (int l = 0; l < kLanes; ++l) {
        lane_segment<P>(B, CODEC, l, beg[l], end[l], thr[l]);
        L[l].in = l == 0 ? PStateT<P>{static_cast<P>(first_bits(CODEC)), start_win(CODEC)} : PStateT<P>{beg[l], 0u};
        lane_parse<CODEC>(pk, B, end[l], l == kLanes - 1, thr[l], L[l], false, L[l]);
    }
    uint32_t ff = 0, rounds = 0;
    for (int round = 0; round < kLanes; ++round) {
        bool stale[kLanes];
        uint64_t prev[kLanes];
        bool any = false;
        for (int l = 0; l < kLanes; ++l) {
            prev[l] = l ? (uint64_t(L[l - 1].out.pos) | (uint64_t(L[l - 1].out.win) << 48)) : 0;
            stale[l] = l > 0 && (uint64_t(L[l].in.pos) | (uint64_t(L[l].in.win) << 48)) != prev[l];
            any = any || stale[l];
        }
        if (!any) break;
        ++rounds;
        for (int l = 0; l < kLanes; ++l) {
            if (!stale[l]) continue;
            const LaneParse<P> old = L[l];
            L[l].in = PStateT<P>{static_cast<P>(prev[l] & ((1ull << 48) - 1)), static_cast<uint32_t>(prev[l] >> 48)};
            lane_parse<CODEC>(pk, B, end[l], l == kLanes - 1, thr[l], L[l], true, old);
        }
    }
    *rounds_out = rounds;
    ff = kLanes;
    for (int l = kLanes - 1; l >= 0; --l)
        if (L[l].fail) ff = l;
    const uint32_t fail_status = ff < kLanes ? L[ff].fail : 0;
    uint32_t cnt[kLanes], off[kLanes], acc = 0;
    for (int l = 0; l < kLanes; ++l) {
        const bool head = !kElf && l == 0;
        cnt[l] = (static_cast<uint32_t>(l) > ff ? 0u : L[l].n) + (head ? 1u : 0u);
        off[l] = acc;
        acc += cnt[l];
    }
    uint64_t prefix[kLanes] = {0};
    int32_t beta_in[kLanes];
    std::vector<uint64_t> rx(kLanes * kRingSlots);
    std::vector<uint8_t> re(kLanes * kRingSlots);
    if (!kRing) {
        uint64_t run = 0;
        int32_t last_beta = INT32_MAX;
        for (int l = 0; l < kLanes; ++l) {
            const bool head = !kElf && l == 0;
            uint64_t x;
            uint32_t bl;
            lane_xor_total<CODEC>(pk, B, L[l].in, cnt[l] - (head ? 1u : 0u), head, x, bl);
            prefix[l] = run;
            beta_in[l] = last_beta;
            run ^= x;
            if (bl != 0xffu) last_beta = static_cast<int32_t>(bl);
        }
    } else {
        for (uint32_t k = 0; k < kRingSlots; ++k) RingView{rx.data(), re.data(), 0}.put(k, 0);
        for (int l = 0; l + 1 < kLanes; ++l)
            lane_syms(pk, B, L[l].in, cnt[l], l == 0, off[l], RingView{rx.data(), re.data(), uint32_t(l) + 1u});
        for (uint32_t l = 0; l + 1 < kLanes; ++l) {
            const RingView dst{rx.data(), re.data(), l + 1}, src{rx.data(), re.data(), l};
            for (uint32_t k = 0; k < kRingSlots; ++k) compose_slot(dst, src, k);
        }
        for (int l = 0; l < kLanes; ++l) beta_in[l] = INT32_MAX;
    }
    int pass = 0;
    std::vector<Rows> rows(kLanes);
    auto walk_all = [&](const uint32_t* lim, uint32_t* nan_j, bool collect) {
        if (kRing && pass > 0) {
            const RingView z{rx.data(), re.data(), static_cast<uint32_t>(kLanes - pass) & (kLanes - 1)};
            for (uint32_t k = 0; k < kRingSlots; ++k) z.put(k, 0);
        }
        for (int l = 0; l < kLanes; ++l) {
            rows[l] = Rows{};
            Rows& R = rows[l];
            auto sink = [&](uint32_t, uint64_t v, uint8_t m, int32_t b) {
                if (collect) {
                    R.v.push_back(v);
                    R.m.push_back(m);
                    R.b.push_back(b);
                }
            };
            const RingView rv{rx.data(), re.data(), static_cast<uint32_t>(l - pass) & (kLanes - 1)};
            nan_j[l] = lane_values<CODEC>(pk, B, L[l].in, lim[l], !kElf && l == 0, off[l], prefix[l], beta_in[l],
                                          kRing ? &rv : nullptr, sink);
        }
        ++pass;
    };
    uint32_t lim[kLanes], nan_j[kLanes];
    for (int l = 0; l < kLanes; ++l) lim[l] = cnt[l];
    auto find_end = [&]() -> bool {
        for (int l = 0; l < kLanes; ++l) {
            if (nan_j[l] < cnt[l]) {
                const uint32_t e = off[l] + nan_j[l];
                for (int m = 0; m < kLanes; ++m) lim[m] = e > off[m] ? std::min(e - off[m], cnt[m]) : 0u;
                return true;
            }
        }
        return false;
    };
    if (!single_pass) {
        walk_all(lim, nan_j, false);
        if (!find_end()) return fail_status ? fail_status : EBI_E_UNEXPECTED_END;
        walk_all(lim, nan_j, true);
    } else {
        walk_all(lim, nan_j, true);
        if (!find_end()) return fail_status ? fail_status : EBI_E_UNEXPECTED_END;
        // lanes past the end marker drop what they produced; the lane holding it stopped there
        for (int l = 0; l < kLanes; ++l)
            if (lim[l] == 0) rows[l] = Rows{};
    }
    for (int l = 0; l < kLanes; ++l)
        for (size_t j = 0; j < rows[l].v.size() && j < lim[l]; ++j) out.push(rows[l].v[j], rows[l].m[j], rows[l].b[j]);
    return 0;
}

template <int CODEC>
uint32_t run(int which, const Peek& peek, uint64_t B, Out& out, uint32_t* rounds) {
    if (which == 0) return serial<CODEC>(peek, B, out);
    if (which == 3) return warp<CODEC, uint64_t>(peek, B, out, false, rounds);  // 64-bit positions
    return warp<CODEC, uint32_t>(peek, B, out, which == 2, rounds);
}

}  // namespace

extern "C" {

// which: 0 sequential reader, 1 warp algorithm (end-marker pass first), 2 warp algorithm (single pass),
// 3 warp algorithm with 64-bit positions.
// codec: EBI_CHIMP, EBI_CHIMP128, EBI_ELF_ON_CHIMP or EBI_ELF.  Returns the chunk's status (0: OK).
uint32_t emu_decode(int which, int codec, const uint8_t* chunk, uint64_t len, uint64_t* vals, uint8_t* meta,
                    int32_t* beta, uint64_t cap, uint64_t* n_out, uint32_t* rounds) {
    std::vector<uint8_t> buf(chunk, chunk + len);
    buf.resize(len + 32, 0);
    const Peek peek{buf.data()};
    Out out{vals, meta, beta, cap, 0};
    uint32_t r = 0, st;
    const uint64_t B = len * 8;
    switch (codec) {
    case CODEC_CHIMP: st = run<CODEC_CHIMP>(which, peek, B, out, &r); break;
    case CODEC_CHIMP128: st = run<CODEC_CHIMP128>(which, peek, B, out, &r); break;
    case CODEC_ELF_CHIMP: st = run<CODEC_ELF_CHIMP>(which, peek, B, out, &r); break;
    case CODEC_ELF: st = run<CODEC_ELF>(which, peek, B, out, &r); break;
    default: return 0xffffffffu;
    }
    *n_out = out.n;
    if (rounds) *rounds = r;
    return st;
}

}  // extern "C"
