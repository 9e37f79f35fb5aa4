// encoder.cpp -- host-side EBI1 writer: Encoder::encode (api/encoder.rs:140-178)
// with FileWriter / ChunkWriter framing (encoder.rs:190-529) and the chunk
// encoders of the codecs this engine decodes:
//   Uncompressed (compressor/uncompressed.rs), RLE (compressor/run_length.rs:49-117),
//   Gorilla (compressor/gorilla.rs:118-190), Chimp (compressor/chimp.rs:51-146),
//   Chimp128 (compressor/chimp_n.rs:126-258), BUFF (compressor/buff.rs:127-307),
//   Elf and ElfOnChimp (compressor/elf.rs: ElfEncoderWrapper over ElfXorEncoder
//   or ChimpEncoder).
// Output bytes equal the reference's except the two wall-clock timing fields
// of FileFooter3, written here as zero.
#include <algorithm>
#include <cmath>
#include <new>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/ebi_gpu.h"
#include "elf_host.h"

namespace {

using Bytes = std::vector<uint8_t>;
constexpr uint64_t kNan = 0x7ff8000000000000ull;

inline uint64_t bits_of(double d) { uint64_t u; std::memcpy(&u, &d, 8); return u; }
inline int lz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }
inline int tz64(uint64_t x) { return x ? __builtin_ctzll(x) : 64; }
void put32(Bytes& b, uint32_t v) { for (int i = 0; i < 4; ++i) b.push_back(uint8_t(v >> (8 * i))); }
void put64(Bytes& b, uint64_t v) { for (int i = 0; i < 8; ++i) b.push_back(uint8_t(v >> (8 * i))); }

// MSB-first bit writer (io/bit_write.rs:46-64, 226-286).
class BitWriter {
  public:
    void bit(bool b) {
        if (pos_ == 8) { buf_.push_back(0); pos_ = 0; }
        if (b) buf_.back() |= uint8_t(1u << (7 - pos_));
        ++pos_;
    }
    void byte(uint8_t v) {
        if (pos_ == 8) { buf_.push_back(v); return; }
        buf_.back() |= uint8_t(v >> pos_);
        buf_.push_back(uint8_t(v << (8 - pos_)));
    }
    void bits(uint64_t v, unsigned n) {
        while (n >= 8) { byte(uint8_t(v >> (n - 8))); n -= 8; }
        for (int i = int(n) - 1; i >= 0; --i) bit((v >> i) & 1);
    }
    Bytes& out() { return buf_; }

  private:
    Bytes buf_;
    int pos_ = 8;
};

const uint8_t kRepr[64] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 7, 7, 7, 7, 7, 7,
                           7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7};
inline uint32_t lead_round(int lz) {
    static const uint8_t r[8] = {0, 8, 12, 16, 18, 20, 22, 24};
    return r[kRepr[lz]];
}

void gorilla(BitWriter& w, const double* v, uint64_t n) {
    uint64_t prev = 0;
    uint32_t lead = 64, trail = 64;
    for (uint64_t i = 0; i <= n; ++i) {
        const uint64_t x = i < n ? bits_of(v[i]) : kNan;  // close(): NaN end marker
        if (i == 0) { w.bits(x, 64); prev = x; continue; }
        const uint64_t d = x ^ prev;
        prev = x;
        if (!d) { w.bit(false); continue; }
        w.bit(true);
        uint32_t lz = std::min<uint32_t>(uint32_t(lz64(d)), 31), tz = uint32_t(tz64(d));
        if (lz >= lead && tz >= trail) {
            w.bit(false);
            w.bits(d >> trail, 64 - lead - trail);
        } else {
            w.bit(true);
            w.bits(lz, 5);
            const uint32_t sig = 64 - lz - tz;
            w.bits(sig - 1, 6);
            w.bits(d >> tz, sig);
            lead = lz;
            trail = tz;
        }
    }
    w.bit(false);
}

void chimp(BitWriter& w, const double* v, uint64_t n) {
    uint64_t prev = 0;
    uint32_t stored = 0xffffffffu;
    for (uint64_t i = 0; i <= n; ++i) {
        const uint64_t x = i < n ? bits_of(v[i]) : kNan;
        if (i == 0) { w.bits(x, 64); prev = x; continue; }
        const uint64_t d = prev ^ x;
        if (!d) {
            w.bits(0, 2);
            stored = 65;
        } else {
            const uint32_t lead = lead_round(lz64(d)), trail = uint32_t(tz64(d));
            if (trail > 6) {
                const uint32_t sig = 64 - lead - trail;
                w.bits(1, 2);
                w.bits(kRepr[lead], 3);
                w.bits(sig, 6);
                w.bits(d >> trail, sig);
                stored = 65;
            } else if (lead == stored) {
                w.bits(2, 2);
                w.bits(d, 64 - lead);
            } else {
                stored = lead;
                w.bits(3, 2);
                w.bits(kRepr[lead], 3);
                w.bits(d, 64 - lead);
            }
        }
        prev = x;
    }
    w.bit(false);
}

void chimp128(BitWriter& w, const double* v, uint64_t n) {
    constexpr uint64_t N = 128, kLsb = (1u << 14) - 1;
    std::vector<uint64_t> ring(N, 0), index_of(kLsb + 1, 0);
    uint32_t stored = 0xffffffffu;
    uint64_t index = 0, cur = 0;
    for (uint64_t i = 0; i <= n; ++i) {
        const uint64_t x = i < n ? bits_of(v[i]) : kNan;
        if (i == 0) {
            ring[0] = x;
            w.bits(x, 64);
            index_of[x & kLsb] = 0;
            continue;
        }
        const uint64_t key = x & kLsb;
        uint64_t d, prev;
        uint32_t trailing = 0;
        const uint64_t ci = index_of[key];
        if (index - ci < N) {
            const uint64_t t = x ^ ring[ci % N];
            trailing = uint32_t(tz64(t));
            if (trailing > 13) { prev = ci % N; d = t; }
            else { prev = index % N; d = ring[prev] ^ x; }
        } else {
            prev = index % N;
            d = ring[prev] ^ x;
        }
        if (!d) {
            w.bits(prev, 9);
            stored = 65;
        } else {
            const uint32_t lead = lead_round(lz64(d));
            if (trailing > 13) {
                const uint32_t sig = 64 - lead - trailing;
                w.bits(512ull * (N + prev) + 64ull * kRepr[lead] + sig, 18);
                w.bits(d >> trailing, sig);
                stored = 65;
            } else if (lead == stored) {
                w.bits(2, 2);
                w.bits(d, 64 - lead);
            } else {
                stored = lead;
                w.bits(24ull + kRepr[lead], 5);
                w.bits(d, 64 - lead);
            }
        }
        cur = (cur + 1) % N;
        ring[cur] = x;
        ++index;
        index_of[key] = index;
    }
    w.bit(false);
}

// ChimpEncoder value by value (compressor/chimp.rs:51-146), the inner
// stream of ElfOnChimp.
struct ChimpStream {
    uint64_t prev = 0;
    uint32_t stored = 0xffffffffu;
    bool first = true;
    void add(BitWriter& w, uint64_t x) {
        if (first) { first = false; prev = x; w.bits(x, 64); return; }
        const uint64_t d = prev ^ x;
        if (!d) {
            w.bits(0, 2);
            stored = 65;
        } else {
            const uint32_t lead = lead_round(lz64(d)), trail = uint32_t(tz64(d));
            if (trail > 6) {
                const uint32_t sig = 64 - lead - trail;
                w.bits(1, 2);
                w.bits(kRepr[lead], 3);
                w.bits(sig, 6);
                w.bits(d >> trail, sig);
                stored = 65;
            } else if (lead == stored) {
                w.bits(2, 2);
                w.bits(d, 64 - lead);
            } else {
                stored = lead;
                w.bits(3, 2);
                w.bits(kRepr[lead], 3);
                w.bits(d, 64 - lead);
            }
        }
        prev = x;
    }
};

// ElfXorEncoder (compressor/elf.rs:164-262).
struct ElfXorStream {
    uint64_t prev = 0;
    uint32_t lead = 0xffffffffu, trail = 0xffffffffu;
    bool first = true;
    void add(BitWriter& w, uint64_t x) {
        if (first) {  // write_first: trailing zeros, then the bits above the lowest set one
            first = false;
            prev = x;
            const uint32_t tz = uint32_t(tz64(x));
            w.bits(tz, 7);
            if (tz < 63) w.bits(x >> (tz + 1), 63 - tz);
            return;
        }
        const uint64_t d = prev ^ x;
        if (!d) { w.bits(1, 2); return; }  // '01': the same value
        const uint32_t l = lead_round(lz64(d)), t = uint32_t(tz64(d));
        if (l == lead && t >= trail) {  // '00': the stored window
            w.bits(0, 2);
            w.bits(d >> trail, 64 - lead - trail);
        } else {
            lead = l;
            trail = t;
            const uint32_t center = 64 - l - t;
            if (center <= 16) {  // '10' + 3-bit leading code + 4-bit center
                w.bits((((2u << 3) | kRepr[l]) << 4) | (center & 15u), 9);
                if (center > 1) w.bits(d >> (t + 1), center - 1);
            } else {             // '11' + 3-bit leading code + 6-bit center
                w.bits((((3u << 3) | kRepr[l]) << 6) | (center & 63u), 11);
                w.bits(d >> (t + 1), center - 1);
            }
        }
        prev = x;
    }
};

// ElfEncoderWrapper::add_value (compressor/elf.rs:92-158): values whose
// decimal digits allow it lose their low mantissa bits (v'), which the
// reader restores from beta*, the number of significant decimal digits.
template <typename Inner>
void elf(BitWriter& w, const double* v, uint64_t n) {
    Inner inner;
    int32_t last = INT32_MAX;
    for (uint64_t i = 0; i < n; ++i) {
        const double x = v[i];
        const uint64_t b = bits_of(x);
        uint64_t vp = b;
        bool erased = false;
        if (x == 0.0 || std::isinf(x)) {
        } else if (x != x) {
            vp = kNan;
        } else {
            bool pow10 = false;
            const double a = std::fabs(x);
            const int32_t sp = ebi::elf::sp_of(a, &pow10);
            const int32_t beta = ebi::elf::significant(a, sp, last);
            const uint32_t alpha = uint32_t(int64_t(beta) - sp - 1);
            const int32_t beta_star = pow10 ? 0 : beta;
            if (beta_star < 16) {
                const uint32_t g = ebi::elf::f_alpha(alpha) + uint32_t((b >> 52) & 0x7ff) - 1023u;
                const int32_t erase = 52 - int32_t(g);
                if (erase > 4) {
                    const uint64_t mask = ~0ull << (erase & 63);
                    if (b & ~mask) {
                        erased = true;
                        vp = b & mask;
                        if (beta_star == last) {
                            w.bit(false);  // '0': the stored beta*
                        } else {
                            w.bits(uint32_t(beta_star) | 0x30u, 6);  // '11' + beta*
                            last = beta_star;
                        }
                    }
                }
            }
        }
        if (!erased) w.bits(2, 2);  // '10': the value as is
        inner.add(w, vp);
    }
    w.bits(2, 2);  // close: '10', the NaN end marker, one 0 bit
    inner.add(w, kNan);
    w.bit(false);
}

int64_t buff_fixed(double value, int32_t frac) {
    const uint64_t vb = bits_of(value);
    const int32_t exp = int32_t((vb >> 52) & 0x7ff) - 1023;
    if (exp < -frac) return 0;
    const int64_t s = 63 - int64_t(exp) - frac;
    uint64_t f = s >= 64 ? 0 : (((vb << 11) | 0x8000000000000000ull) >> (uint64_t(s) & 63));
    if (vb >> 63) f = ~(f - 1);
    return int64_t(f);
}

int buff(Bytes& o, const double* v, uint64_t n, uint64_t scale) {
    static const uint32_t kMap[13] = {0, 5, 8, 11, 15, 18, 21, 25, 28, 31, 35, 38, 50};
    const int prec = scale == 0 ? 0 : std::max(0, int(std::log10(float(scale))));
    if (prec > 12) return EBI_E_INVALID;
    const uint32_t frac = kMap[prec];
    std::vector<int64_t> fx(n);
    uint64_t imin = 0, imax = 0;
    for (uint64_t i = 0; i < n; ++i) {
        fx[i] = buff_fixed(v[i], int32_t(frac));
        if (fx[i] < fx[imin]) imin = i;
        if (fx[i] > fx[imax]) imax = i;
    }
    const int64_t base = fx[imin];
    const uint64_t span = uint64_t(fx[imax]) - uint64_t(base);
    const uint32_t bits = span ? uint32_t(64 - lz64(span)) : 0;
    put32(o, uint32_t(uint64_t(base)));
    put32(o, uint32_t(uint64_t(base) >> 32));
    put32(o, uint32_t(n));
    put32(o, bits);
    put32(o, frac);
    uint32_t rem = bits;
    if (!(rem > 0 && rem < 8)) {
        while (rem >= 8) {
            rem -= 8;
            for (uint64_t i = 0; i < n; ++i) o.push_back(uint8_t(uint8_t((uint64_t(fx[i]) - uint64_t(base)) >> rem) ^ 0x80));
        }
    }
    if (rem > 0) {  // LSB-first tail of `rem` bits per row
        const size_t at = o.size();
        o.resize(at + std::max<uint64_t>(1, (n * rem + 7) / 8), 0);
        for (uint64_t i = 0; i < n; ++i) {
            const uint32_t d = uint32_t(uint64_t(fx[i]) - uint64_t(base)) & ((1u << rem) - 1);
            for (uint32_t b = 0; b < rem; ++b) {
                const uint64_t bp = i * rem + b;
                if ((d >> b) & 1) o[at + (bp >> 3)] |= uint8_t(1u << (bp & 7));
            }
        }
    }
    return EBI_OK;
}

void rle(Bytes& o, const double* v, uint64_t n) {
    const size_t hdr = o.size();
    put64(o, 0);
    uint64_t fields = 0;
    if (n) {
        uint64_t pv = bits_of(v[0]);
        uint32_t run = 1;
        auto field = [&](uint32_t r, uint64_t x) { o.push_back(uint8_t(r)); put64(o, x); ++fields; };
        for (uint64_t i = 1; i < n; ++i) {
            const uint64_t x = bits_of(v[i]);
            if (x == pv && run < 255) { ++run; continue; }
            field(run, pv);
            pv = x;
            run = 1;
        }
        field(run, pv);
    }
    for (int i = 0; i < 8; ++i) o[hdr + i] = uint8_t(fields >> (8 * i));
}

int chunk(Bytes& o, const double* v, uint64_t n, int scheme, uint64_t scale) {
    switch (scheme) {
        case EBI_UNCOMPRESSED: for (uint64_t i = 0; i < n; ++i) put64(o, bits_of(v[i])); return EBI_OK;
        case EBI_RLE: rle(o, v, n); return EBI_OK;
        case EBI_BUFF: return buff(o, v, n, scale);
        case EBI_GORILLA: case EBI_CHIMP: case EBI_CHIMP128: case EBI_ELF_ON_CHIMP: case EBI_ELF: {
            BitWriter w;
            if (scheme == EBI_GORILLA) gorilla(w, v, n);
            else if (scheme == EBI_CHIMP) chimp(w, v, n);
            else if (scheme == EBI_CHIMP128) chimp128(w, v, n);
            else if (scheme == EBI_ELF_ON_CHIMP) elf<ChimpStream>(w, v, n);
            else elf<ElfXorStream>(w, v, n);
            o.insert(o.end(), w.out().begin(), w.out().end());
            return EBI_OK;
        }
        default: return EBI_E_UNSUPPORTED;
    }
}

}  // namespace

extern "C" int ebi_encode(const double* v, uint64_t n, int scheme, int kind, uint64_t value, uint64_t scale,
                          uint8_t** out, uint64_t* out_len) {
    if (!out || !out_len || (!v && n) || scheme < 0 || scheme > EBI_ELF || kind < 0 || kind > 2) return EBI_E_INVALID;
    try {
        Bytes o;
        o.insert(o.end(), {'E', 'B', 'I', '1', 0, uint8_t(scheme), uint8_t(kind), 0});
        put64(o, kind == EBI_CHUNK_FULL ? 0 : value);
        put64(o, 0);  // footer offset
        for (uint16_t x : {uint16_t(0), uint16_t(1), uint16_t(14)}) { o.push_back(uint8_t(x)); o.push_back(uint8_t(x >> 8)); }
        const uint64_t per = kind == EBI_CHUNK_FULL ? n : kind == EBI_CHUNK_RECORD_COUNT ? value
                                                    : uint64_t(std::ceil((double(value) / 8.0) * 1.5));
        std::vector<uint64_t> foot;
        uint64_t pos = 0;
        while (per > 0 && pos < n) {
            const uint64_t take = std::min(per, n - pos);
            foot.push_back(o.size());
            foot.push_back(pos);
            const int st = chunk(o, v + pos, take, scheme, scale);
            if (st) return st;
            pos += take;
        }
        const uint64_t footer = o.size();
        put64(o, pos);
        put64(o, foot.size() / 2);
        for (uint64_t x : foot) put64(o, x);
        o.push_back(8);
        put64(o, scheme == EBI_BUFF ? scale : 8192);
        o.resize(o.size() + 16 + 9 * 16 + 4, 0);
        for (int i = 0; i < 8; ++i) o[16 + i] = uint8_t(footer >> (8 * i));  // offset_of!(FileHeader, footer_offset)
        uint8_t* m = static_cast<uint8_t*>(std::malloc(o.size() ? o.size() : 1));
        if (!m) return EBI_E_OOM;
        std::memcpy(m, o.data(), o.size());
        *out = m;
        *out_len = o.size();
        return EBI_OK;
    } catch (const std::bad_alloc&) {
        return EBI_E_OOM;
    }
}

extern "C" void ebi_free(void* p) { std::free(p); }
