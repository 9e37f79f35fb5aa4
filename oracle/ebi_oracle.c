/*
 * ebi_oracle.c -- CPU restatement of lemolatoon/ebi's chunked decode-and-query
 * path.  TEST INFRASTRUCTURE ONLY (see ebi_oracle.h): the parity checker for
 * the GPU engine and the timed CPU baseline.  Every function names the
 * reference file:line it restates.  All arithmetic follows the reference's
 * release-build semantics (wrapping integer arithmetic); where the reference
 * would panic in a debug build on a malformed stream, this file returns
 * ORA_E_CORRUPT or ORA_E_UNEXPECTED_END instead.
 */
#include "ebi_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define NAN_BITS 0x7ff8000000000000ull /* f64::NAN.to_bits() */

/* ------------------------------------------------------------------------ */
/* small helpers                                                             */
/* ------------------------------------------------------------------------ */
static inline uint64_t f2u(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }
static inline double u2f(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static inline int clz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }
static inline int ctz64(uint64_t x) { return x ? __builtin_ctzll(x) : 64; }
static inline uint32_t rd_u32le(const uint8_t* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
static inline uint64_t rd_u64le(const uint8_t* p) {
    return (uint64_t)rd_u32le(p) | ((uint64_t)rd_u32le(p + 4) << 32);
}
static inline int mask_test(const uint64_t* m, uint64_t nbits, uint64_t r) {
    return r < nbits && ((m[r >> 6] >> (r & 63)) & 1);
}
static inline void bit_set(uint64_t* m, uint64_t r) { m[r >> 6] |= 1ull << (r & 63); }

/* growable byte buffer */
typedef struct { uint8_t* p; size_t len, cap; int oom; } obuf;
static void ob_reserve(obuf* b, size_t extra) {
    if (b->oom || b->len + extra <= b->cap) return;
    size_t nc = b->cap ? b->cap * 2 : 256;
    while (nc < b->len + extra) nc *= 2;
    uint8_t* np = (uint8_t*)realloc(b->p, nc);
    if (!np) { b->oom = 1; return; }
    b->p = np; b->cap = nc;
}
static void ob_push(obuf* b, const void* s, size_t n) {
    ob_reserve(b, n);
    if (b->oom) return;
    memcpy(b->p + b->len, s, n); b->len += n;
}
static void ob_u8(obuf* b, uint8_t v) { ob_push(b, &v, 1); }
static void ob_u16(obuf* b, uint16_t v) { uint8_t t[2] = {(uint8_t)v, (uint8_t)(v >> 8)}; ob_push(b, t, 2); }
static void ob_u32(obuf* b, uint32_t v) {
    uint8_t t[4] = {(uint8_t)v, (uint8_t)(v >> 8), (uint8_t)(v >> 16), (uint8_t)(v >> 24)};
    ob_push(b, t, 4);
}
static void ob_u64(obuf* b, uint64_t v) { ob_u32(b, (uint32_t)v); ob_u32(b, (uint32_t)(v >> 32)); }
static void ob_zero(obuf* b, size_t n) { ob_reserve(b, n); if (b->oom) return; memset(b->p + b->len, 0, n); b->len += n; }

/* ------------------------------------------------------------------------ */
/* MSB-first bit writer: BufferedBitWriter (io/bit_write.rs:46-64,226-286)   */
/* ------------------------------------------------------------------------ */
typedef struct { obuf b; int bit_pos; /* 8: the next write opens a new byte */ } bitw;
static void bw_init(bitw* w) { memset(w, 0, sizeof *w); w->bit_pos = 8; }
static void bw_bit(bitw* w, int bit) {                       /* bit_write.rs:240-252 */
    if (w->bit_pos == 8) { ob_u8(&w->b, 0); w->bit_pos = 0; }
    if (w->b.oom) return;
    if (bit) w->b.p[w->b.len - 1] |= (uint8_t)(1u << (7 - w->bit_pos));
    w->bit_pos++;
}
static void bw_byte(bitw* w, uint8_t byte) {                  /* bit_write.rs:278-286 */
    if (w->bit_pos == 8) { ob_u8(&w->b, byte); return; }
    if (w->b.oom) return;
    w->b.p[w->b.len - 1] |= (uint8_t)(byte >> w->bit_pos);
    ob_u8(&w->b, (uint8_t)(byte << (8 - w->bit_pos)));
}
static void bw_bits(bitw* w, uint64_t bits, unsigned num) {    /* bit_write.rs:46-64 */
    unsigned rem = num;
    while (rem >= 8) { bw_byte(w, (uint8_t)(bits >> (rem - 8))); rem -= 8; }
    if (rem > 0) {
        uint64_t v = bits & ((1ull << rem) - 1);
        for (int i = (int)rem - 1; i >= 0; --i) bw_bit(w, (int)((v >> i) & 1));
    }
}

/* ------------------------------------------------------------------------ */
/* MSB-first bit reader: BufferedBitReader::read_bits (io/bit_read.rs:293-318)*/
/* Returns 0 (None) when fewer than n bits remain.                           */
/* ------------------------------------------------------------------------ */
typedef struct { const uint8_t* buf; uint64_t len; uint64_t pos; } bitr;
static inline uint64_t peek64(const uint8_t* buf, uint64_t len, uint64_t bitpos) {
    uint64_t byte = bitpos >> 3;
    unsigned sh = (unsigned)(bitpos & 7);
    uint64_t hi = 0;
    for (int i = 0; i < 8; ++i) hi = (hi << 8) | (byte + i < len ? buf[byte + i] : 0);
    uint64_t nx = byte + 8 < len ? buf[byte + 8] : 0;
    return sh ? (hi << sh) | (nx >> (8 - sh)) : hi;
}
static inline int br_bits(bitr* r, unsigned n, uint64_t* out) {
    if (r->len * 8 - r->pos < n) return 0;
    if (n == 0) { *out = 0; return 1; }
    uint64_t w = peek64(r->buf, r->len, r->pos);
    *out = n == 64 ? w : (w >> (64 - n));
    r->pos += n;
    return 1;
}
int ora_read_bits(const uint8_t* buf, uint64_t len, uint64_t* bitpos, int n, uint64_t* out) {
    bitr r = {buf, len, *bitpos};
    if (n < 0 || n > 64) return 0;
    int ok = br_bits(&r, (unsigned)n, out);
    *bitpos = r.pos;
    return ok;
}

/* ------------------------------------------------------------------------ */
/* Gorilla encoder: modified_tsz::GorillaFloatEncoder                        */
/* (compressor/gorilla.rs:118-190, close = encode(NaN) + one 0 bit :27-30) */
/* ------------------------------------------------------------------------ */
static void gorilla_encode(bitw* w, const double* v, uint64_t n) {
    uint64_t value = 0;
    uint32_t lead = 64, trail = 64;  /* :262-263 sentinels */
    int first = 1;
    for (uint64_t i = 0; i <= n; ++i) {
        uint64_t bits = i < n ? f2u(v[i]) : NAN_BITS;
        if (first) {                                          /* write_first :293-301 */
            bw_bits(w, bits, 64);
            value = bits;
            first = 0;
            continue;
        }
        uint64_t x = bits ^ value;                            /* write_next_value :304-365 */
        value = bits;
        if (x == 0) { bw_bit(w, 0); continue; }
        bw_bit(w, 1);
        uint32_t lz = (uint32_t)clz64(x);
        if (lz >= 32) lz = 31;                                 /* 5-bit clamp :321-323 */
        uint32_t tz = (uint32_t)ctz64(x);
        if (lz >= lead && tz >= trail) {
            bw_bit(w, 0);
            bw_bits(w, x >> trail, 64 - lead - trail);
        } else {
            bw_bit(w, 1);
            bw_bits(w, lz, 5);
            uint32_t sig = 64 - lz - tz;
            bw_bits(w, sig - 1, 6);
            bw_bits(w, x >> tz, sig);
            lead = lz; trail = tz;
        }
    }
    bw_bit(w, 0);
}

/* ------------------------------------------------------------------------ */
/* Chimp encoder (compressor/chimp.rs:51-146)                                */
/* ------------------------------------------------------------------------ */
static const uint8_t LEAD_REPR[64] = {
    0,0,0,0,0,0,0,0,1,1,1,1,2,2,2,2,3,3,4,4,5,5,6,6,7,7,7,7,7,7,7,7,
    7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7,7};
static const uint8_t LEAD_ROUND[64] = {
    0,0,0,0,0,0,0,0,8,8,8,8,12,12,12,12,16,16,18,18,20,20,22,22,24,24,24,24,24,24,24,24,
    24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24,24};
static const uint32_t LEAD_DECODE[8] = {0, 8, 12, 16, 18, 20, 22, 24}; /* decoder/chunk_reader/chimp.rs:38 */

static void chimp_encode(bitw* w, const double* v, uint64_t n) {
    uint32_t stored_lead = 0xffffffffu;
    uint64_t stored = 0;
    int first = 1;
    for (uint64_t i = 0; i <= n; ++i) {
        uint64_t val = i < n ? f2u(v[i]) : NAN_BITS;          /* close :93-96 */
        if (first) { first = 0; stored = val; bw_bits(w, val, 64); continue; }
        uint64_t x = stored ^ val;                             /* compress_value :99-146 */
        if (x == 0) {
            bw_bit(w, 0); bw_bit(w, 0);
            stored_lead = 65;
        } else {
            uint32_t lead = LEAD_ROUND[clz64(x)];
            uint32_t trail = (uint32_t)ctz64(x);
            if (trail > 6) {
                uint32_t sig = 64 - lead - trail;
                bw_bit(w, 0); bw_bit(w, 1);
                bw_bits(w, LEAD_REPR[lead], 3);
                bw_bits(w, sig, 6);
                bw_bits(w, x >> trail, sig);
                stored_lead = 65;
            } else if (lead == stored_lead) {
                bw_bit(w, 1); bw_bit(w, 0);
                bw_bits(w, x, 64 - lead);
            } else {
                stored_lead = lead;
                bw_bit(w, 1); bw_bit(w, 1);
                bw_bits(w, LEAD_REPR[lead], 3);
                bw_bits(w, x, 64 - lead);
            }
        }
        stored = val;
    }
    bw_bit(w, 0);
}

/* ------------------------------------------------------------------------ */
/* Chimp128 encoder: ChimpNEncoder<128> (compressor/chimp_n.rs:126-258)       */
/* ------------------------------------------------------------------------ */
#define CN 128
#define CN_LOG2 7
#define CN_THRESHOLD (6 + CN_LOG2)             /* :140 */
#define CN_SET_LSB ((1u << (CN_THRESHOLD + 1)) - 1) /* :141 */
#define CN_FLAG_ZERO (CN_LOG2 + 2)             /* :142 */
#define CN_FLAG_ONE (CN_LOG2 + 11)             /* :143 */

static int chimp128_encode(bitw* w, const double* v, uint64_t n) {
    uint64_t* stored = (uint64_t*)calloc(CN, sizeof(uint64_t));
    uint64_t* indices = (uint64_t*)calloc((size_t)1 << (CN_THRESHOLD + 1), sizeof(uint64_t));
    if (!stored || !indices) { free(stored); free(indices); return ORA_E_OOM; }
    uint32_t stored_lead = 0xffffffffu;
    uint64_t index = 0, current = 0;
    int first = 1;
    for (uint64_t i = 0; i <= n; ++i) {
        uint64_t val = i < n ? f2u(v[i]) : NAN_BITS;           /* close :191-194 */
        if (first) {                                            /* write_first :183-189 */
            first = 0;
            stored[current] = val;
            bw_bits(w, val, 64);
            indices[val & CN_SET_LSB] = index;
            continue;
        }
        uint64_t key = val & CN_SET_LSB;                        /* compress_value :196-258 */
        uint64_t x, prev;
        uint32_t trailing = 0;
        uint64_t curr_index = indices[key];
        if (index - curr_index < CN) {
            uint64_t temp = val ^ stored[curr_index % CN];
            trailing = (uint32_t)ctz64(temp);
            if (trailing > CN_THRESHOLD) { prev = curr_index % CN; x = temp; }
            else { prev = index % CN; x = stored[prev] ^ val; }
        } else {
            prev = index % CN;
            x = stored[prev] ^ val;
        }
        if (x == 0) {
            bw_bits(w, prev, CN_FLAG_ZERO);
            stored_lead = 65;
        } else {
            uint32_t lead = LEAD_ROUND[clz64(x)];
            if (trailing > CN_THRESHOLD) {
                uint32_t sig = 64 - lead - trailing;
                bw_bits(w, 512ull * (CN + prev) + 64ull * LEAD_REPR[lead] + sig, CN_FLAG_ONE);
                bw_bits(w, x >> trailing, sig);
                stored_lead = 65;
            } else if (lead == stored_lead) {
                bw_bits(w, 2, 2);
                bw_bits(w, x, 64 - lead);
            } else {
                stored_lead = lead;
                bw_bits(w, 24ull + LEAD_REPR[lead], 5);
                bw_bits(w, x, 64 - lead);
            }
        }
        current = (current + 1) % CN;
        stored[current] = val;
        index += 1;
        indices[key] = index;
    }
    bw_bit(w, 0);
    free(stored); free(indices);
    return ORA_OK;
}

/* ------------------------------------------------------------------------ */
/* Elf decimal helpers (compression_common/elf.rs).  Rust's float -> int     */
/* casts saturate (NaN -> 0); integer arithmetic wraps as in release builds.  */
/* ------------------------------------------------------------------------ */
static const uint32_t ELF_F[21] = {0, 4, 7, 10, 14, 17, 20, 24, 27, 30, 34, 37, 40, 44, 47, 50, 54, 57, 60, 64, 67};
static int32_t sat_i32(double x) {
    if (x != x) return 0;
    if (x >= 2147483647.0) return INT32_MAX;
    if (x <= -2147483648.0) return INT32_MIN;
    return (int32_t)x;
}
static uint32_t sat_u32(double x) {
    if (x != x || x <= 0.0) return 0;
    if (x >= 4294967295.0) return UINT32_MAX;
    return (uint32_t)x;
}
static int64_t sat_i64(double x) {
    if (x != x) return 0;
    if (x >= 9223372036854775807.0) return INT64_MAX;
    if (x <= -9223372036854775808.0) return INT64_MIN;
    return (int64_t)x;
}
/* get_10i_p / get_10i_n (:97-113): the table, else "1.0E{i}".parse::<f64>() */
static const double ELF_10I_P[21] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9, 1e10,
                                     1e11, 1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20};
static const double ELF_10I_N[21] = {1e-0,  1e-1,  1e-2,  1e-3,  1e-4,  1e-5,  1e-6,  1e-7,  1e-8,  1e-9, 1e-10,
                                     1e-11, 1e-12, 1e-13, 1e-14, 1e-15, 1e-16, 1e-17, 1e-18, 1e-19, 1e-20};
static double elf_10i_p(uint32_t i) {
    if (i < 21) return ELF_10I_P[i];
    char b[32];
    snprintf(b, sizeof b, "1.0E%u", i);
    return strtod(b, NULL);
}
static double elf_10i_n(uint32_t i) {
    if (i < 21) return ELF_10I_N[i];
    char b[32];
    snprintf(b, sizeof b, "1.0E-%u", i);
    return strtod(b, NULL);
}
/* get_f_alpha (:33-39) */
static uint32_t elf_f_alpha(uint32_t alpha) {
    if (alpha < 21) return ELF_F[alpha];
    return sat_u32(ceil((double)alpha * 3.321928094887362347870319429489390175864831393));
}
/* get_sp (:115-133) and get_sp_and_10i_n_flag (:135-155) */
static int32_t elf_sp(double v, int* flag) {
    static const double GT[10] = {1, 10, 100, 1000, 10000, 100000, 1000000, 10000000, 100000000, 1000000000};
    static const double LT[11] = {1.0, 0.1, 0.01, 0.001, 0.0001, 0.00001, 0.000001, 0.0000001, 0.00000001,
                                  0.000000001, 0.0000000001};
    if (flag) *flag = 0;
    if (v >= 1.0) {
        for (int i = 0; i < 9; ++i) if (v < GT[i + 1]) return i;
    } else {
        for (int i = 1; i < 11; ++i)
            if (v >= LT[i]) { if (flag) *flag = v == LT[i]; return -i; }
    }
    double l = log10(v);
    if (flag) *flag = l == floor(l);
    return sat_i32(floor(l));
}
/* round_up (:48-55) */
static double elf_round_up(double v, uint32_t alpha) {
    double scale = elf_10i_p(alpha);
    return v < 0.0 ? floor(v * scale) / scale : ceil(v * scale) / scale;
}
/* get_significant_count (:57-95) */
static int32_t elf_significant(double v, int32_t sp, int32_t last) {
    int32_t i;
    if (last != INT32_MAX && last != 0) { i = last - sp - 1; if (i < 1) i = 1; }
    else if (last == INT32_MAX) i = 17 - sp - 1;
    else if (sp >= 0) i = 1;
    else i = -sp;
    double temp = v * elf_10i_p((uint32_t)i);
    int64_t ti = sat_i64(temp);
    while ((double)ti != temp) {
        i += 1;
        temp = v * elf_10i_p((uint32_t)i);
        if (isinf(temp)) return 17;
        ti = sat_i64(temp);
    }
    if (temp / elf_10i_p((uint32_t)i) != v) return 17;
    while (i > 0 && ti % 10 == 0) { i -= 1; ti /= 10; }
    return sp + i + 1;
}

/* ------------------------------------------------------------------------ */
/* Elf / ElfOnChimp encoders (compressor/elf.rs)                             */
/* ------------------------------------------------------------------------ */
/* Chimp encoder as a stream of values (compressor/chimp.rs:51-146) */
typedef struct { uint32_t stored_lead; uint64_t stored; int first; } chimp_enc;
static void chimp_enc_add(bitw* w, chimp_enc* e, uint64_t val) {
    if (e->first) { e->first = 0; e->stored = val; bw_bits(w, val, 64); return; }
    uint64_t x = e->stored ^ val;
    if (x == 0) {
        bw_bit(w, 0); bw_bit(w, 0);
        e->stored_lead = 65;
    } else {
        uint32_t lead = LEAD_ROUND[clz64(x)];
        uint32_t trail = (uint32_t)ctz64(x);
        if (trail > 6) {
            uint32_t sig = 64 - lead - trail;
            bw_bit(w, 0); bw_bit(w, 1);
            bw_bits(w, LEAD_REPR[lead], 3);
            bw_bits(w, sig, 6);
            bw_bits(w, x >> trail, sig);
            e->stored_lead = 65;
        } else if (lead == e->stored_lead) {
            bw_bit(w, 1); bw_bit(w, 0);
            bw_bits(w, x, 64 - lead);
        } else {
            e->stored_lead = lead;
            bw_bit(w, 1); bw_bit(w, 1);
            bw_bits(w, LEAD_REPR[lead], 3);
            bw_bits(w, x, 64 - lead);
        }
    }
    e->stored = val;
}
/* ElfXorEncoder (compressor/elf.rs:164-262) */
typedef struct { uint32_t lead, trail; uint64_t stored; int first; } elfx_enc;
static void elfx_add(bitw* w, elfx_enc* e, uint64_t bits) {
    if (e->first) {                                            /* write_first :192-206 */
        e->first = 0;
        e->stored = bits;
        uint32_t tz = bits ? (uint32_t)ctz64(bits) : 64;
        bw_bits(w, tz, 7);
        if (tz < 63) bw_bits(w, bits >> (tz + 1), 63 - tz);    /* tz 63 writes no bits */
        return;
    }
    uint64_t x = e->stored ^ bits;                             /* compress_float_inner :212-262 */
    if (x == 0) { bw_bits(w, 1, 2); return; }                  /* case 01 */
    uint32_t lead = LEAD_ROUND[clz64(x)];
    uint32_t trail = (uint32_t)ctz64(x);
    if (lead == e->lead && trail >= e->trail) {                /* case 00 */
        uint32_t center = 64 - e->lead - e->trail;
        bw_bits(w, 0, 2);
        bw_bits(w, x >> e->trail, center);
    } else {
        e->lead = lead;
        e->trail = trail;
        uint32_t center = 64 - lead - trail;
        uint32_t repr = LEAD_REPR[lead];
        if (center <= 16) {                                     /* case 10 */
            bw_bits(w, (((0x2u << 3) | repr) << 4) | (center & 0xf), 9);
            if (center > 1) bw_bits(w, x >> (trail + 1), center - 1);
        } else {                                                /* case 11 */
            bw_bits(w, (((0x3u << 3) | repr) << 6) | (center & 0x3f), 11);
            bw_bits(w, x >> (trail + 1), center - 1);
        }
    }
    e->stored = bits;
}
/* ElfEncoderWrapper::add_value (:92-158) over ElfXorEncoder or ChimpEncoder */
static void elf_encode(bitw* w, const double* v, uint64_t n, int on_chimp) {
    elfx_enc ex = {0xffffffffu, 0xffffffffu, 0, 1};
    chimp_enc ec = {0xffffffffu, 0, 1};
    int32_t last = INT32_MAX;
    for (uint64_t i = 0; i <= n; ++i) {
        uint64_t vp;
        if (i == n) {                                          /* close :61-66: case 10, then the XOR close */
            bw_bits(w, 2, 2);
            vp = NAN_BITS;
        } else {
            double x = v[i];
            uint64_t vb = f2u(x);
            if (x == 0.0 || isinf(x)) { bw_bits(w, 2, 2); vp = vb; }
            else if (x != x) { bw_bits(w, 2, 2); vp = NAN_BITS; }
            else {
                int flag;
                double ax = fabs(x);
                int32_t sp = elf_sp(ax, &flag);                /* get_alpha_and_beta_star :41-47 */
                int32_t beta = elf_significant(ax, sp, last);
                uint32_t alpha = (uint32_t)((int64_t)beta - sp - 1);
                int32_t beta_star = flag == 1 ? 0 : beta;
                uint64_t mask = ~0ull;
                uint64_t delta = 0;
                int32_t erase = 0;
                if (beta_star < 16) {
                    uint64_t e = (vb >> 52) & 0x7ff;
                    uint32_t g = elf_f_alpha(alpha) + (uint32_t)e - 1023u;
                    erase = 52 - (int32_t)g;
                    if (erase > 4) { mask = ~0ull << (erase & 63); delta = ~mask & vb; }
                    else { mask = ~0ull; delta = 0; }
                }
                if (beta_star < 16 && erase > 4 && delta != 0) {
                    if (beta_star == last) bw_bit(w, 0);           /* case 0 */
                    else {                                         /* case 11 */
                        bw_bits(w, (uint32_t)(beta_star | 0x30), 6);
                        last = beta_star;
                    }
                    vp = mask & vb;
                } else { bw_bits(w, 2, 2); vp = vb; }              /* case 10 */
            }
        }
        if (on_chimp) chimp_enc_add(w, &ec, vp);
        else elfx_add(w, &ex, vp);
    }
    bw_bit(w, 0);                                              /* the XOR encoder's closing bit */
}

/* ------------------------------------------------------------------------ */
/* BUFF fixed-point helpers (compression_common/buff.rs:1-52)                */
/* ------------------------------------------------------------------------ */
static const uint64_t PRECISION_MAP[13] = {0, 5, 8, 11, 15, 18, 21, 25, 28, 31, 35, 38, 50};

static inline uint64_t shr_wrap(uint64_t x, int64_t s) { return x >> ((uint64_t)s & 63); }

int64_t ora_buff_fixed(double value, int32_t frac) {
    /* into_fixed_representation_with_fractional_part_bits_length :40-51 */
    uint64_t vb = f2u(value);
    int32_t exp = (int32_t)((vb & 0x7ff0000000000000ull) >> 52) - 1023;
    if (exp < -frac) return 0;
    /* into_fixed_representation :11-31 */
    uint64_t sign = vb & 0x8000000000000000ull;
    int64_t s = 63 - (int64_t)exp - frac;
    uint64_t fixed = s >= 64 ? 0 : shr_wrap((vb << 11) | 0x8000000000000000ull, s);
    if (sign) fixed = ~(fixed - 1);
    return (int64_t)fixed;
}

int32_t ora_buff_precision(uint64_t scale) {
    /* Precalculated::precalculate :131-135 -- (scale as f32).log10() as usize */
    if (scale == 0) return 0;
    float l = log10f((float)scale);
    return l <= 0.0f ? 0 : (int32_t)l;
}

/* LSB-first packed field: BitPack::read_bits (compression_common/buff.rs:206-245) */
static inline uint32_t lsb_get(const uint8_t* base, uint64_t bitpos, unsigned nbits) {
    uint64_t byte = bitpos >> 3;
    unsigned sh = (unsigned)(bitpos & 7);
    uint32_t w = base[byte];
    if (sh + nbits > 8) w |= (uint32_t)base[byte + 1] << 8;
    return (w >> sh) & ((1u << nbits) - 1);
}

/* buff_simd256_encode (compressor/buff.rs:127-165, 234-307) */
static int buff_encode(obuf* o, const double* v, uint64_t n, uint64_t scale) {
    int32_t prec = ora_buff_precision(scale);
    if (prec < 0 || prec > 12) return ORA_E_INVALID;     /* PRECISION_MAP.get().unwrap() */
    uint32_t frac = (uint32_t)PRECISION_MAP[prec];
    int64_t* fx = (int64_t*)malloc((n ? n : 1) * sizeof(int64_t));
    if (!fx) return ORA_E_OOM;
    int64_t mn = INT64_MAX, mx = INT64_MIN;
    uint64_t mni = 0, mxi = 0;
    for (uint64_t i = 0; i < n; ++i) {
        fx[i] = ora_buff_fixed(v[i], (int32_t)frac);
        if (fx[i] < mn) { mn = fx[i]; mni = i; }
        if (fx[i] > mx) { mx = fx[i]; mxi = i; }
    }
    int64_t base = fx[mni];
    uint64_t delta = (uint64_t)fx[mxi] - (uint64_t)fx[mni];
    uint32_t bits = delta == 0 ? 0 : (uint32_t)(64 - clz64(delta));
    ob_u32(o, (uint32_t)(uint64_t)base);
    ob_u32(o, (uint32_t)((uint64_t)base >> 32));
    ob_u32(o, (uint32_t)n);
    ob_u32(o, bits);
    ob_u32(o, frac);
    uint32_t rem = bits;
    int tail_only = rem > 0 && rem < 8;
    if (!tail_only) {
        while (rem >= 8) {
            rem -= 8;
            ob_reserve(o, n);
            if (o->oom) break;
            for (uint64_t i = 0; i < n; ++i)
                o->p[o->len + i] = (uint8_t)((uint8_t)(((uint64_t)fx[i] - (uint64_t)base) >> rem) ^ 0x80);
            o->len += n;
        }
    }
    if (rem > 0) {                     /* finish_write_byte + LSB-first write_bits */
        size_t nb = (size_t)((n * rem + 7) / 8);
        if (nb == 0) nb = 1;
        size_t at = o->len;
        ob_zero(o, nb);
        if (!o->oom) {
            for (uint64_t i = 0; i < n; ++i) {
                uint32_t d = (uint32_t)(((uint64_t)fx[i] - (uint64_t)base)) & ((1u << rem) - 1);
                uint64_t bp = i * rem;
                for (uint32_t b = 0; b < rem; ++b, ++bp)
                    if ((d >> b) & 1) o->p[at + (bp >> 3)] |= (uint8_t)(1u << (bp & 7));
            }
        }
    }
    free(fx);
    return o->oom ? ORA_E_OOM : ORA_OK;
}

/* RunLengthCompressor (compressor/run_length.rs:49-117): u64 field count, then (u8, f64le) */
static void rle_encode(obuf* o, const double* v, uint64_t n) {
    size_t hdr = o->len;
    ob_u64(o, 0);
    uint64_t fields = 0;
    if (n) {
        uint64_t pv = f2u(v[0]);
        uint32_t run = 1;
        for (uint64_t i = 1; i < n; ++i) {
            uint64_t b = f2u(v[i]);
            if (b == pv && run < 255) { run++; continue; }     /* bytewise equality, cap 255 */
            ob_u8(o, (uint8_t)run); ob_u64(o, pv); fields++;
            pv = b; run = 1;
        }
        ob_u8(o, (uint8_t)run); ob_u64(o, pv); fields++;       /* prepare() flushes the last run */
    }
    if (!o->oom) for (int i = 0; i < 8; ++i) o->p[hdr + i] = (uint8_t)(fields >> (8 * i));
}

static int encode_chunk(obuf* o, const double* v, uint64_t n, int scheme, uint64_t scale) {
    bitw w;
    switch (scheme) {
    case ORA_UNCOMPRESSED:
        for (uint64_t i = 0; i < n; ++i) ob_u64(o, f2u(v[i]));
        return o->oom ? ORA_E_OOM : ORA_OK;
    case ORA_RLE:
        rle_encode(o, v, n);
        return o->oom ? ORA_E_OOM : ORA_OK;
    case ORA_BUFF:
        return buff_encode(o, v, n, scale);
    case ORA_GORILLA:
    case ORA_CHIMP:
    case ORA_CHIMP128:
    case ORA_ELF_ON_CHIMP:
    case ORA_ELF: {
        int st = ORA_OK;
        bw_init(&w);
        if (scheme == ORA_GORILLA) gorilla_encode(&w, v, n);
        else if (scheme == ORA_CHIMP) chimp_encode(&w, v, n);
        else if (scheme == ORA_CHIMP128) st = chimp128_encode(&w, v, n);
        else elf_encode(&w, v, n, scheme == ORA_ELF_ON_CHIMP);
        if (st == ORA_OK && !w.b.oom) ob_push(o, w.b.p, w.b.len);
        free(w.b.p);
        if (st != ORA_OK) return st;
        return (w.b.oom || o->oom) ? ORA_E_OOM : ORA_OK;
    }
    default:
        return ORA_E_INVALID;
    }
}

int ora_encode_chunk(const double* v, uint64_t n, int scheme, uint64_t scale, uint8_t** out,
                     uint64_t* out_len) {
    obuf o = {0};
    int st = encode_chunk(&o, v, n, scheme, scale);
    if (st != ORA_OK) { free(o.p); return st; }
    *out = o.p; *out_len = o.len;
    return ORA_OK;
}

/* ------------------------------------------------------------------------ */
/* EBI1 file writer: FileWriter + ChunkWriter (encoder.rs:190-529)           */
/* Header (format.rs:143-172, 30 bytes): "EBI1", field_type u8, scheme u8,   */
/* chunk kind u8, reserved u8, chunk value u64, footer_offset u64,           */
/* version [u16;3] = 0.1.14 (ebi/Cargo.toml).  The two timing fields of      */
/* FileFooter3 are written as zero (the reference writes wall-clock times).  */
/* ------------------------------------------------------------------------ */
int ora_encode(const double* v, uint64_t n, int scheme, int chunk_kind, uint64_t chunk_value,
               uint64_t scale, uint8_t** out, uint64_t* out_len) {
    if (scheme < 0 || scheme > ORA_ELF || chunk_kind < 0 || chunk_kind > 2) return ORA_E_INVALID;
    obuf o = {0};
    ob_push(&o, "EBI1", 4);
    ob_u8(&o, 0);
    ob_u8(&o, (uint8_t)scheme);
    ob_u8(&o, (uint8_t)chunk_kind);
    ob_u8(&o, 0);
    ob_u64(&o, chunk_kind == ORA_CHUNK_FULL ? 0 : chunk_value);
    ob_u64(&o, 0);                         /* footer offset, patched below */
    ob_u16(&o, 0); ob_u16(&o, 1); ob_u16(&o, 14);
    uint64_t per;                           /* records per chunk (encoder.rs:441-482) */
    if (chunk_kind == ORA_CHUNK_FULL) per = n;
    else if (chunk_kind == ORA_CHUNK_RECORD_COUNT) per = chunk_value;
    else per = (uint64_t)ceil(((double)chunk_value / 8.0) * 1.5);
    uint64_t nchunks = 0, cap = 16;
    uint64_t* foot = (uint64_t*)malloc(cap * 2 * sizeof(uint64_t));
    if (!foot) { free(o.p); return ORA_E_OOM; }
    uint64_t pos = 0;
    int st = ORA_OK;
    while (per > 0 && pos < n) {
        uint64_t take = n - pos < per ? n - pos : per;
        if (nchunks == cap) {
            cap *= 2;
            uint64_t* nf = (uint64_t*)realloc(foot, cap * 2 * sizeof(uint64_t));
            if (!nf) { st = ORA_E_OOM; break; }
            foot = nf;
        }
        foot[2 * nchunks] = o.len;
        foot[2 * nchunks + 1] = pos;
        st = encode_chunk(&o, v + pos, take, scheme, scale);
        if (st != ORA_OK) break;
        nchunks++;
        pos += take;
    }
    if (st != ORA_OK) { free(foot); free(o.p); return st; }
    uint64_t footer_off = o.len;
    ob_u64(&o, pos);                       /* FileFooter0 {number_of_records, number_of_chunks} */
    ob_u64(&o, nchunks);
    for (uint64_t i = 0; i < nchunks; ++i) { ob_u64(&o, foot[2 * i]); ob_u64(&o, foot[2 * i + 1]); }
    ob_u8(&o, 8);                          /* config: size byte + u64 (capacity or scale) */
    ob_u64(&o, scheme == ORA_BUFF ? scale : 8192);
    ob_zero(&o, 16 + 9 * 16 + 4);          /* FileFooter3 */
    free(foot);
    if (o.oom) { free(o.p); return ORA_E_OOM; }
    for (int i = 0; i < 8; ++i) o.p[16 + i] = (uint8_t)(footer_off >> (8 * i));  /* offset_of!(FileHeader, footer_offset) */
    *out = o.p; *out_len = o.len;
    return ORA_OK;
}

void ora_free(void* p) { free(p); }

/* ------------------------------------------------------------------------ */
/* EBI1 reader: FileReader::fetch_header / fetch_footer (decoder.rs:131-220) */
/* ------------------------------------------------------------------------ */
struct ora_file {
    const uint8_t* data;
    uint64_t len;
    int scheme;
    uint64_t footer_off;
    uint64_t n_records;
    uint64_t n_chunks;
    uint64_t* phys;   /* n_chunks */
    uint64_t* logi;   /* n_chunks */
    uint64_t config;  /* scale for BUFF, capacity otherwise */
    int32_t precision;
};

int ora_open(const uint8_t* d, uint64_t len, ora_file** out) {
    *out = NULL;
    if (len < 30) return ORA_E_IO;
    if (d[4] != 0) return ORA_E_CONVERSION;          /* FieldType (deserialize.rs:179-188) */
    if (d[5] > 12) return ORA_E_CONVERSION;          /* CompressionScheme */
    if (d[6] > 2) return ORA_E_CONVERSION;           /* ChunkOptionKind */
    int scheme = d[5];
    uint64_t fo = rd_u64le(d + 16);                  /* FileHeader::footer_offset (format.rs:143-151) */
    if (fo > len || len - fo < 16) return ORA_E_IO;
    uint64_t nrec = rd_u64le(d + fo), nch = rd_u64le(d + fo + 8);
    uint64_t p = fo + 16;
    if (nch > (len - p) / 16) return ORA_E_IO;
    uint64_t cf = p + nch * 16;
    if (cf + 1 > len) return ORA_E_IO;
    uint64_t csz = d[cf];
    if (cf + 1 + csz > len) return ORA_E_IO;
    if (csz < 8) return ORA_E_CORRUPT;                /* from_le_bytes slices [..8] */
    if (cf + 1 + csz + 164 > len) return ORA_E_IO;    /* FileFooter3 */
    if (scheme > ORA_ELF) return ORA_E_INVALID;  /* codecs outside this path */
    ora_file* f = (ora_file*)calloc(1, sizeof *f);
    if (!f) return ORA_E_OOM;
    f->phys = (uint64_t*)malloc((nch ? nch : 1) * 8);
    f->logi = (uint64_t*)malloc((nch ? nch : 1) * 8);
    if (!f->phys || !f->logi) { ora_close(f); return ORA_E_OOM; }
    for (uint64_t i = 0; i < nch; ++i) {
        f->phys[i] = rd_u64le(d + p + 16 * i);
        f->logi[i] = rd_u64le(d + p + 16 * i + 8);
    }
    f->data = d; f->len = len; f->scheme = scheme; f->footer_off = fo;
    f->n_records = nrec; f->n_chunks = nch; f->config = rd_u64le(d + cf + 1);
    f->precision = -1;
    *out = f;
    return ORA_OK;
}

void ora_close(ora_file* f) {
    if (!f) return;
    free(f->phys); free(f->logi); free(f);
}
uint64_t ora_num_records(const ora_file* f) { return f->n_records; }
uint64_t ora_num_chunks(const ora_file* f) { return f->n_chunks; }
int ora_scheme(const ora_file* f) { return f->scheme; }
void ora_set_precision(ora_file* f, int32_t p) { f->precision = p; }

/* GeneralChunkHandle::{chunk_size, number_of_records} (decoder.rs:283-328) */
static void chunk_geom(const ora_file* f, uint64_t i, uint64_t* phys, uint64_t* size,
                       uint64_t* row, uint64_t* rows) {
    uint64_t np = i + 1 < f->n_chunks ? f->phys[i + 1] : f->footer_off;
    uint64_t nl = i + 1 < f->n_chunks ? f->logi[i + 1] : f->n_records;
    *phys = f->phys[i]; *size = np - f->phys[i];
    *row = f->logi[i]; *rows = nl - f->logi[i];
}
int ora_chunk_info(const ora_file* f, uint64_t i, uint64_t* phys, uint64_t* size, uint64_t* row,
                   uint64_t* rows) {
    if (i >= f->n_chunks) return ORA_E_INVALID;
    chunk_geom(f, i, phys, size, row, rows);
    return ORA_OK;
}

/* ------------------------------------------------------------------------ */
/* Chunk decoders (decompress): each appends the decoded values              */
/* ------------------------------------------------------------------------ */
typedef struct { double* v; uint64_t n, cap; } dvec;
static int dv_push(dvec* d, double x) {
    if (d->n == d->cap) {
        uint64_t nc = d->cap ? d->cap * 2 : 1024;
        double* np = (double*)realloc(d->v, nc * sizeof(double));
        if (!np) return 0;
        d->v = np; d->cap = nc;
    }
    d->v[d->n++] = x;
    return 1;
}
#define PUSH(x) do { if (!dv_push(out, (x))) return ORA_E_OOM; } while (0)
#define RB(n, dst) do { if (!br_bits(&r, (n), (dst))) return ORA_E_UNEXPECTED_END; } while (0)

/* GorillaDecoder::next (decoder/chunk_reader/gorilla.rs:90-157) */
static int gorilla_decode(const uint8_t* c, uint64_t len, dvec* out) {
    bitr r = {c, len, 0};
    uint64_t value = 0, t;
    uint32_t lead = 0, trail = 0;
    RB(64, &value);
    for (;;) {
        if (value == NAN_BITS) return ORA_OK;
        PUSH(u2f(value));
        RB(1, &t);
        if (!t) continue;                                   /* '0': repeat */
        RB(1, &t);
        if (t) {                                            /* '11': new window */
            uint64_t l, s;
            RB(5, &l); RB(6, &s);
            if (l + s + 1 > 64) return ORA_E_CORRUPT;       /* u8 underflow */
            lead = (uint32_t)l; trail = 64 - lead - (uint32_t)(s + 1);
        }
        uint64_t bits;
        RB(64 - lead - trail, &bits);
        value ^= bits << trail;
    }
}

/* ChimpDecoder::read_value / next_value (decoder/chunk_reader/chimp.rs:58-124) */
static int chimp_decode(const uint8_t* c, uint64_t len, dvec* out) {
    bitr r = {c, len, 0};
    uint32_t stored_lead = 0xffffffffu, stored_trail = 0;
    uint64_t val, t;
    RB(64, &val);
    for (;;) {
        if (val == NAN_BITS) return ORA_OK;
        PUSH(u2f(val));
        uint64_t flag;
        RB(2, &flag);
        if (flag == 3) {
            RB(3, &t);
            stored_lead = LEAD_DECODE[t];
            RB(64 - stored_lead, &t);
            val ^= t;
        } else if (flag == 2) {
            if (stored_lead > 64) return ORA_E_CORRUPT;
            RB(64 - stored_lead, &t);
            val ^= t;
        } else if (flag == 1) {
            RB(3, &t);
            stored_lead = LEAD_DECODE[t];
            uint64_t sig;
            RB(6, &sig);
            if (sig == 0) sig = 64;
            if (sig + stored_lead > 64) return ORA_E_CORRUPT;
            stored_trail = 64 - (uint32_t)sig - stored_lead;
            RB(64 - stored_lead - stored_trail, &t);
            val ^= t << stored_trail;
        }
    }
}

/* ChimpNDecoder<128>::next / next_value (decoder/chunk_reader/chimp_n.rs:160-285) */
static int chimp128_decode(const uint8_t* c, uint64_t len, dvec* out) {
    bitr r = {c, len, 0};
    uint64_t ring[CN];
    memset(ring, 0, sizeof ring);
    uint32_t stored_lead = 0xffffffffu, stored_trail = 0;
    uint64_t val, t;
    unsigned cur = 0;
    RB(64, &val);
    ring[cur] = val;
    if (val == NAN_BITS) return ORA_OK;
    for (;;) {
        PUSH(u2f(val));
        uint64_t flag;
        RB(2, &flag);
        if (flag == 3 || flag == 2) {
            if (flag == 3) { RB(3, &t); stored_lead = LEAD_DECODE[t]; }
            if (stored_lead > 64) return ORA_E_CORRUPT;
            RB(64 - stored_lead, &t);
            val ^= t;
            if (val == NAN_BITS) return ORA_OK;
            cur = (cur + 1) % CN; ring[cur] = val;
        } else if (flag == 1) {
            uint64_t temp;
            RB(CN_LOG2 + 9, &temp);
            uint64_t idx = (temp >> 9) & (CN - 1);
            stored_lead = LEAD_DECODE[(temp >> 6) & 7];
            uint64_t sig = temp & 63;
            val = ring[idx];
            if (sig == 0) sig = 64;
            if (sig + stored_lead > 64) return ORA_E_CORRUPT;
            stored_trail = 64 - (uint32_t)sig - stored_lead;
            RB(64 - stored_lead - stored_trail, &t);
            val ^= t << stored_trail;
            if (val == NAN_BITS) return ORA_OK;
            cur = (cur + 1) % CN; ring[cur] = val;
        } else {
            RB(CN_LOG2, &t);
            val = ring[t];                                  /* no NaN check on '00' */
            cur = (cur + 1) % CN; ring[cur] = val;
        }
    }
}

/* Elf / ElfOnChimp readers (decoder/chunk_reader/elf.rs): the wrapper's
 * prefix (0: restore with the current beta*, 10: value as is, 11: new 4-bit
 * beta* then restore) before every value of the inner XOR stream; the inner
 * stream ends at the NaN end marker. */
typedef struct { uint64_t val; uint32_t lead; int first; } chimp_dec;      /* ChimpDecoder as a stream */
static int chimp_dec_next(bitr* r, chimp_dec* d, uint64_t* out, int* end) {
    uint64_t t;
    *end = 0;
    if (d->first) {
        d->first = 0;
        if (!br_bits(r, 64, &d->val)) return ORA_E_UNEXPECTED_END;
    } else {
        uint64_t flag;
        if (!br_bits(r, 2, &flag)) return ORA_E_UNEXPECTED_END;
        if (flag == 3) {
            if (!br_bits(r, 3, &t)) return ORA_E_UNEXPECTED_END;
            d->lead = LEAD_DECODE[t];
            if (!br_bits(r, 64 - d->lead, &t)) return ORA_E_UNEXPECTED_END;
            d->val ^= t;
        } else if (flag == 2) {
            if (d->lead > 64) return ORA_E_CORRUPT;
            if (!br_bits(r, 64 - d->lead, &t)) return ORA_E_UNEXPECTED_END;
            d->val ^= t;
        } else if (flag == 1) {
            uint64_t sig;
            if (!br_bits(r, 3, &t)) return ORA_E_UNEXPECTED_END;
            d->lead = LEAD_DECODE[t];
            if (!br_bits(r, 6, &sig)) return ORA_E_UNEXPECTED_END;
            if (sig == 0) sig = 64;
            if (sig + d->lead > 64) return ORA_E_CORRUPT;
            uint32_t trail = 64 - (uint32_t)sig - d->lead;
            if (!br_bits(r, (unsigned)sig, &t)) return ORA_E_UNEXPECTED_END;
            d->val ^= t << trail;
        }
    }
    if (d->val == NAN_BITS) { *end = 1; return ORA_OK; }
    *out = d->val;
    return ORA_OK;
}
typedef struct { uint64_t val; uint32_t lead, trail; int first; } elfx_dec;  /* ElfXorDecoder (:104-258) */
static int elfx_dec_next(bitr* r, elfx_dec* d, uint64_t* out, int* end) {
    uint64_t t;
    *end = 0;
    if (d->first) {                                             /* read_first :121-141 */
        d->first = 0;
        if (!br_bits(r, 7, &t)) return ORA_E_UNEXPECTED_END;
        uint32_t tz = (uint32_t)t;
        if (tz < 64) {
            uint64_t b;
            if (!br_bits(r, 63 - tz, &b)) return ORA_E_UNEXPECTED_END;
            d->val = ((b << 1) | 1) << tz;
        } else d->val = 0;
        if (d->val == NAN_BITS) { *end = 1; return ORA_OK; }
        *out = d->val;
        return ORA_OK;
    }
    uint64_t flag;
    if (!br_bits(r, 2, &flag)) return ORA_E_UNEXPECTED_END;    /* decompress_float_inner :143-221 */
    if (flag == 1) { *out = d->val; return ORA_OK; }           /* case 01: the same value */
    uint64_t value;
    if (flag == 3 || flag == 2) {
        uint64_t lac;
        unsigned hb = flag == 3 ? 9 : 7, cb = flag == 3 ? 6 : 4;
        if (!br_bits(r, hb, &lac)) return ORA_E_UNEXPECTED_END;
        d->lead = LEAD_DECODE[lac >> cb];
        uint32_t center = (uint32_t)(lac & ((1u << cb) - 1));
        if (center == 0) center = 1u << cb;
        if (d->lead + center > 64) return ORA_E_CORRUPT;
        d->trail = 64 - d->lead - center;
        if (flag == 2 && center == 1) value = 1ull << d->trail;
        else {
            uint64_t b;
            if (!br_bits(r, center - 1, &b)) return ORA_E_UNEXPECTED_END;
            value = ((b << 1) | 1) << d->trail;
        }
    } else {                                                    /* case 00 */
        if (d->lead > 64 || d->trail > 64 || d->lead + d->trail > 64) return ORA_E_CORRUPT;
        uint32_t center = 64 - d->lead - d->trail;
        uint64_t b;
        if (!br_bits(r, center, &b)) return ORA_E_UNEXPECTED_END;
        value = center ? b << d->trail : 0;
    }
    value ^= d->val;
    if (value == NAN_BITS) { *end = 1; return ORA_OK; }
    d->val = value;
    *out = value;
    return ORA_OK;
}
/* recover_v_by_beta_star (:68-84) */
static double elf_recover(double vp, int32_t beta) {
    int32_t sp = elf_sp(fabs(vp), NULL);
    if (beta == 0) {
        double v = elf_10i_n((uint32_t)(-(int64_t)sp - 1));
        return vp < 0.0 ? -v : v;
    }
    return elf_round_up(vp, (uint32_t)((int64_t)beta - sp - 1));
}
static int elf_decode(const uint8_t* c, uint64_t len, int on_chimp, dvec* out) {
    bitr r = {c, len, 0};
    elfx_dec dx = {0, 0xffffffffu, 0xffffffffu, 1};
    chimp_dec dc = {0, 0xffffffffu, 1};
    int32_t beta = INT32_MAX;
    for (;;) {
        uint64_t b, vp = 0;
        int restore, end = 0, st;
        if (!br_bits(&r, 1, &b)) return ORA_E_UNEXPECTED_END;     /* next_value :42-64 */
        if (!b) restore = 1;
        else {
            if (!br_bits(&r, 1, &b)) return ORA_E_UNEXPECTED_END;
            if (!b) restore = 0;
            else {
                if (!br_bits(&r, 4, &b)) return ORA_E_UNEXPECTED_END;
                beta = (int32_t)(uint32_t)b;
                restore = 1;
            }
        }
        st = on_chimp ? chimp_dec_next(&r, &dc, &vp, &end) : elfx_dec_next(&r, &dx, &vp, &end);
        if (st) return st;
        if (end) return ORA_OK;
        PUSH(restore ? elf_recover(u2f(vp), beta) : u2f(vp));
    }
}

/* RunLengthReaderImpl::decompress (decoder/chunk_reader/run_length.rs:68-91) */
static int rle_decode(const uint8_t* c, uint64_t len, dvec* out) {
    if (len < 8) return ORA_E_IO;
    uint64_t nf = rd_u64le(c);
    uint64_t p = 8;
    for (uint64_t i = 0; i < nf; ++i) {
        if (len - p < 9) return ORA_E_IO;
        unsigned run = c[p];
        double v = u2f(rd_u64le(c + p + 1));
        p += 9;
        for (unsigned k = 0; k < run; ++k) PUSH(v);
    }
    return ORA_OK;
}

/* UncompressedReaderImpl::decompress (decoder/chunk_reader/uncompressed.rs:56-71) */
static int raw_decode(const uint8_t* c, uint64_t len, uint64_t n_rows, dvec* out) {
    if (n_rows > len / 8) return ORA_E_IO;
    for (uint64_t i = 0; i < n_rows; ++i) PUSH(u2f(rd_u64le(c + 8 * i)));
    return ORA_OK;
}

/* BUFF header: base (i64 as two u32), n, bits, frac (decode.rs:5-17) */
typedef struct { int64_t base; uint32_t n, bits, frac; double scale; } buffh;
static int buff_header(const uint8_t* c, uint64_t len, buffh* h) {
    if (len < 20) return ORA_E_UNEXPECTED_END;
    h->base = (int64_t)((uint64_t)rd_u32le(c) | ((uint64_t)rd_u32le(c + 4) << 32));
    h->n = rd_u32le(c + 8); h->bits = rd_u32le(c + 12); h->frac = rd_u32le(c + 16);
    if (h->bits > 64) return ORA_E_CORRUPT;
    h->scale = ldexp(1.0, (int)h->frac);                    /* 2.0f64.powi(frac) */
    return ORA_OK;
}
/* bytes needed for planes + tail */
static int buff_check_len(const buffh* h, uint64_t len) {
    uint64_t need = 20 + (uint64_t)(h->bits / 8) * h->n + ((uint64_t)h->n * (h->bits % 8) + 7) / 8;
    return need <= len ? ORA_OK : ORA_E_UNEXPECTED_END;
}
static inline double buff_value(const buffh* h, uint64_t delta) {
    return (double)(int64_t)((uint64_t)h->base + delta) / h->scale;
}

/* buff_simd256_decode (buff/decode.rs:5-70) and decode_with_precision
 * (buff/controlled_precision.rs:5-75); precision < 0 means full precision. */
static int buff_decode(const uint8_t* c, uint64_t len, int32_t precision, dvec* out) {
    buffh h;
    int st = buff_header(c, len, &h);
    if (st) return st;
    if (h.bits == 0) {
        for (uint32_t i = 0; i < h.n; ++i) PUSH((double)h.base / h.scale);
        return ORA_OK;
    }
    if ((st = buff_check_len(&h, len))) return st;
    const uint8_t* p = c + 20;
    if (h.bits < 8) {
        for (uint32_t i = 0; i < h.n; ++i) PUSH(buff_value(&h, lsb_get(p, (uint64_t)i * h.bits, h.bits)));
        return ORA_OK;
    }
    uint32_t unnecessary = 0;
    if (precision >= 0) {
        if (precision > 12) return ORA_E_INVALID;
        uint32_t cf = (uint32_t)PRECISION_MAP[precision];
        unnecessary = h.frac > cf ? h.frac - cf : 0;
    }
    uint64_t* fx = (uint64_t*)calloc(h.n ? h.n : 1, 8);
    if (!fx) return ORA_E_OOM;
    uint32_t rem = h.bits - 8;
    for (uint32_t i = 0; i < h.n; ++i) fx[i] = (uint64_t)(p[i] ^ 0x80) << rem;
    p += h.n;
    while (rem >= 8 && (precision < 0 || rem > unnecessary)) {
        rem -= 8;
        for (uint32_t i = 0; i < h.n; ++i) fx[i] |= (uint64_t)(p[i] ^ 0x80) << rem;
        p += h.n;
    }
    if (rem > 0 && (precision < 0 || rem > unnecessary))
        for (uint32_t i = 0; i < h.n; ++i) fx[i] |= lsb_get(p, (uint64_t)i * rem, rem);
    for (uint32_t i = 0; i < h.n; ++i)
        if (!dv_push(out, buff_value(&h, fx[i]))) { free(fx); return ORA_E_OOM; }
    free(fx);
    return ORA_OK;
}

int ora_decode_chunk(const uint8_t* c, uint64_t len, int scheme, uint64_t n_rows, double* o,
                     uint64_t cap, uint64_t* n_out) {
    dvec d = {0};
    dvec* out = &d;
    int st;
    switch (scheme) {
    case ORA_UNCOMPRESSED: st = raw_decode(c, len, n_rows, out); break;
    case ORA_RLE: st = rle_decode(c, len, out); break;
    case ORA_BUFF: st = buff_decode(c, len, -1, out); break;
    case ORA_GORILLA: st = gorilla_decode(c, len, out); break;
    case ORA_CHIMP: st = chimp_decode(c, len, out); break;
    case ORA_CHIMP128: st = chimp128_decode(c, len, out); break;
    case ORA_ELF_ON_CHIMP: st = elf_decode(c, len, 1, out); break;
    case ORA_ELF: st = elf_decode(c, len, 0, out); break;
    default: st = ORA_E_INVALID;
    }
    if (st == ORA_OK) {
        if (d.n > cap) st = ORA_E_INVALID;
        else { if (d.n) memcpy(o, d.v, d.n * 8); *n_out = d.n; }
    }
    free(d.v);
    return st;
}

/* ------------------------------------------------------------------------ */
/* Predicate evaluation (decoder/query.rs:396-437)                            */
/* ------------------------------------------------------------------------ */
static inline int pred_eval(const ora_pred* p, double v) {
    if (p->kind == ORA_PRED_EQ) return v == p->value;
    if (p->kind == ORA_PRED_NE) return v != p->value;
    int s = p->start_kind == ORA_BOUND_INCLUSIVE ? v >= p->start
          : p->start_kind == ORA_BOUND_EXCLUSIVE ? v > p->start : 1;
    int e = p->end_kind == ORA_BOUND_INCLUSIVE ? v <= p->end
          : p->end_kind == ORA_BOUND_EXCLUSIVE ? v < p->end : 1;
    return s && e;
}

/* ------------------------------------------------------------------------ */
/* BUFF in-situ operators over per-chunk row sets (u8 per row, rows 0..L)    */
/* ------------------------------------------------------------------------ */
/* buff_simd256_cmp_filter<IS_GREATER, INCLUSIVE> (buff/filter_cmp.rs:299-451).
 * mask: chunk-relative set or NULL (None).  Writes out[0..L). */
static int buff_cmp_filter(const uint8_t* c, uint64_t len, int greater, int inclusive, double pred,
                           const uint8_t* mask, uint64_t L, uint8_t* out) {
    buffh h;
    int st = buff_header(c, len, &h);
    if (st) return st;
    memset(out, 0, L);
    int64_t fp = ora_buff_fixed(pred, (int32_t)h.frac);
    if (fp < h.base) {                                       /* :328-330 */
        if (greater) memset(out, 1, h.n < L ? h.n : L);
        return ORA_OK;
    }
    if (h.bits == 0) {                                       /* :331-339 */
        int p = greater ? (inclusive ? h.base >= fp : h.base > fp)
                        : (inclusive ? h.base <= fp : h.base < fp);
        if (p) memset(out, 1, h.n < L ? h.n : L);
        return ORA_OK;
    }
    uint64_t dp = (uint64_t)fp - (uint64_t)h.base;
    uint32_t pbits = dp == 0 ? 0 : (uint32_t)(64 - clz64(dp));
    if (h.bits < pbits) {                                    /* :341-351 */
        if (!greater) memset(out, 1, h.n < L ? h.n : L);
        return ORA_OK;
    }
    if ((st = buff_check_len(&h, len))) return st;
    uint8_t* chk = (uint8_t*)malloc(L ? L : 1);
    uint8_t* nxt = (uint8_t*)malloc(L ? L : 1);
    if (!chk || !nxt) { free(chk); free(nxt); return ORA_E_OOM; }
    int have_chk = 0;
    if (mask) { memcpy(chk, mask, L); have_chk = 1; }
    const uint8_t* p = c + 20;
    uint32_t rem = h.bits;
    while (rem >= 8) {                                       /* :357-385 */
        rem -= 8;
        uint8_t pb = (uint8_t)(dp >> rem);
        int any = 0;
        memset(nxt, 0, L);
        for (uint64_t r = 0; r < h.n && r < L; ++r) {
            if (have_chk && !chk[r]) continue;
            uint8_t b = p[r] ^ 0x80;
            if (b > pb) { if (greater) out[r] = 1; }
            else if (b == pb) { nxt[r] = 1; any = 1; }
            else if (!greater) out[r] = 1;
        }
        if (have_chk) for (uint64_t r = h.n; r < L; ++r) if (chk[r]) { free(chk); free(nxt); return ORA_E_UNEXPECTED_END; }
        p += h.n;
        if (!any) { free(chk); free(nxt); return ORA_OK; }
        memcpy(chk, nxt, L); have_chk = 1;
    }
    if (rem > 0) {                                           /* :387-444 */
        uint8_t pb = (uint8_t)(dp & ((1u << rem) - 1));
        for (uint64_t r = 0; r < h.n && r < L; ++r) {
            if (have_chk && !chk[r]) continue;
            uint8_t b = (uint8_t)lsb_get(p, r * rem, rem);
            if (b > pb) { if (greater) out[r] = 1; }
            else if (b == pb) { if (inclusive) out[r] = 1; }
            else if (!greater) out[r] = 1;
        }
    } else if (inclusive && have_chk) {                      /* :445-449 */
        for (uint64_t r = 0; r < L; ++r) if (chk[r]) out[r] = 1;
    }
    free(chk); free(nxt);
    return ORA_OK;
}

/* buff_simd256_equal_filter (buff/filter_eq.rs:74-200) */
static int buff_eq_filter(const uint8_t* c, uint64_t len, double pred, const uint8_t* mask,
                          uint64_t L, uint8_t* out) {
    buffh h;
    int st = buff_header(c, len, &h);
    if (st) return st;
    memset(out, 0, L);
    int64_t fp = ora_buff_fixed(pred, (int32_t)h.frac);
    if (fp < h.base) return ORA_OK;                          /* :103-105 */
    if (h.bits == 0) {                                       /* :106-112 */
        if (fp == h.base) memset(out, 1, h.n < L ? h.n : L);
        return ORA_OK;
    }
    if ((st = buff_check_len(&h, len))) return st;
    uint64_t dp = (uint64_t)fp - (uint64_t)h.base;
    uint8_t* res = (uint8_t*)malloc(L ? L : 1);
    if (!res) return ORA_E_OOM;
    int have = 0;
    if (mask) { memcpy(res, mask, L); have = 1; }
    const uint8_t* p = c + 20;
    uint32_t rem = h.bits;
    while (rem >= 8) {                                       /* :120-160 */
        rem -= 8;
        uint8_t pb = (uint8_t)(dp >> rem);
        int any = 0;
        for (uint64_t r = 0; r < L; ++r) {
            int in = have ? res[r] : r < h.n;
            if (in && r >= h.n) { free(res); return ORA_E_UNEXPECTED_END; }
            res[r] = (uint8_t)(in && (uint8_t)(p[r] ^ 0x80) == pb);
            any |= res[r];
        }
        have = 1;
        p += h.n;
        if (!any) { free(res); return ORA_OK; }
    }
    if (rem > 0) {                                           /* :163-197 */
        if (have) {
            uint8_t pb = (uint8_t)(dp & ((1u << rem) - 1));
            for (uint64_t r = 0; r < h.n && r < L; ++r)
                out[r] = (uint8_t)(res[r] && lsb_get(p, r * rem, rem) == pb);
        } else {
            for (uint64_t r = 0; r < h.n && r < L; ++r)      /* quirk: compares with dp as u8 */
                out[r] = (uint8_t)(lsb_get(p, r * rem, rem) == (uint8_t)dp);
        }
    } else {
        if (have) memcpy(out, res, L);
        else memset(out, 1, h.n < L ? h.n : L);
    }
    free(res);
    return ORA_OK;
}

/* sum_with_bitmask (buff/sum.rs:60-119) */
static int buff_sum(const uint8_t* c, uint64_t len, const uint8_t* mask, uint64_t L, double* out) {
    buffh h;
    int st = buff_header(c, len, &h);
    if (st) return st;
    if (h.bits == 0) { *out = ((double)h.base / h.scale) * (double)h.n; return ORA_OK; } /* :81-84 */
    if ((st = buff_check_len(&h, len))) return st;
    if (mask) for (uint64_t r = h.n; r < L; ++r) if (mask[r]) return ORA_E_UNEXPECTED_END;
    uint32_t nbytes = h.bits / 8, tb = h.bits % 8;
    const uint8_t* p = c + 20;
    uint64_t sum = 0, count = 0;
    for (int i = (int)nbytes - 1; i >= 0; --i) {
        uint64_t s = 0;
        for (uint64_t r = 0; r < h.n; ++r) if (!mask || mask[r]) s += (uint64_t)(p[r] ^ 0x80);
        sum += s << ((uint64_t)(i * 8 + tb) & 63);
        p += h.n;
    }
    if (tb) {
        uint64_t s = 0;
        for (uint64_t r = 0; r < h.n; ++r) if (!mask || mask[r]) s += lsb_get(p, r * tb, tb);
        sum += s;
    }
    if (mask) { for (uint64_t r = 0; r < L; ++r) count += mask[r]; }
    else count = h.n;
    *out = (double)(int64_t)(sum + (uint64_t)h.base * count) / h.scale;
    return ORA_OK;
}

/* max_with_bitmask<IS_MIN> (buff/min_max.rs:161-277); mask non-empty */
static int buff_max_masked(const uint8_t* c, uint64_t len, int is_min, const uint8_t* mask,
                           uint64_t L, double* out) {
    buffh h;
    int st = buff_header(c, len, &h);
    if (st) return st;
    if (h.bits == 0) { *out = (double)h.base / h.scale; return ORA_OK; }
    if ((st = buff_check_len(&h, len))) return st;
    for (uint64_t r = h.n; r < L; ++r) if (mask[r]) return ORA_E_UNEXPECTED_END;
    uint8_t* chk = (uint8_t*)malloc(L ? L : 1);
    if (!chk) return ORA_E_OOM;
    memcpy(chk, mask, L);
    const uint8_t* p = c + 20;
    uint32_t rem = h.bits;
    while (rem > 0) {
        int best = is_min ? 255 : 0;
        uint64_t cut = 0;      /* rows before cut were dropped by a later, better row */
        if (rem < 8) {                                       /* tail, flipped (:193-226) */
            for (uint64_t r = 0; r < h.n; ++r) {
                if (!chk[r]) continue;
                int v = (int)(lsb_get(p, r * rem, rem) ^ 0x80);
                if (v == best) continue;
                if ((!is_min && v > best) || (is_min && v < best)) { cut = r; best = v; }
                else chk[r] = 0;
            }
            memset(chk, 0, cut);
            break;
        }
        for (uint64_t r = 0; r < h.n; ++r) {                 /* find_max_subcolumn (:130-159) */
            if (!chk[r]) continue;
            int v = p[r] ^ 0x80;
            if (v == best) continue;
            if ((!is_min && v > best) || (is_min && v < best)) { cut = r; best = v; }
            else chk[r] = 0;
        }
        memset(chk, 0, cut);
        p += h.n;
        rem -= 8;
    }
    uint64_t idx = 0;
    while (idx < h.n && !chk[idx]) idx++;
    free(chk);
    if (idx >= h.n) return ORA_E_CORRUPT;
    p = c + 20;
    uint64_t delta = 0;
    rem = h.bits;
    while (rem > 0) {                                        /* reconstruction (:240-271) */
        if (rem < 8) { delta = (delta << rem) | lsb_get(p, idx * rem, rem); break; }
        delta = (delta << 8) | (uint64_t)(p[idx] ^ 0x80);
        p += h.n;
        rem -= 8;
    }
    *out = buff_value(&h, delta);
    return ORA_OK;
}

/* max_without_bitmask (buff/min_max.rs:160-313) */
static int buff_max_all(const uint8_t* c, uint64_t len, double* out) {
    buffh h;
    int st = buff_header(c, len, &h);
    if (st) return st;
    if (h.bits == 0) { *out = (double)h.base / h.scale; return ORA_OK; }
    if ((st = buff_check_len(&h, len))) return st;
    uint8_t* chk = (uint8_t*)calloc(h.n ? h.n : 1, 1);
    if (!chk) return ORA_E_OOM;
    const uint8_t* p = c + 20;
    int best = 0;
    uint64_t cut = 0;
    for (uint64_t r = 0; r < h.n; ++r) {                    /* first subcolumn (:309-345) */
        int v = h.bits >= 8 ? (p[r] ^ 0x80) : (int)lsb_get(p, r * h.bits, h.bits);
        if (v == best) chk[r] = 1;
        else if (v > best) { cut = r; chk[r] = 1; best = v; }
    }
    memset(chk, 0, cut);
    uint32_t rem = h.bits >= 8 ? h.bits - 8 : 0;
    if (h.bits >= 8) p += h.n;
    while (rem > 0) {                                        /* :350-391 */
        best = 0;
        cut = 0;
        int tail = rem < 8;
        for (uint64_t r = 0; r < h.n; ++r) {
            if (!chk[r]) continue;
            int v = tail ? (int)lsb_get(p, r * rem, rem) : (p[r] ^ 0x80);
            if (v == best) continue;
            if (v > best) { cut = r; best = v; }
            else chk[r] = 0;
        }
        memset(chk, 0, cut);
        if (tail) break;
        p += h.n;
        rem -= 8;
    }
    uint64_t idx = 0;
    while (idx < h.n && !chk[idx]) idx++;
    free(chk);
    if (idx >= h.n) return ORA_E_CORRUPT;
    p = c + 20;
    uint64_t delta = 0;
    rem = h.bits;
    while (rem > 0) {
        if (rem < 8) { delta = (delta << rem) | lsb_get(p, idx * rem, rem); break; }
        delta = (delta << 8) | (uint64_t)(p[idx] ^ 0x80);
        p += h.n;
        rem -= 8;
    }
    *out = buff_value(&h, delta);
    return ORA_OK;
}

/* ------------------------------------------------------------------------ */
/* Per-chunk query work (GeneralChunkReader dispatch, chunk_reader.rs:127-216)*/
/* ------------------------------------------------------------------------ */
enum { OP_MATERIALIZE, OP_FILTER, OP_FILTER_MATERIALIZE, OP_SUM, OP_MIN, OP_MAX, OP_FILTER_AGG };

typedef struct {
    int status;
    dvec vals;            /* materialize / filter_materialize output */
    uint64_t* bits;       /* filter result, chunk-relative, nwords words */
    uint64_t nwords;
    int any;              /* filter result non-empty */
    double sum, mn, mx;
} chunk_res;

typedef struct {
    ora_file* f;
    int op;
    const ora_pred* pred;
    const uint64_t* mask;
    const uint64_t* sel;
    uint64_t nsel;
    chunk_res* res;
    uint64_t next;
    pthread_mutex_t mu;
} job_t;

static int decode_any(const ora_file* f, const uint8_t* c, uint64_t len, uint64_t rows, dvec* out) {
    switch (f->scheme) {
    case ORA_UNCOMPRESSED: return raw_decode(c, len, rows, out);
    case ORA_RLE: return rle_decode(c, len, out);
    case ORA_BUFF: return buff_decode(c, len, f->precision, out);
    case ORA_GORILLA: return gorilla_decode(c, len, out);
    case ORA_CHIMP: return chimp_decode(c, len, out);
    case ORA_CHIMP128: return chimp128_decode(c, len, out);
    case ORA_ELF_ON_CHIMP: return elf_decode(c, len, 1, out);
    case ORA_ELF: return elf_decode(c, len, 0, out);
    default: return ORA_E_INVALID;
    }
}

/* BUFFReader::filter (decoder/chunk_reader/buff.rs:128-228): chunk-relative
 * result in out[0..L); mask_c is the input bitmask restricted to the chunk. */
static int buff_filter(const uint8_t* c, uint64_t len, const ora_pred* p, const uint8_t* mask_c,
                       uint64_t nfoot, uint64_t L, uint8_t* out) {
    int st;
    if (p->kind == ORA_PRED_EQ || p->kind == ORA_PRED_NE) {
        if ((st = buff_eq_filter(c, len, p->value, mask_c, L, out))) return st;
        if (p->kind == ORA_PRED_NE)
            for (uint64_t r = 0; r < L; ++r)
                out[r] = (uint8_t)((mask_c ? mask_c[r] : r < nfoot) && !out[r]);
        return ORA_OK;
    }
    int hs = p->start_kind != ORA_BOUND_NONE, he = p->end_kind != ORA_BOUND_NONE;
    if (!hs && !he) {
        for (uint64_t r = 0; r < L; ++r) out[r] = (uint8_t)(mask_c ? mask_c[r] : r < nfoot);
        return ORA_OK;
    }
    uint8_t* right = NULL;
    if (hs && (st = buff_cmp_filter(c, len, 1, p->start_kind == ORA_BOUND_INCLUSIVE, p->start, mask_c, L, out)))
        return st;
    if (he) {
        uint8_t* dst = out;
        if (hs) { right = (uint8_t*)malloc(L ? L : 1); if (!right) return ORA_E_OOM; dst = right; }
        if ((st = buff_cmp_filter(c, len, 0, p->end_kind == ORA_BOUND_INCLUSIVE, p->end, mask_c, L, dst))) {
            free(right); return st;
        }
        if (hs) for (uint64_t r = 0; r < L; ++r) out[r] &= right[r];
    }
    free(right);
    return ORA_OK;
}

static void run_chunk(job_t* j, uint64_t slot) {
    ora_file* f = j->f;
    uint64_t ci = j->sel[slot];
    chunk_res* R = &j->res[slot];
    uint64_t phys, size, off, rows;
    chunk_geom(f, ci, &phys, &size, &off, &rows);
    R->sum = 0.0; R->mn = INFINITY; R->mx = -INFINITY;
    if (phys > f->len || size > f->len - phys || phys + size < phys) { R->status = ORA_E_IO; return; }
    const uint8_t* c = f->data + phys;
    const uint64_t* m = j->mask;
    uint64_t N = f->n_records;
    int op = j->op;
    int needs_filter = op == OP_FILTER || op == OP_FILTER_MATERIALIZE || op == OP_FILTER_AGG;

    if (f->scheme == ORA_BUFF && op != OP_MATERIALIZE) {
        /* BUFF in-situ operators work on chunk-relative row sets. */
        buffh h;
        int st = buff_header(c, size, &h);
        if (st) { R->status = st; return; }
        uint64_t L = h.n > rows ? h.n : rows;
        uint8_t* mc = NULL;
        uint8_t* fr = NULL;
        if (m) {
            mc = (uint8_t*)calloc(L ? L : 1, 1);
            if (!mc) { R->status = ORA_E_OOM; return; }
            for (uint64_t r = 0; r < rows; ++r) mc[r] = (uint8_t)mask_test(m, N, off + r);
        }
        if (needs_filter) {
            fr = (uint8_t*)calloc(L ? L : 1, 1);
            if (!fr) { free(mc); R->status = ORA_E_OOM; return; }
            st = buff_filter(c, size, j->pred, mc, rows, L, fr);
            if (st) { free(mc); free(fr); R->status = st; return; }
            R->nwords = (L + 63) / 64;
            R->bits = (uint64_t*)calloc(R->nwords ? R->nwords : 1, 8);
            if (!R->bits) { free(mc); free(fr); R->status = ORA_E_OOM; return; }
            for (uint64_t r = 0; r < L; ++r) if (fr[r]) { bit_set(R->bits, r); R->any = 1; }
        }
        if (op == OP_FILTER_MATERIALIZE) {
            /* BUFFReader::filter_materialize (buff.rs:230-241): filter, then default_materialize */
            dvec d = {0};
            st = buff_decode(c, size, f->precision, &d);
            if (!st) for (uint64_t i = 0; i < d.n; ++i) if (i < L && fr[i] && !dv_push(&R->vals, d.v[i])) { st = ORA_E_OOM; break; }
            free(d.v);
        } else if (op == OP_SUM || op == OP_MIN || op == OP_MAX || op == OP_FILTER_AGG) {
            const uint8_t* am = op == OP_FILTER_AGG ? fr : mc;   /* the bitmask the aggregate sees */
            int has_mask = op == OP_FILTER_AGG || m != NULL;
            int run = 1;
            if (op == OP_FILTER_AGG) run = R->any;               /* Decoder skips empty intersections */
            if (run) {
                if (op == OP_SUM || op == OP_FILTER_AGG)
                    st = buff_sum(c, size, has_mask ? am : NULL, L, &R->sum);
                if (!st && (op == OP_MIN || op == OP_FILTER_AGG)) {
                    /* BUFFReader::min (buff.rs:274-303) */
                    int empty = 1;
                    if (has_mask) for (uint64_t r = 0; r < L; ++r) if (am[r]) { empty = 0; break; }
                    if (!has_mask) R->mn = (double)h.base / h.scale;  /* min_without_bitmask */
                    else if (empty) R->mn = NAN;
                    else st = buff_max_masked(c, size, 1, am, L, &R->mn);
                }
                if (!st && (op == OP_MAX || op == OP_FILTER_AGG)) {
                    /* BUFFReader::max (buff.rs:243-272) */
                    int empty = 1;
                    if (has_mask) for (uint64_t r = 0; r < L; ++r) if (am[r]) { empty = 0; break; }
                    if (!has_mask) st = buff_max_all(c, size, &R->mx);
                    else if (empty) R->mx = NAN;
                    else st = buff_max_masked(c, size, 0, am, L, &R->mx);
                }
            }
        }
        free(mc); free(fr);
        R->status = st;
        return;
    }

    /* decompress, then the default operators (decoder/query.rs:14-154) */
    dvec d = {0};
    int st = decode_any(f, c, size, rows, &d);
    if (st) { free(d.v); R->status = st; return; }
    if (needs_filter) {
        R->nwords = (d.n + 63) / 64;
        R->bits = (uint64_t*)calloc(R->nwords ? R->nwords : 1, 8);
        if (!R->bits) { free(d.v); R->status = ORA_E_OOM; return; }
    }
    double s = 0.0, mn = INFINITY, mx = -INFINITY;
    for (uint64_t i = 0; i < d.n; ++i) {
        uint64_t row = off + i;
        if (m && !mask_test(m, N, row)) continue;
        double v = d.v[i];
        switch (op) {
        case OP_MATERIALIZE:
            if (!dv_push(&R->vals, v)) st = ORA_E_OOM;
            break;
        case OP_FILTER:
            if (pred_eval(j->pred, v)) { bit_set(R->bits, i); R->any = 1; }
            break;
        case OP_FILTER_MATERIALIZE:
            if (pred_eval(j->pred, v) && !dv_push(&R->vals, v)) st = ORA_E_OOM;
            break;
        case OP_SUM: s += v; break;
        case OP_MIN: mn = fmin(mn, v); break;
        case OP_MAX: mx = fmax(mx, v); break;
        case OP_FILTER_AGG:
            if (pred_eval(j->pred, v)) {
                bit_set(R->bits, i); R->any = 1;
                s += v; mn = fmin(mn, v); mx = fmax(mx, v);
            }
            break;
        }
        if (st) break;
    }
    R->sum = s; R->mn = mn; R->mx = mx;
    free(d.v);
    R->status = st;
}

static void* worker(void* arg) {
    job_t* j = (job_t*)arg;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        uint64_t s = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (s >= j->nsel) return NULL;
        run_chunk(j, s);
    }
}

/* Decoder chunk loop (api/decoder.rs:202-439): selects chunks by chunk_id and
 * by a non-empty intersection with the bitmask, runs them, and leaves the
 * per-chunk results in j->res for the caller to combine in chunk order. */
static int run_job(job_t* j, int64_t chunk_id, int threads) {
    ora_file* f = j->f;
    uint64_t* sel = (uint64_t*)malloc((f->n_chunks ? f->n_chunks : 1) * 8);
    if (!sel) return ORA_E_OOM;
    uint64_t ns = 0;
    for (uint64_t ci = 0; ci < f->n_chunks; ++ci) {
        if (chunk_id >= 0 && (uint64_t)chunk_id != ci) continue;
        if (j->mask) {
            uint64_t phys, size, off, rows;
            chunk_geom(f, ci, &phys, &size, &off, &rows);
            uint32_t lo = (uint32_t)off, hi = (uint32_t)(off + rows); /* logical_record_range_u32 */
            int any = 0;
            for (uint64_t r = lo; r < hi && r < f->n_records; ++r)
                if (mask_test(j->mask, f->n_records, r)) { any = 1; break; }
            if (!any) continue;
        }
        sel[ns++] = ci;
    }
    j->sel = sel; j->nsel = ns; j->next = 0;
    j->res = (chunk_res*)calloc(ns ? ns : 1, sizeof(chunk_res));
    if (!j->res) { free(sel); return ORA_E_OOM; }
    if (threads <= 1 || ns <= 1) {
        for (uint64_t s = 0; s < ns; ++s) {
            run_chunk(j, s);
            if (j->res[s].status) break;   /* the reference stops at the first error */
        }
    } else {
        pthread_mutex_init(&j->mu, NULL);
        int nt = threads < (int)ns ? threads : (int)ns;
        pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nt);
        int started = 0;
        for (int t = 0; th && t < nt; ++t) if (pthread_create(&th[t], NULL, worker, j) == 0) started++;
        if (started == 0) worker(j);
        for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
        free(th);
        pthread_mutex_destroy(&j->mu);
    }
    for (uint64_t s = 0; s < ns; ++s) if (j->res[s].status) return j->res[s].status;
    return ORA_OK;
}

static void free_job(job_t* j) {
    for (uint64_t s = 0; s < j->nsel; ++s) { free(j->res[s].vals.v); free(j->res[s].bits); }
    free(j->res); free((void*)j->sel);
}

static int collect_vals(job_t* j, double* out, uint64_t cap, uint64_t* n_out) {
    uint64_t n = 0;
    for (uint64_t s = 0; s < j->nsel; ++s) n += j->res[s].vals.n;
    if (n > cap) return ORA_E_INVALID;
    n = 0;
    for (uint64_t s = 0; s < j->nsel; ++s) {
        if (j->res[s].vals.n) memcpy(out + n, j->res[s].vals.v, j->res[s].vals.n * 8);
        n += j->res[s].vals.n;
    }
    *n_out = n;
    return ORA_OK;
}

static void collect_bits(job_t* j, uint64_t* out_mask) {
    ora_file* f = j->f;
    uint64_t N = f->n_records;
    memset(out_mask, 0, ((N + 63) / 64) * 8);
    for (uint64_t s = 0; s < j->nsel; ++s) {
        chunk_res* R = &j->res[s];
        uint64_t phys, size, off, rows;
        chunk_geom(f, j->sel[s], &phys, &size, &off, &rows);
        for (uint64_t w = 0; w < R->nwords; ++w) {
            uint64_t word = R->bits[w];
            while (word) {
                int b = __builtin_ctzll(word);
                word &= word - 1;
                uint64_t row = off + w * 64 + (uint64_t)b;
                if (row < N) bit_set(out_mask, row);        /* result |= filtered */
            }
        }
    }
}

int ora_materialize(ora_file* f, const uint64_t* mask, int64_t chunk_id, double* out, uint64_t cap,
                    uint64_t* n_out, int threads) {
    job_t j = {0};
    j.f = f; j.op = OP_MATERIALIZE; j.mask = mask;
    int st = run_job(&j, chunk_id, threads);
    if (!st) st = collect_vals(&j, out, cap, n_out);
    free_job(&j);
    return st;
}

int ora_filter(ora_file* f, const ora_pred* p, const uint64_t* mask, int64_t chunk_id,
               uint64_t* out_mask, int threads) {
    job_t j = {0};
    j.f = f; j.op = OP_FILTER; j.pred = p; j.mask = mask;
    int st = run_job(&j, chunk_id, threads);
    if (!st) collect_bits(&j, out_mask);
    free_job(&j);
    return st;
}

int ora_filter_materialize(ora_file* f, const ora_pred* p, const uint64_t* mask, int64_t chunk_id,
                           double* out, uint64_t cap, uint64_t* n_out, int threads) {
    job_t j = {0};
    j.f = f; j.op = OP_FILTER_MATERIALIZE; j.pred = p; j.mask = mask;
    int st = run_job(&j, chunk_id, threads);
    if (!st) st = collect_vals(&j, out, cap, n_out);
    free_job(&j);
    return st;
}

static int agg(ora_file* f, int op, const uint64_t* mask, int64_t chunk_id, double* out, int threads) {
    job_t j = {0};
    j.f = f; j.op = op; j.mask = mask;
    int st = run_job(&j, chunk_id, threads);
    if (!st) {
        double r = op == OP_SUM ? 0.0 : op == OP_MIN ? INFINITY : -INFINITY;
        for (uint64_t s = 0; s < j.nsel; ++s) {
            if (op == OP_SUM) r += j.res[s].sum;              /* result += chunk sum, chunk order */
            else if (op == OP_MIN) r = fmin(r, j.res[s].mn);
            else r = fmax(r, j.res[s].mx);
        }
        *out = r;
    }
    free_job(&j);
    return st;
}
int ora_sum(ora_file* f, const uint64_t* m, int64_t cid, double* o, int t) { return agg(f, OP_SUM, m, cid, o, t); }
int ora_min(ora_file* f, const uint64_t* m, int64_t cid, double* o, int t) { return agg(f, OP_MIN, m, cid, o, t); }
int ora_max(ora_file* f, const uint64_t* m, int64_t cid, double* o, int t) { return agg(f, OP_MAX, m, cid, o, t); }

int ora_filter_agg(ora_file* f, const ora_pred* p, const uint64_t* mask, int64_t chunk_id,
                   uint64_t* out_mask, double* sum, double* mn, double* mx, int threads) {
    job_t j = {0};
    j.f = f; j.op = OP_FILTER_AGG; j.pred = p; j.mask = mask;
    int st = run_job(&j, chunk_id, threads);
    if (!st) {
        if (out_mask) collect_bits(&j, out_mask);
        double s = 0.0, a = INFINITY, b = -INFINITY;
        for (uint64_t k = 0; k < j.nsel; ++k) {
            if (!j.res[k].any) continue;   /* the second call skips chunks the filter left empty */
            s += j.res[k].sum;
            a = fmin(a, j.res[k].mn);
            b = fmax(b, j.res[k].mx);
        }
        if (sum) *sum = s;
        if (mn) *mn = a;
        if (mx) *mx = b;
    }
    free_job(&j);
    return st;
}

/* ------------------------------------------------------------------------ */
/* multi-column aggregation (api/decoder.rs:755-917, decoder/expr.rs:11-135) */
/* ------------------------------------------------------------------------ */
typedef struct { int32_t kind; uint32_t index; double lit; int32_t lhs, rhs; } enode;

/* Postfix nodes -> tree (children by index); returns the root or -1. */
static int32_t expr_tree(const ora_expr_node* nodes, uint32_t n, enode* t) {
    int32_t* st = (int32_t*)malloc((n ? n : 1) * sizeof(int32_t));
    if (!st) return -1;
    uint32_t sp = 0;
    for (uint32_t i = 0; i < n; ++i) {
        t[i].kind = nodes[i].kind; t[i].index = nodes[i].index; t[i].lit = nodes[i].literal;
        t[i].lhs = t[i].rhs = -1;
        if (nodes[i].kind == ORA_EXPR_INDEX || nodes[i].kind == ORA_EXPR_LITERAL) { st[sp++] = (int32_t)i; continue; }
        if (nodes[i].kind < ORA_EXPR_ADD || nodes[i].kind > ORA_EXPR_DIV || sp < 2) { free(st); return -1; }
        t[i].rhs = st[--sp];
        t[i].lhs = st[--sp];
        st[sp++] = (int32_t)i;
    }
    int32_t root = sp == 1 ? st[0] : -1;
    free(st);
    return root;
}

/* Op::doit (expr.rs:19-28) */
static inline double op_doit(int32_t op, double l, double r) {
    switch (op) {
    case ORA_EXPR_ADD: return l + r;
    case ORA_EXPR_SUB: return l - r;
    case ORA_EXPR_MUL: return l * r;
    default: return l / r;
    }
}

/* The selected values of one chunk (GeneralChunkReader::materialize with the
 * bitmask; an empty intersection materializes nothing). */
static int chunk_vals(ora_file* f, const uint64_t* mask, uint64_t c, dvec* out) {
    job_t j = {0};
    j.f = f; j.op = OP_MATERIALIZE; j.mask = mask;
    int st = run_job(&j, (int64_t)c, 1);
    out->v = NULL; out->n = out->cap = 0;
    if (!st && j.nsel == 1) { *out = j.res[0].vals; j.res[0].vals.v = NULL; j.res[0].vals.n = 0; }
    free_job(&j);
    return st;
}

/* Expr::compute_chunk (expr.rs:67-135) */
static int expr_chunk(ora_file* const* files, const enode* t, int32_t k, const uint64_t* mask, uint64_t c,
                      dvec* out) {
    const enode* e = &t[k];
    if (e->kind == ORA_EXPR_LITERAL) return ORA_E_PRECONDITION;
    if (e->kind == ORA_EXPR_INDEX) return chunk_vals(files[e->index], mask, c, out);
    const enode *L = &t[e->lhs], *R = &t[e->rhs];
    const int ll = L->kind == ORA_EXPR_LITERAL, rl = R->kind == ORA_EXPR_LITERAL;
    if (ll && rl) return ORA_E_PRECONDITION;
    if (!ll && !rl) {
        dvec a, b;
        int st = expr_chunk(files, t, e->lhs, mask, c, &a);
        if (st) return st;
        st = expr_chunk(files, t, e->rhs, mask, c, &b);
        if (st) { free(a.v); return st; }
        const uint64_t n = a.n < b.n ? a.n : b.n;  /* zip stops at the shorter */
        for (uint64_t i = 0; i < n; ++i) a.v[i] = op_doit(e->kind, a.v[i], b.v[i]);
        a.n = n;
        free(b.v);
        *out = a;
        return ORA_OK;
    }
    int st = expr_chunk(files, t, ll ? e->rhs : e->lhs, mask, c, out);
    if (st) return st;
    for (uint64_t i = 0; i < out->n; ++i)
        out->v[i] = ll ? op_doit(e->kind, L->lit, out->v[i]) : op_doit(e->kind, out->v[i], R->lit);
    return ORA_OK;
}

int ora_aggregate(ora_file* const* files, uint32_t n_files, int kind, const ora_expr_node* nodes,
                  uint32_t n_nodes, const uint64_t* mask, double* scalar, double* array, uint64_t cap,
                  uint64_t* n_array) {
    if (!files || n_files == 0 || !nodes || kind < ORA_AGGR_NONE || kind > ORA_AGGR_SUM) return ORA_E_INVALID;
    enode* t = (enode*)malloc((n_nodes ? n_nodes : 1) * sizeof(enode));
    if (!t) return ORA_E_OOM;
    const int32_t root = expr_tree(nodes, n_nodes, t);
    int st = root < 0 ? ORA_E_INVALID : ORA_OK;
    for (uint32_t i = 0; !st && i < n_nodes; ++i)
        if (t[i].kind == ORA_EXPR_INDEX && t[i].index >= n_files) st = ORA_E_INVALID;  /* decoders[i] panics */
    if (st) { free(t); return st; }
    if (n_array) *n_array = 0;
    if (t[root].kind == ORA_EXPR_INDEX) {
        /* in-situ dispatch (AggregationKind::dispatch, api/decoder.rs:816-828) */
        free(t);
        ora_file* f = files[nodes[root].index];
        if (kind == ORA_AGGR_NONE) return ORA_E_INVALID;  /* todo!() */
        if (kind == ORA_AGGR_SUM) return ora_sum(f, mask, -1, scalar, 1);
        if (kind == ORA_AGGR_MIN) return ora_min(f, mask, -1, scalar, 1);
        return ora_max(f, mask, -1, scalar, 1);
    }
    /* AggregationResult::zero (api/decoder.rs:773-780) */
    double r = kind == ORA_AGGR_MAX ? -INFINITY : kind == ORA_AGGR_MIN ? INFINITY : 0.0;
    uint64_t na = 0;
    const uint64_t nc = files[0]->n_chunks;
    for (uint64_t c = 0; !st && c < nc; ++c) {
        for (uint32_t d = 0; d < n_files; ++d)
            if (c >= files[d]->n_chunks) st = ORA_E_INVALID;  /* chunk_handles[i] panics */
        if (st) break;
        dvec v;
        st = expr_chunk(files, t, root, mask, c, &v);
        if (st) break;
        /* dispatch_on_vec (api/decoder.rs:830-837), then concat (:791-808) */
        if (kind == ORA_AGGR_NONE) {
            if (array && na + v.n <= cap && v.n) memcpy(array + na, v.v, v.n * 8);
            na += v.n;
        } else if (kind == ORA_AGGR_SUM) {
            double s = -0.0;  /* <f64 as Sum>: a sequential fold */
            for (uint64_t i = 0; i < v.n; ++i) s += v.v[i];
            r += s;
        } else if (kind == ORA_AGGR_MAX) {
            double m = -INFINITY;
            for (uint64_t i = 0; i < v.n; ++i) m = fmax(m, v.v[i]);
            r = fmax(r, m);
        } else {
            double m = INFINITY;
            for (uint64_t i = 0; i < v.n; ++i) m = fmin(m, v.v[i]);
            r = fmin(r, m);
        }
        free(v.v);
    }
    free(t);
    if (st) return st;
    if (kind == ORA_AGGR_NONE) {
        if (n_array) *n_array = na;
        return na > cap ? ORA_E_INVALID : ORA_OK;
    }
    if (scalar) *scalar = r;
    return ORA_OK;
}
