// finalize.cuh -- the fold of per-chunk results into the query's result
// (Decoder's `result += chunk`, `result = result.min(chunk)`,
// `result = result.max(chunk)`, api/decoder.rs:323-439): BUFF in chunk order
// on exact integers, the other codecs as an exact fixed-point sum (the same in
// any order); shared by the single-query folds (query.cu) and the batched
// launch (batch.cu).
#pragma once

#include <climits>
#include <cstring>

#include "fold.cuh"
#include "values.cuh"

namespace ebi {
namespace {

constexpr int kFinThreads = 1024;

template <typename T, typename F>
__device__ __forceinline__ T block_reduce(T v, F op, T* sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = lane < static_cast<int>(blockDim.x >> 5) ? sh[lane] : sh[0];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) sh[0] = v;
    }
    __syncthreads();
    return sh[0];
}

// ---- the fold of the other codecs' partials ---------------------------------
// Integer pipes only (GB300's FP64 pipe is a small fraction of its integer
// rate; a double-double fold in one CTA was bound by it).  A chunk's
// compensated sum hi + lo enters as two terms of a signed 192-bit fixed-point
// sum, its min / max as ordered keys.
//
// Slices of kSliceChunks chunks are folded by one warp each (lane l: chunks 2l
// and 2l + 1 of the slice).  With T the largest exponent field among the
// slice's finite nonzero terms, a term +-m * 2^k (m < 2^53, k = max(field, 1)
// - 1075) becomes +-floor(m * 2^(k - e)) in units of 2^e, e = T - 1172: every
// term is below 2^150 and a slice's sum below 2^157.  The slices meet at the
// query's largest T, Tq: a slice's sum is shifted down (floor) by Tq - T, and
// the sum of the shifted slices is exact, so it is the same in any order and
// on every path (a grid of warps for one column, one CTA per query in a
// batch).  Error: below 2^-148 of the largest term, per term (double-double:
// about 2^-106).  The total rounds to nearest, ties to even.  Non-finite terms
// set flags instead: a NaN, or +inf and -inf together, give NaN; one infinity
// gives itself, as the reference's sequential f64 sum does.
struct Wide {
    unsigned long long w0, w1, w2;  // two's complement, w2 the top limb
};

__host__ __device__ __forceinline__ int clz64(unsigned long long x) {  // x != 0
#ifdef __CUDA_ARCH__
    return __clzll(static_cast<long long>(x));
#else
    return __builtin_clzll(x);
#endif
}

__host__ __device__ __forceinline__ Wide wide_add(const Wide& a, const Wide& b) {
    Wide r;
    r.w0 = a.w0 + b.w0;
    const unsigned long long c0 = r.w0 < a.w0;
    const unsigned long long t = a.w1 + b.w1;
    r.w1 = t + c0;
    const unsigned long long c1 = (t < a.w1) | (r.w1 < t);
    r.w2 = a.w2 + b.w2 + c1;
    return r;
}

__host__ __device__ __forceinline__ Wide wide_neg(const Wide& a) {
    Wide r;
    r.w0 = ~a.w0 + 1ull;
    const unsigned long long c0 = a.w0 == 0;
    r.w1 = ~a.w1 + c0;
    r.w2 = ~a.w2 + (c0 & (a.w1 == 0));
    return r;
}

// floor(a / 2^n)
__host__ __device__ __forceinline__ Wide wide_sar(const Wide& a, uint32_t n) {
    const unsigned long long fill = static_cast<long long>(a.w2) < 0 ? ~0ull : 0ull;
    if (n >= 192) return Wide{fill, fill, fill};
    const uint32_t li = n >> 6, sh = n & 63;
    auto limb = [&](uint32_t i) { return i == 0 ? a.w0 : i == 1 ? a.w1 : i == 2 ? a.w2 : fill; };
    auto out = [&](uint32_t i) { return sh ? (limb(i + li) >> sh) | (limb(i + li + 1) << (64 - sh)) : limb(i + li); };
    return Wide{out(0), out(1), out(2)};
}

__device__ __forceinline__ Wide wide_shfl_xor(const Wide& a, int o) {
    return Wide{__shfl_xor_sync(0xffffffffu, a.w0, o), __shfl_xor_sync(0xffffffffu, a.w1, o),
                __shfl_xor_sync(0xffffffffu, a.w2, o)};
}

// Exponent field of a finite term as the fold scales it (0 for +-0).
__host__ __device__ __forceinline__ uint32_t term_top(unsigned long long b) {
    if (!(b & kAbsMask)) return 0;
    const uint32_t f = static_cast<uint32_t>(b >> 52) & 0x7ffu;
    return f ? f : 1u;
}

// A finite term in units of 2^(T - 1172), truncated toward zero; T >= term_top(b).
__host__ __device__ __forceinline__ Wide term_wide(unsigned long long b, uint32_t T) {
    Wide r{0ull, 0ull, 0ull};
    const uint32_t f = static_cast<uint32_t>(b >> 52) & 0x7ffu;
    unsigned long long m = b & 0xfffffffffffffull;
    if (f) m |= 1ull << 52;
    if (!m) return r;
    const int d = static_cast<int>(f ? f : 1u) - static_cast<int>(T) + 97;  // <= 97
    if (d >= 0) {
        const uint32_t sh = static_cast<uint32_t>(d) & 63;
        const unsigned long long lo = m << sh, hi = sh ? m >> (64 - sh) : 0ull;
        if (d < 64) { r.w0 = lo; r.w1 = hi; }
        else { r.w1 = lo; r.w2 = hi; }
    } else if (d > -64) {
        r.w0 = m >> static_cast<uint32_t>(-d);
    }
    return (b >> 63) ? wide_neg(r) : r;
}

// a * 2^e rounded to the nearest double, ties to even (+0 for a = 0).
__host__ __device__ inline double wide_to_f64(Wide a, int e) {
    const bool neg = static_cast<long long>(a.w2) < 0;
    if (neg) a = wide_neg(a);
    int L;  // bit length
    if (a.w2) L = 192 - clz64(a.w2);
    else if (a.w1) L = 128 - clz64(a.w1);
    else if (a.w0) L = 64 - clz64(a.w0);
    else return 0.0;
    int lsb = e + L - 53;  // weight of the result's last mantissa bit
    if (lsb < -1074) lsb = -1074;
    const int r = lsb - e;  // bits dropped
    unsigned long long mant;
    if (r <= 0) {
        mant = a.w0 << static_cast<uint32_t>(-r);  // exact: a < 2^53 here
    } else {
        mant = wide_sar(a, static_cast<uint32_t>(r)).w0;
        const uint32_t rb = static_cast<uint32_t>(r - 1);  // the round bit
        const unsigned long long rl = rb < 64 ? a.w0 : rb < 128 ? a.w1 : a.w2;
        const bool round = (rl >> (rb & 63)) & 1ull;
        auto low = [](unsigned long long w, uint32_t n) { return n >= 64 ? w : (w & ((1ull << n) - 1ull)); };
        const bool sticky = rb <= 64 ? low(a.w0, rb) != 0
                          : rb <= 128 ? (a.w0 | low(a.w1, rb - 64)) != 0
                                      : (a.w0 | a.w1 | low(a.w2, rb - 128)) != 0;
        if (round && (sticky || (mant & 1ull))) ++mant;
        if (mant >> 53) { mant >>= 1; ++lsb; }
    }
    unsigned long long bits;
    if (mant >> 52) {
        const int biased = lsb + 1075;
        bits = biased >= 2047 ? 0x7ff0000000000000ull
                              : (static_cast<unsigned long long>(biased) << 52) | (mant & 0xfffffffffffffull);
    } else {
        bits = mant;  // subnormal: lsb = -1074
    }
    if (neg) bits |= kSignBit;
    double d;
    memcpy(&d, &bits, sizeof d);
    return d;
}

// The terms of chunk acc a (included in the query): its sum's hi and lo bits,
// zero where a non-finite part sets a flag instead (a non-finite hi carries
// the plain IEEE sum, its lo is meaningless).
__device__ __forceinline__ void chunk_terms(const ChunkAcc& a, unsigned long long& hb, unsigned long long& lb,
                                            uint32_t& special) {
    hb = static_cast<unsigned long long>(__double_as_longlong(a.fsum_hi));
    lb = static_cast<unsigned long long>(__double_as_longlong(a.fsum_lo));
    auto flag = [](unsigned long long b) -> uint32_t {
        return (b & kAbsMask) > 0x7ff0000000000000ull ? 1u : (b >> 63) ? 4u : 2u;
    };
    if ((hb & kAbsMask) >= 0x7ff0000000000000ull) {
        special |= flag(hb);
        hb = lb = 0;
    } else if ((lb & kAbsMask) >= 0x7ff0000000000000ull) {
        special |= flag(lb);
        lb = 0;
    }
}

__device__ __forceinline__ unsigned long long u64_min(unsigned long long a, unsigned long long b) { return a < b ? a : b; }
__device__ __forceinline__ unsigned long long u64_max(unsigned long long a, unsigned long long b) { return a > b ? a : b; }

// A chunk's accumulator through L2 (other CTAs of the same launch wrote it).
__device__ __forceinline__ ChunkAcc load_acc_cg(const ChunkAcc* p) {
    static_assert(sizeof(ChunkAcc) == 80, "five 16-byte words per chunk");
    const uint4* v = reinterpret_cast<const uint4*>(p);
    uint4 w[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) w[i] = __ldcg(v + i);
    ChunkAcc a;
    memcpy(&a, w, sizeof a);
    return a;
}

// Slice s of query q by one warp (every lane returns the slice's part); re-arms its chunks.
__device__ __forceinline__ ValPart slice_fold(const QueryParams& q, uint32_t s) {
    const int lane = threadIdx.x & 31;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    unsigned long long t[4] = {0ull, 0ull, 0ull, 0ull};
    unsigned long long mn = kKeyPosInf, mx = kKeyNegInf, cnt = 0;
    uint32_t special = 0, bad = 0xffffffffu, bad_st = 0;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const uint32_t c = s * kSliceChunks + 2 * lane + k;
        if (c < q.n_chunks) {
            const ChunkAcc a = load_acc_cg(q.acc + c);
            if (a.status && bad == 0xffffffffu) { bad = c; bad_st = a.status; }
            if (chunk_included(q, a)) {
                chunk_terms(a, t[2 * k], t[2 * k + 1], special);
                mn = u64_min(mn, order_key(static_cast<unsigned long long>(__double_as_longlong(a.fmin))));
                mx = u64_max(mx, order_key(static_cast<unsigned long long>(__double_as_longlong(a.fmax))));
                cnt += a.count;
            }
            ChunkAcc rest = {};
            rest.dmin = ~0ull;
            rest.fmin = inf;
            rest.fmax = -inf;
            q.acc[c] = rest;
        }
    }
    const uint32_t top = __reduce_max_sync(0xffffffffu, max(max(term_top(t[0]), term_top(t[1])),
                                                            max(term_top(t[2]), term_top(t[3]))));
    Wide w = wide_add(wide_add(term_wide(t[0], top), term_wide(t[1], top)),
                      wide_add(term_wide(t[2], top), term_wide(t[3], top)));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        w = wide_add(w, wide_shfl_xor(w, o));
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        mn = u64_min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = u64_max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    ValPart p;
    p.w0 = w.w0;
    p.w1 = w.w1;
    p.w2 = w.w2;
    p.mn = mn;
    p.mx = mx;
    p.cnt = cnt;
    p.top = top;
    p.special = __reduce_or_sync(0xffffffffu, special);
    p.bad = __reduce_min_sync(0xffffffffu, bad);
    const uint32_t owner = __ffs(__ballot_sync(0xffffffffu, bad == p.bad)) - 1;
    p.bad_st = __shfl_sync(0xffffffffu, bad_st, owner);
    return p;
}

// The query's running total: shifted slice sums and the other fields.
struct ValTotal {
    Wide w;
    unsigned long long mn, mx, cnt;
    uint32_t special, bad, bad_st;
};

__device__ __forceinline__ ValTotal val_total_rest() {
    return ValTotal{Wide{0ull, 0ull, 0ull}, kKeyPosInf, kKeyNegInf, 0ull, 0u, 0xffffffffu, 0u};
}

// t += slice part p, its sum shifted to the query's largest exponent field tq.
__device__ __forceinline__ void val_total_add(ValTotal& t, const ValPart& p, uint32_t tq) {
    t.w = wide_add(t.w, wide_sar(Wide{p.w0, p.w1, p.w2}, tq - p.top));
    t.mn = u64_min(t.mn, p.mn);
    t.mx = u64_max(t.mx, p.mx);
    t.cnt += p.cnt;
    t.special |= p.special;
    if (p.bad < t.bad) { t.bad = p.bad; t.bad_st = p.bad_st; }
}

__device__ __forceinline__ void val_total_merge(ValTotal& t, const ValTotal& o) {
    t.w = wide_add(t.w, o.w);
    t.mn = u64_min(t.mn, o.mn);
    t.mx = u64_max(t.mx, o.mx);
    t.cnt += o.cnt;
    t.special |= o.special;
    if (o.bad < t.bad) { t.bad = o.bad; t.bad_st = o.bad_st; }
}

// Warp merge (every lane ends with the total).
__device__ __forceinline__ ValTotal val_total_warp(ValTotal t) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ValTotal b;
        b.w = wide_shfl_xor(t.w, o);
        b.mn = __shfl_xor_sync(0xffffffffu, t.mn, o);
        b.mx = __shfl_xor_sync(0xffffffffu, t.mx, o);
        b.cnt = __shfl_xor_sync(0xffffffffu, t.cnt, o);
        b.special = __shfl_xor_sync(0xffffffffu, t.special, o);
        b.bad = __shfl_xor_sync(0xffffffffu, t.bad, o);
        b.bad_st = __shfl_xor_sync(0xffffffffu, t.bad_st, o);
        val_total_merge(t, b);
    }
    return t;
}

__device__ inline QueryResult val_total_result(const ValTotal& t, uint32_t tq) {
    QueryResult r;
    r.status = t.bad == 0xffffffffu ? 0u : t.bad_st;
    r.bad_chunk = t.bad;
    if ((t.special & 1u) || (t.special & 6u) == 6u) r.sum = __longlong_as_double(0x7fffffffffffffffll);
    else if (t.special & 2u) r.sum = __longlong_as_double(0x7ff0000000000000ll);
    else if (t.special & 4u) r.sum = __longlong_as_double(static_cast<long long>(0xfff0000000000000ull));
    else r.sum = wide_to_f64(t.w, static_cast<int>(tq) - 1172);
    r.min = __longlong_as_double(static_cast<long long>(key_bits(t.mn)));
    r.max = __longlong_as_double(static_cast<long long>(key_bits(t.mx)));
    r.count = t.cnt;
    return r;
}

// The largest exponent field among the included chunks' terms (thread-local
// part of the query's tq: chunks c0, c0 + stride, ...).
__device__ __forceinline__ uint32_t terms_top(const QueryParams& q, uint32_t c0, uint32_t stride) {
    uint32_t top = 0;
    for (uint32_t c = c0; c < q.n_chunks; c += stride) {
        const ChunkAcc a = q.acc[c];
        if (!chunk_included(q, a)) continue;
        unsigned long long hb, lb;
        uint32_t sp = 0;
        chunk_terms(a, hb, lb, sp);
        top = max(top, max(term_top(hb), term_top(lb)));
    }
    return top;
}

// The whole fold of a non-BUFF query by one CTA of kFinThreads threads (the
// batched path: one CTA per query): the query's tq first, then warps fold
// slices 32 at a time and keep the shifted sums.
__device__ inline void fold_values_cta(const QueryParams& q, QueryResult* res) {
    __shared__ uint32_t s_top[kFinThreads / 32];
    __shared__ ValTotal s_tot[kFinThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    constexpr int kWarps = kFinThreads / 32;
    uint32_t tq = __reduce_max_sync(0xffffffffu, terms_top(q, threadIdx.x, kFinThreads));
    if (lane == 0) s_top[wid] = tq;
    __syncthreads();  // every read of the accumulators above precedes the slices' re-arming
    tq = 0;
    for (int w = 0; w < kWarps; ++w) tq = max(tq, s_top[w]);
    const uint32_t S = value_slices(q.n_chunks);
    ValTotal t = val_total_rest();
    for (uint32_t s = wid; s < S; s += kWarps) val_total_add(t, slice_fold(q, s), tq);
    if (lane == 0) s_tot[wid] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kWarps; ++w) val_total_merge(t, s_tot[w]);
        *res = val_total_result(t, tq);
    }
}

// ---- the grid fold's scratch: slice parts, then the CTA counter --------------
__device__ __forceinline__ unsigned int* fold_counters(ValPart* parts, uint32_t S) {
    return reinterpret_cast<unsigned int*>(parts + S);
}

__device__ __forceinline__ ValPart load_part(const ValPart* p) {
    const ulonglong2* v = reinterpret_cast<const ulonglong2*>(p);
    const ulonglong2 a = __ldcg(v), b = __ldcg(v + 1), c = __ldcg(v + 2);
    const uint4 d = __ldcg(reinterpret_cast<const uint4*>(p) + 3);
    ValPart r;
    r.w0 = a.x;
    r.w1 = a.y;
    r.w2 = b.x;
    r.mn = b.y;
    r.mx = c.x;
    r.cnt = c.y;
    r.top = d.x;
    r.special = d.y;
    r.bad = d.z;
    r.bad_st = d.w;
    return r;
}

// One warp sums the S slice parts (written by other CTAs: read through L2) into *res.
__device__ inline void fold_parts_warp(const ValPart* parts, uint32_t S, QueryResult* res) {
    const int lane = threadIdx.x & 31;
    uint32_t tq = 0;
    for (uint32_t i = lane; i < S; i += 32) tq = max(tq, __ldcg(&parts[i].top));
    tq = __reduce_max_sync(0xffffffffu, tq);
    ValTotal t = val_total_rest();
    for (uint32_t i = lane; i < S; i += 32) val_total_add(t, load_part(parts + i), tq);
    t = val_total_warp(t);
    if (lane == 0) *res = val_total_result(t, tq);
}

// Folds BUFF query q's per-chunk partials in chunk order into *res and
// re-arms q.acc.  A CTA of kFinThreads threads.
__device__ __forceinline__ void finalize_chunks(const QueryParams& q, QueryResult* res) {
    __shared__ unsigned long long sh_u[32];
    __shared__ long long sh_i[32];
    const uint32_t nc = q.n_chunks;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);

    uint32_t bad = 0xffffffffu;
    unsigned long long cnt = 0;
    // integer facts (BUFF)
    long long ssum = 0, smax = LLONG_MIN, smin = LLONG_MAX;
    unsigned long long sabs = 0;
    uint32_t fracmin = 0xffffffffu, fracmax = 0, exact = 1, any = 0;
    // each thread folds a contiguous run of chunks, runs combine in thread order
    const uint32_t per = (nc + kFinThreads - 1) / kFinThreads;
    const uint32_t c0 = min(nc, threadIdx.x * per), c1 = min(nc, c0 + per);
    for (uint32_t c = c0; c < c1; ++c) {
        const ChunkAcc a = q.acc[c];
        if (a.status && bad == 0xffffffffu) bad = c;
        if (!chunk_included(q, a)) continue;
        any = 1;
        cnt += a.count;
        const BuffVal v = buff_value(q, c, a);
        exact &= v.sum_exact;
        ssum += v.sum_fixed;
        const unsigned long long ab = static_cast<unsigned long long>(v.sum_fixed < 0 ? -v.sum_fixed : v.sum_fixed);
        sabs = (sabs + ab < sabs || sabs + ab > (1ull << 62)) ? (1ull << 62) : sabs + ab;
        smax = max(smax, v.max_fixed);
        smin = min(smin, v.min_fixed);
        fracmin = min(fracmin, v.frac);
        fracmax = max(fracmax, v.frac);
    }
    bad = block_reduce<unsigned long long>(bad, [](unsigned long long x, unsigned long long y) { return x < y ? x : y; }, sh_u);
    cnt = block_reduce<unsigned long long>(cnt, [](unsigned long long x, unsigned long long y) { return x + y; }, sh_u);
    any = static_cast<uint32_t>(block_reduce<unsigned long long>(any, [](unsigned long long x, unsigned long long y) { return x | y; }, sh_u));
    QueryResult r;
    r.status = 0;
    r.bad_chunk = static_cast<uint32_t>(bad);
    r.count = cnt;
    ssum = block_reduce<long long>(ssum, [](long long x, long long y) { return x + y; }, sh_i);
    smax = block_reduce<long long>(smax, [](long long x, long long y) { return x > y ? x : y; }, sh_i);
    smin = block_reduce<long long>(smin, [](long long x, long long y) { return x < y ? x : y; }, sh_i);
    sabs = block_reduce<unsigned long long>(sabs, [](unsigned long long x, unsigned long long y) {
        return x + y > (1ull << 62) ? (1ull << 62) : x + y; }, sh_u);
    exact = static_cast<uint32_t>(block_reduce<unsigned long long>(exact, [](unsigned long long x, unsigned long long y) { return x & y; }, sh_u));
    fracmin = static_cast<uint32_t>(block_reduce<unsigned long long>(fracmin, [](unsigned long long x, unsigned long long y) { return x < y ? x : y; }, sh_u));
    fracmax = static_cast<uint32_t>(block_reduce<unsigned long long>(fracmax, [](unsigned long long x, unsigned long long y) { return x > y ? x : y; }, sh_u));
    if (threadIdx.x == 0) {
        if (!any) {
            r.sum = 0.0; r.min = inf; r.max = -inf;
        } else if (fracmin == fracmax) {
            // Every chunk value is integer * 2^-frac: min and max convert once.
            r.max = fold_scale(smax, fracmin);
            r.min = fold_scale(smin, fracmin);
            if (exact && sabs < (1ull << 53)) {
                // Each chunk sum and every prefix of the chunk-ordered fold is
                // an exact multiple of 2^-frac below 2^53 of them, so the
                // reference's sequential f64 fold is exact: it equals the total.
                r.sum = fold_scale(ssum, fracmin);
            } else {
                double s = 0.0;  // the reference's sequential `result += chunk_sum`
                for (uint32_t c = 0; c < nc; ++c) {
                    const ChunkAcc a = q.acc[c];
                    if (chunk_included(q, a)) s += buff_chunk_sum_f64(buff_value(q, c, a), c, q);
                }
                r.sum = s;
            }
        } else {
            double s = 0.0, a1 = inf, b1 = -inf;
            for (uint32_t c = 0; c < nc; ++c) {
                const ChunkAcc a = q.acc[c];
                if (!chunk_included(q, a)) continue;
                const BuffVal v = buff_value(q, c, a);
                s += buff_chunk_sum_f64(v, c, q);
                a1 = fmin(a1, fold_scale(v.min_fixed, v.frac));
                b1 = fmax(b1, fold_scale(v.max_fixed, v.frac));
            }
            r.sum = s; r.min = a1; r.max = b1;
        }
    }
    if (threadIdx.x == 0) {
        if (r.bad_chunk != 0xffffffffu) r.status = q.acc[r.bad_chunk].status;
        *res = r;
    }
    __syncthreads();
    // re-arm the accumulators for the next query
    for (uint32_t c = threadIdx.x; c < nc; c += blockDim.x) {
        ChunkAcc a = {};
        a.dmin = ~0ull;
        a.fmin = inf;
        a.fmax = -inf;
        q.acc[c] = a;
    }
}


}  // namespace
}  // namespace ebi
