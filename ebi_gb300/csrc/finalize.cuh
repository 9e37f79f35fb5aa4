// finalize.cuh -- the chunk-ordered fold of per-chunk results (Decoder's
// `result += chunk`, `result = result.min(chunk)`, `result = result.max(chunk)`,
// api/decoder.rs:323-439), shared by the single-query finalize (query.cu) and
// the batched launch (batch.cu).
#pragma once

#include <climits>

#include "fold.cuh"

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

// Folds query q's per-chunk partials in chunk order into *res and re-arms
// q.acc.  A CTA of kFinThreads threads.
__device__ __forceinline__ void finalize_chunks(const QueryParams& q, QueryResult* res) {
    __shared__ unsigned long long sh_u[32];
    __shared__ long long sh_i[32];
    __shared__ double sh_h[32], sh_l[32];
    const uint32_t nc = q.n_chunks;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);

    uint32_t bad = 0xffffffffu;
    unsigned long long cnt = 0;
    // integer facts (BUFF)
    long long ssum = 0, smax = LLONG_MIN, smin = LLONG_MAX;
    unsigned long long sabs = 0;
    uint32_t fracmin = 0xffffffffu, fracmax = 0, exact = 1, any = 0;
    // floating facts (other codecs)
    double mn = inf, mx = -inf, hi = 0.0, lo = 0.0;
    // each thread folds a contiguous run of chunks, runs combine in thread order
    const uint32_t per = (nc + kFinThreads - 1) / kFinThreads;
    const uint32_t c0 = min(nc, threadIdx.x * per), c1 = min(nc, c0 + per);
    for (uint32_t c = c0; c < c1; ++c) {
        const ChunkAcc a = q.acc[c];
        if (a.status && bad == 0xffffffffu) bad = c;
        if (!chunk_included(q, a)) continue;
        any = 1;
        cnt += a.count;
        if (q.scheme == EBI_BUFF) {
            const BuffVal v = buff_value(q, c, a);
            exact &= v.sum_exact;
            ssum += v.sum_fixed;
            const unsigned long long ab = static_cast<unsigned long long>(v.sum_fixed < 0 ? -v.sum_fixed : v.sum_fixed);
            sabs = (sabs + ab < sabs || sabs + ab > (1ull << 62)) ? (1ull << 62) : sabs + ab;
            smax = max(smax, v.max_fixed);
            smin = min(smin, v.min_fixed);
            fracmin = min(fracmin, v.frac);
            fracmax = max(fracmax, v.frac);
        } else {
            mn = fmin(mn, a.fmin);
            mx = fmax(mx, a.fmax);
            dd_add(hi, lo, a.fsum_hi, a.fsum_lo);
        }
    }
    bad = block_reduce<unsigned long long>(bad, [](unsigned long long x, unsigned long long y) { return x < y ? x : y; }, sh_u);
    cnt = block_reduce<unsigned long long>(cnt, [](unsigned long long x, unsigned long long y) { return x + y; }, sh_u);
    any = static_cast<uint32_t>(block_reduce<unsigned long long>(any, [](unsigned long long x, unsigned long long y) { return x | y; }, sh_u));
    QueryResult r;
    r.status = 0;
    r.bad_chunk = static_cast<uint32_t>(bad);
    r.count = cnt;
    if (q.scheme == EBI_BUFF) {
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
    } else {
        mn = block_reduce<double>(mn, [](double x, double y) { return fmin(x, y); }, sh_h);
        mx = block_reduce<double>(mx, [](double x, double y) { return fmax(x, y); }, sh_h);
        // double-double partial sums in a fixed tree (lane order = chunk order)
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double oh = __shfl_down_sync(0xffffffffu, hi, o), ol = __shfl_down_sync(0xffffffffu, lo, o);
            if ((lane & (2 * o - 1)) == 0) dd_add(hi, lo, oh, ol);
        }
        if (lane == 0) { sh_h[wid] = hi; sh_l[wid] = lo; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double th = 0.0, tl = 0.0;
            for (int w = 0; w < kFinThreads / 32; ++w) dd_add(th, tl, sh_h[w], sh_l[w]);
            r.sum = th + tl;
            r.min = mn;
            r.max = mx;
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
