// query.cu -- kernels shared by every codec: chunk selection, tile scans and
// the chunk-ordered fold of per-chunk results (Decoder's `result += chunk`,
// `result = result.min(chunk)`, `result = result.max(chunk)`,
// api/decoder.rs:323-439).
#include "internal.h"

namespace ebi {
namespace {

constexpr int kFinThreads = 1024;

__global__ void acc_init_kernel(ChunkAcc* acc, uint32_t n) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        ChunkAcc a = {};
        a.dmin = ~0ull;
        a.fmin = __longlong_as_double(0x7ff0000000000000ll);
        a.fmax = __longlong_as_double(static_cast<long long>(0xfff0000000000000ull));
        acc[c] = a;
    }
}

// acc[c].selected for chunk c = blockIdx.x (grid-stride): the chunk passes
// chunk_id and the input bitmask intersects its rows (api/decoder.rs:258-268).
__global__ void select_chunks_kernel(QueryParams q) {
    __shared__ int any;
    for (uint32_t c = blockIdx.x; c < q.n_chunks; c += gridDim.x) {
        if (threadIdx.x == 0) any = 0;
        __syncthreads();
        const ChunkDesc cd = q.chunks[c];
        const bool id_ok = q.chunk_id < 0 || static_cast<uint64_t>(q.chunk_id) == c;
        if (id_ok) {
            // logical_record_range_u32: rows [row_off, row_off + n_rows)
            for (uint64_t r = uint64_t(threadIdx.x) * 32; r < cd.n_rows && !any; r += uint64_t(blockDim.x) * 32) {
                const uint64_t left = cd.n_rows - r;
                uint32_t w = mask_word(q.in_mask, cd.row_off + r, q.n_records);
                if (left < 32) w &= (1u << left) - 1u;
                if (w) any = 1;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) q.acc[c].selected = static_cast<uint32_t>(id_ok && any);
        __syncthreads();
    }
}

// Exclusive scan of tile counts (one CTA; tiles are few thousands).
__global__ void tile_scan_kernel(const unsigned long long* counts, unsigned long long* offsets, uint32_t n) {
    __shared__ unsigned long long wsum[32];
    __shared__ unsigned long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (uint32_t base = 0; base < n; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const unsigned long long v = i < n ? counts[i] : 0;
        unsigned long long inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) wsum[wid] = inc;
        __syncthreads();
        if (wid == 0) {
            unsigned long long x = lane < static_cast<int>(blockDim.x >> 5) ? wsum[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            wsum[lane] = x;  // inclusive warp prefix
        }
        __syncthreads();
        const unsigned long long before = (wid ? wsum[wid - 1] : 0) + carry;
        if (i < n) offsets[i] = before + inc - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + inc;
        __syncthreads();
    }
    if (threadIdx.x == 0) offsets[n] = carry;
}

struct BuffHdr {
    int64_t base;
    uint32_t n, bits, frac;
};
__device__ BuffHdr read_buff_hdr(const QueryParams& q, uint32_t c) {
    const uint8_t* p = q.file + q.chunks[c].byte_off;
    BuffHdr h;
    h.base = static_cast<int64_t>(load_u64_unaligned(p));
    h.n = load_u32_unaligned(p + 8);
    h.bits = load_u32_unaligned(p + 12);
    h.frac = load_u32_unaligned(p + 16);
    return h;
}
__device__ double pow2(uint32_t frac) {  // 2.0f64.powi(frac): exact, +inf past 1023
    return frac <= 1023 ? __longlong_as_double(static_cast<long long>(uint64_t(1023 + frac) << 52))
                        : __longlong_as_double(0x7ff0000000000000ll);
}

// One chunk's contribution, in the reference's arithmetic.
struct ChunkVal {
    double sum, mn, mx;
    long long exact;       // BUFF: the sum as an integer multiple of 2^-frac, when exact
    uint32_t frac;
    bool exact_ok;         // |exact| < 2^53 and sum == exact * 2^-frac
    bool included;
};

__device__ ChunkVal chunk_value(const QueryParams& q, uint32_t c, const ChunkAcc& a) {
    ChunkVal v;
    v.included = q.op == OP_FILTER_AGG ? a.count > 0 : a.selected != 0;
    v.sum = 0.0;
    v.mn = __longlong_as_double(0x7ff0000000000000ll);
    v.mx = -v.mn;
    v.exact = 0; v.frac = 0; v.exact_ok = false;
    if (!v.included || a.status) { v.included = false; return v; }
    if (q.scheme == EBI_BUFF) {
        const BuffHdr h = read_buff_hdr(q, c);
        const double scale = pow2(h.frac);
        v.frac = h.frac;
        const double basev = static_cast<double>(h.base) / scale;
        const bool has_mask = q.in_mask != nullptr || q.op == OP_FILTER_AGG;
        if (h.bits == 0) {
            // sum_with_bitmask: base / scale * number_of_records (buff/sum.rs:81-84)
            v.sum = basev * static_cast<double>(h.n);
            v.mn = v.mx = basev;
            const __int128 p = static_cast<__int128>(h.base) * h.n;
            v.exact_ok = p < (static_cast<__int128>(1) << 53) && p > -(static_cast<__int128>(1) << 53) &&
                         h.base < (1ll << 53) && h.base > -(1ll << 53) && h.frac <= 1022;
            v.exact = static_cast<long long>(p);
        } else {
            const unsigned long long cnt = a.count;
            const long long s = static_cast<long long>(a.isum + static_cast<unsigned long long>(h.base) * cnt);
            v.sum = static_cast<double>(s) / scale;
            v.exact = s;
            v.exact_ok = s < (1ll << 53) && s > -(1ll << 53) && h.frac <= 1022;
            v.mx = static_cast<double>(static_cast<long long>(static_cast<unsigned long long>(h.base) + a.dmax)) / scale;
            // min_without_bitmask returns base / scale (buff/min_max.rs:435-460)
            v.mn = has_mask ? static_cast<double>(static_cast<long long>(static_cast<unsigned long long>(h.base) + a.dmin)) / scale
                            : basev;
        }
    } else {
        v.sum = a.fsum_hi;
        v.mn = a.fmin;
        v.mx = a.fmax;
    }
    return v;
}

__global__ void __launch_bounds__(kFinThreads) finalize_kernel(QueryParams q, QueryResult* res) {
    __shared__ uint32_t s_bad[32];
    __shared__ double s_mn[32], s_mx[32], s_hi[32], s_lo[32];
    __shared__ unsigned long long s_cnt[32], s_abs[32];
    __shared__ long long s_exact[32];
    __shared__ uint32_t s_fracmin[32], s_fracmax[32], s_allexact[32];
    const uint32_t nc = q.n_chunks;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);

    uint32_t bad = 0xffffffffu;
    double mn = inf, mx = -inf, hi = 0.0, lo = 0.0;
    unsigned long long cnt = 0, sabs = 0;
    long long sexact = 0;
    uint32_t fracmin = 0xffffffffu, fracmax = 0, allexact = 1;
    // Each thread folds a contiguous run of chunks in order; runs are then
    // combined in thread order, so the combination order is fixed.
    const uint32_t per = (nc + kFinThreads - 1) / kFinThreads;
    const uint32_t c0 = threadIdx.x * per, c1 = min(nc, c0 + per);
    for (uint32_t c = c0; c < c1; ++c) {
        const ChunkAcc a = q.acc[c];
        if (a.status && bad == 0xffffffffu) bad = c;
        const ChunkVal v = chunk_value(q, c, a);
        if (!v.included) continue;
        cnt += a.count;
        mn = fmin(mn, v.mn);
        mx = fmax(mx, v.mx);
        if (q.scheme == EBI_BUFF) {
            allexact &= v.exact_ok;
            if (v.exact_ok) {
                sexact += v.exact;
                const unsigned long long ab = static_cast<unsigned long long>(v.exact < 0 ? -v.exact : v.exact);
                sabs = sabs + ab < sabs || sabs + ab > (1ull << 62) ? (1ull << 62) : sabs + ab;
            }
            fracmin = min(fracmin, v.frac);
            fracmax = max(fracmax, v.frac);
        } else {
            dd_add(hi, lo, q.acc[c].fsum_hi, q.acc[c].fsum_lo);
        }
    }
    // warp reduction (lane order = chunk order)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        bad = min(bad, __shfl_xor_sync(0xffffffffu, bad, o));
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        {
            const unsigned long long x = __shfl_xor_sync(0xffffffffu, sabs, o);
            sabs = sabs + x > (1ull << 62) ? (1ull << 62) : sabs + x;
        }
        sexact += __shfl_xor_sync(0xffffffffu, sexact, o);
        fracmin = min(fracmin, __shfl_xor_sync(0xffffffffu, fracmin, o));
        fracmax = max(fracmax, __shfl_xor_sync(0xffffffffu, fracmax, o));
        allexact &= __shfl_xor_sync(0xffffffffu, allexact, o);
    }
    // double-double partial sums combined in a fixed tree over lanes
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double oh = __shfl_down_sync(0xffffffffu, hi, o), ol = __shfl_down_sync(0xffffffffu, lo, o);
        if ((lane & (2 * o - 1)) == 0) dd_add(hi, lo, oh, ol);
    }
    if (lane == 0) {
        s_bad[wid] = bad; s_mn[wid] = mn; s_mx[wid] = mx; s_hi[wid] = hi; s_lo[wid] = lo;
        s_cnt[wid] = cnt; s_abs[wid] = sabs; s_exact[wid] = sexact;
        s_fracmin[wid] = fracmin; s_fracmax[wid] = fracmax; s_allexact[wid] = allexact;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        QueryResult r;
        r.status = 0; r.bad_chunk = 0xffffffffu;
        double tmn = inf, tmx = -inf, th = 0.0, tl = 0.0;
        unsigned long long tc = 0, tabs = 0;
        long long tex = 0;
        uint32_t fmn = 0xffffffffu, fmx = 0, ae = 1;
        for (int w = 0; w < kFinThreads / 32; ++w) {
            if (s_bad[w] < r.bad_chunk) r.bad_chunk = s_bad[w];
            tmn = fmin(tmn, s_mn[w]); tmx = fmax(tmx, s_mx[w]);
            dd_add(th, tl, s_hi[w], s_lo[w]);
            tc += s_cnt[w]; tex += s_exact[w];
            tabs = tabs + s_abs[w] > (1ull << 62) ? (1ull << 62) : tabs + s_abs[w];
            fmn = min(fmn, s_fracmin[w]); fmx = max(fmx, s_fracmax[w]); ae &= s_allexact[w];
        }
        if (r.bad_chunk != 0xffffffffu) r.status = q.acc[r.bad_chunk].status;
        r.min = tmn; r.max = tmx; r.count = tc;
        if (q.scheme == EBI_BUFF) {
            if (tc == 0 && fmn == 0xffffffffu) {
                r.sum = 0.0;
            } else if (ae && fmn == fmx && tabs < (1ull << 53)) {
                // Every chunk sum and every prefix of the chunk-ordered fold is an
                // exact multiple of 2^-frac below 2^53 ulps: the sequential fold
                // of the reference is exact, so it equals the exact total.
                r.sum = static_cast<double>(tex) / pow2(fmn);
            } else {
                // the reference's sequential `result += chunk_sum`
                double s = 0.0;
                for (uint32_t c = 0; c < nc; ++c) {
                    const ChunkVal v = chunk_value(q, c, q.acc[c]);
                    if (v.included) s += v.sum;
                }
                r.sum = s;
            }
        } else {
            r.sum = th + tl;
        }
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

cudaError_t launch_acc_init(ChunkAcc* acc, uint32_t n, cudaStream_t s) {
    if (!n) return cudaSuccess;
    acc_init_kernel<<<(n + 255) / 256, 256, 0, s>>>(acc, n);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_select_chunks(const QueryParams& q, cudaStream_t s) {
    if (!q.n_chunks) return cudaSuccess;
    const uint32_t grid = q.n_chunks < 4096 ? q.n_chunks : 4096;
    select_chunks_kernel<<<grid, 256, 0, s>>>(q);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_tile_scan(const unsigned long long* counts, unsigned long long* offsets, uint32_t n,
                             cudaStream_t s) {
    tile_scan_kernel<<<1, 1024, 0, s>>>(counts, offsets, n);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_finalize(const QueryParams& q, QueryResult* res, cudaStream_t s) {
    finalize_kernel<<<1, kFinThreads, 0, s>>>(q, res);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ebi
