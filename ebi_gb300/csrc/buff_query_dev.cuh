// buff_query_dev.cuh -- device pieces shared by the BUFF scan kernels
// (buff_scan.cu): the query compiled per chunk into one range test on the
// delta, per-chunk partials with the warp's exact totals, and the last CTA's
// fold of the query result.
#pragma once

#include <climits>

#include <cuda/atomic>

#include "buff_common.cuh"
#include "fold.cuh"

namespace ebi {
namespace {
using namespace buff;

// The query folded, per chunk, into one unsigned range test on the delta:
//   sel = (negate ? ~cmp : cmp) & (use_mask ? bitmask : valid rows)
// with cmp = lo <= delta <= hi (all rows when `full`, none when `empty`).
// It reproduces the reference's in-situ decisions, including the shortcuts
// that return all rows without looking at the input bitmask.
struct RangeProg {
    uint64_t lo, hi;
    uint32_t empty, full, negate, use_mask;
};

__device__ RangeProg compile_prog(const QueryParams& q, const BuffPred& k, uint32_t bits, bool has_mask) {
    RangeProg g{0, ~0ull, 0, 0, 0, 0};
    const uint64_t dmax = bits >= 64 ? ~0ull : ((1ull << bits) - 1);
    if (q.op == OP_AGG) {  // no predicate: the rows of the bitmask (all rows without one)
        g.full = 1;
        g.use_mask = has_mask;
        return g;
    }
    if (q.pred.kind == EBI_PRED_RANGE) {
        const bool la = k.lmode == SIDE_ABSENT, ra = k.rmode == SIDE_ABSENT;
        if (k.lmode == SIDE_NONE || k.rmode == SIDE_NONE) g.empty = 1;
        if (k.lmode == SIDE_CMP) {
            if (!k.lincl && k.lthr >= dmax) g.empty = 1;
            else g.lo = k.lincl ? k.lthr : k.lthr + 1;
        }
        if (k.rmode == SIDE_CMP) {
            if (!k.rincl && k.rthr == 0) g.empty = 1;
            else g.hi = k.rincl ? k.rthr : k.rthr - 1;
        }
        if (!g.empty && g.lo > g.hi) g.empty = 1;
        g.use_mask = k.lmode == SIDE_CMP || k.rmode == SIDE_CMP || (la && ra);
    } else {
        if (k.emode == SIDE_NONE) g.empty = 1;
        else if (k.emode == SIDE_CMP) { g.lo = g.hi = k.etgt; g.use_mask = 1; }
        if (q.pred.kind == EBI_PRED_NE) { g.negate = 1; g.use_mask = 1; }
    }
    g.full = !g.empty && g.lo == 0 && g.hi >= dmax;
    g.use_mask = g.use_mask && has_mask;
    return g;
}

struct Partial {
    unsigned long long sum, cnt, mx, mn;
};


__device__ __forceinline__ unsigned long long sat_add(unsigned long long a, unsigned long long b) {
    const unsigned long long c = a + b;
    return c < a ? ~0ull : c;
}

// Ends a warp's run over one chunk: per-chunk partials (for the chunk-ordered
// fallback fold) and the warp's exact query totals.
// `to_acc` false: the column's totals are exact whatever the query (see
// cta_finish), and the chunk-ordered fold that reads the accumulators never runs.
__device__ __forceinline__ void flush_partial(const QueryParams& q, uint32_t chunk, int64_t base, Partial& p,
                                              WarpTot& wt, bool to_acc = true) {
    const unsigned long long s = warp_sum(p.sum), c = warp_sum(p.cnt), mx = warp_max_u64(p.mx), mn = warp_min_u64(p.mn);
    if ((threadIdx.x & 31) == 0 && c) {
        if (to_acc) {
            ChunkAcc* a = q.acc + chunk;
            atomicAdd(&a->isum, s);
            atomicAdd(&a->count, c);
            atomicMax(&a->dmax, mx);
            atomicMin(&a->dmin, mn);
        }
        const __int128 piece = static_cast<__int128>(s) + static_cast<__int128>(base) * static_cast<__int128>(c);
        const __int128 ap = piece < 0 ? -piece : piece;
        wt.sum_fixed += static_cast<unsigned long long>(piece);
        if (ap >= (static_cast<__int128>(1) << 53)) wt.nonexact = 1;
        else wt.abs_bound = sat_add(wt.abs_bound, static_cast<unsigned long long>(ap));
        wt.count += c;
        const long long fmax = static_cast<long long>(static_cast<unsigned long long>(base) + mx);
        const long long fmin = static_cast<long long>(static_cast<unsigned long long>(base) + mn);
        wt.max_fixed = fmax > wt.max_fixed ? fmax : wt.max_fixed;
        wt.min_fixed = fmin < wt.min_fixed ? fmin : wt.min_fixed;
    }
    p.sum = 0; p.cnt = 0; p.mx = 0; p.mn = ~0ull;
}

__device__ __forceinline__ void chunk_error(const QueryParams& q, ScanTotals* T, uint32_t c, uint32_t code) {
    set_status(q.acc + c, code);
    atomicMin(&T->bad_chunk, c);
}

// A scan's totals at rest (the state every query starts from).
__device__ __forceinline__ void scan_totals_rest(ScanTotals* T) {
    T->sum_fixed = 0; T->abs_bound = 0; T->count = 0;
    T->max_fixed = LLONG_MIN; T->min_fixed = LLONG_MAX;
    T->done = 0; T->bad_chunk = 0xffffffffu; T->nonexact = 0; T->next = 0;
}

// The last CTA's fold of the query totals (chunk-ordered fallback when the
// exact integer total does not apply).
__device__ void scan_finalize(const QueryParams& q, const BuffChunkInfo* info, ScanTotals* T, const ScanTotals& t,
                              QueryResult* res, uint32_t frac, bool fast_ok, bool exact) {
    __shared__ QueryResult r;
    if (threadIdx.x == 0) {
        const double inf = __longlong_as_double(0x7ff0000000000000ll);
        r.status = 0;
        r.bad_chunk = t.bad_chunk;
        if (t.bad_chunk != 0xffffffffu) r.status = q.acc[t.bad_chunk].status;
        r.count = t.count;
        r.sum = 0.0; r.min = inf; r.max = -inf;
        if (fast_ok && !t.nonexact && t.abs_bound < (1ull << 52)) {
            // Every chunk sum and every prefix of the chunk-ordered fold is an
            // exact multiple of 2^-frac below 2^53 of them: the reference's
            // sequential f64 fold is exact and equals the exact total.
            if (t.count) {
                r.sum = fold_scale(static_cast<long long>(t.sum_fixed), frac);
                r.max = fold_scale(t.max_fixed, frac);
                r.min = fold_scale(t.min_fixed, frac);
            }
        } else {
            fold_buff_chunks(q, r);
        }
        *res = r;
        scan_totals_rest(T);
    }
    __syncthreads();
    // re-arm the accumulators the query touched (all of them but in an exact
    // query without an input bitmask and without errors)
    if (exact && q.in_mask == nullptr && t.bad_chunk == 0xffffffffu) return;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    for (uint32_t c = threadIdx.x; c < q.n_chunks; c += blockDim.x) {
        ChunkAcc a = {};
        a.dmin = ~0ull;
        a.fmin = inf;
        a.fmax = -inf;
        q.acc[c] = a;
    }
}

__device__ __forceinline__ void add_tot(WarpTot& a, const WarpTot& b) {
    a.sum_fixed += b.sum_fixed;
    a.count += b.count;
    a.abs_bound = sat_add(a.abs_bound, b.abs_bound);
    a.max_fixed = b.max_fixed > a.max_fixed ? b.max_fixed : a.max_fixed;
    a.min_fixed = b.min_fixed < a.min_fixed ? b.min_fixed : a.min_fixed;
    a.nonexact |= b.nonexact;
}

// Every CTA stores its warps' totals in its slot; the last CTA to finish
// reduces the slots and folds the query into *res (the exact integer totals,
// else the chunk-ordered fold).  One atomic per CTA (the `done` count).
// `exact`: the column's totals are exact for any query (its chunks share one
// frac and the sum of |value| over all rows stays below 2^52), so the
// per-chunk accumulators are neither fed nor re-armed.
// totals_only: the CTA adds its totals into T with fire-and-forget atomics
// and no CTA folds (no fence, no slot reduction): the host reads T after the
// kernel and scales the exact totals itself.  Only for exact columns queried
// without an input bitmask, whose per-chunk accumulators are never touched.
__device__ __forceinline__ void cta_finish(const QueryParams& q, const BuffChunkInfo* info, ScanTotals* T,
                                           QueryResult* res, uint32_t frac, bool fast_ok, const WarpTot* wtot,
                                           int n_warps, bool exact = false, bool totals_only = false) {
    WarpTot* slots = scan_slots(T);
    __syncthreads();
    if (totals_only) {
        if (threadIdx.x == 0) {
            WarpTot c{0, 0, 0, LLONG_MIN, LLONG_MAX, 0};
            for (int w = 0; w < n_warps; ++w) add_tot(c, wtot[w]);
            if (c.count) {
                atomicAdd(&T->sum_fixed, c.sum_fixed);
                atomicAdd(&T->count, c.count);
                atomicMax(&T->max_fixed, c.max_fixed);
                atomicMin(&T->min_fixed, c.min_fixed);
                // every CTA's bound is below 2^52 or flagged: the sum of at most kScanSlots of them cannot wrap
                if (c.nonexact || c.abs_bound >= (1ull << 52)) atomicOr(&T->nonexact, 1u);
                else atomicAdd(&T->abs_bound, c.abs_bound);
            }
        }
        return;
    }
    __shared__ unsigned int s_last;
    if (threadIdx.x == 0) {
        WarpTot c{0, 0, 0, LLONG_MIN, LLONG_MAX, 0};
        for (int w = 0; w < n_warps; ++w) add_tot(c, wtot[w]);
        slots[blockIdx.x] = c;
        // release: the slot is visible before the count; acquire: the last
        // CTA sees every slot (its other threads through the barrier below)
        cuda::atomic_ref<unsigned int, cuda::thread_scope_device> done(T->done);
        s_last = done.fetch_add(1u, cuda::memory_order_acq_rel) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    // reduce the CTAs' slots (published before their `done` increments,
    // read from L2): per thread, then per warp, then across warps
    WarpTot c{0, 0, 0, LLONG_MIN, LLONG_MAX, 0};
    static_assert(sizeof(WarpTot) == 48, "three 16-byte words per slot");
    for (uint32_t i = threadIdx.x; i < gridDim.x; i += blockDim.x) {
        // L2 loads (the slots were written by other SMs), three per slot, all in flight together
        const ulonglong2* p = reinterpret_cast<const ulonglong2*>(slots + i);
        const ulonglong2 a = __ldcg(p), b = __ldcg(p + 1), d = __ldcg(p + 2);
        WarpTot x;
        x.sum_fixed = a.x;
        x.count = a.y;
        x.abs_bound = b.x;
        x.max_fixed = static_cast<long long>(b.y);
        x.min_fixed = static_cast<long long>(d.x);
        x.nonexact = static_cast<unsigned int>(d.y);
        add_tot(c, x);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        WarpTot y;
        y.sum_fixed = __shfl_xor_sync(0xffffffffu, c.sum_fixed, o);
        y.count = __shfl_xor_sync(0xffffffffu, c.count, o);
        y.abs_bound = __shfl_xor_sync(0xffffffffu, c.abs_bound, o);
        y.max_fixed = __shfl_xor_sync(0xffffffffu, c.max_fixed, o);
        y.min_fixed = __shfl_xor_sync(0xffffffffu, c.min_fixed, o);
        y.nonexact = __shfl_xor_sync(0xffffffffu, c.nonexact, o);
        add_tot(c, y);
    }
    __shared__ WarpTot part[32];
    __shared__ ScanTotals t;
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        WarpTot a{0, 0, 0, LLONG_MIN, LLONG_MAX, 0};
        for (uint32_t w = 0; w < (blockDim.x + 31) / 32; ++w) add_tot(a, part[w]);
        t.sum_fixed = a.sum_fixed;
        t.count = a.count;
        t.abs_bound = a.abs_bound;
        t.max_fixed = a.max_fixed;
        t.min_fixed = a.min_fixed;
        t.nonexact = a.nonexact;
        t.bad_chunk = __ldcg(&T->bad_chunk);
    }
    __syncthreads();
    scan_finalize(q, info, T, t, res, frac, fast_ok, exact);
}

}  // namespace
}  // namespace ebi
