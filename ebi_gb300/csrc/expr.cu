// expr.cu -- Aggregation / Expr over several resident columns
// (api/decoder.rs:755-917, decoder/expr.rs:11-135).
//
// An aggregation whose expression is a bare Index runs that column's own
// query (the in-situ sum / min / max).  The others are evaluated on the
// device in three steps:
//   1. every referenced column materializes the rows of the mask (all rows
//      without one) into a compact device array, with the output offset of
//      each of its chunks (the engine's own materialize: the same decode and
//      the same per-chunk counts as the single-column query);
//   2. expr_prepare (one CTA) takes per chunk c and aggregation a the number
//      of values the expression yields, len[a][c] = the shortest of its
//      columns' chunk-c runs (the zip of Expr::compute_chunk), lays out the
//      work items (4,096 values of one chunk each) and the output offsets of
//      array results;
//   3. expr_eval (persistent CTAs over the items) runs each aggregation's
//      program on the values of its item -- straight-line accumulator code
//      compiled on the host, one rounded IEEE operation per Op::doit -- and
//      writes a compensated partial sum and min / max keys per item, or the
//      values themselves for an array result; expr_fold (one CTA per
//      aggregation) combines the items in chunk order.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "column.h"
#include "expr_fused.cuh"
#include "expr_prog.h"
#include "values.cuh"

namespace ebi {
namespace {

constexpr int kExprThreads = 256;
constexpr int kExprPerThread = 16;
constexpr uint32_t kExprItem = kExprThreads * kExprPerThread;  // values per work item
constexpr int kMaxInstr = 2 * EBI_EXPR_MAX_NODES;  // one aggregation's program
constexpr int kPassInstr = 2 * kMaxInstr;          // one pass (shared memory)
constexpr int kMaxStack = 8;    // pushed accumulators
constexpr int kMaxAggs = 8;     // aggregations per evaluation pass
constexpr int kMaxCols = 16;    // distinct columns per evaluation pass

struct ExprPass {
    uint32_t n_aggs, n_cols, n_chunks;
    uint32_t kind[kMaxAggs];       // EBI_AGGR_*
    uint32_t first[kMaxAggs + 1];  // instructions of aggregation a: [first[a], first[a + 1])
    uint32_t cols[kMaxAggs];       // bit j: the aggregation reads column slot j
    const double* vals[kMaxCols];  // compact values of column slot j
    double* out[kMaxAggs];         // array results (EBI_AGGR_NONE)
    uint64_t out_cap[kMaxAggs];
};

// An item's partial (sum hi, sum lo, min key, max key as doubles' bits) or
// an aggregation's result (sum, min, max).
struct alignas(32) Quad {
    double x, y, z, w;
};

// Device scratch of a pass.
struct ExprScratch {
    unsigned long long* off;   // [n_cols][n_chunks + 1]: output offset of each chunk of each column
    unsigned long long* len;   // [n_aggs][n_chunks]
    unsigned long long* aoff;  // [n_aggs][n_chunks]: array output offset
    unsigned long long* item0; // [n_chunks + 1]: first item of each chunk
    unsigned long long* totals;  // [n_aggs + 1]: array lengths, then the item count
    Quad* part;             // [n_aggs][grid]: per CTA sum hi, sum lo, min key, max key
    Quad* res;              // [n_aggs]: sum, min, max, count
    const Instr* prog;
};

__device__ __forceinline__ double op_doit(uint8_t op, double l, double r) {
    switch (op) {
    case I_ADD: return __dadd_rn(l, r);
    case I_SUB: return __dsub_rn(l, r);
    case I_MUL: return __dmul_rn(l, r);
    default: return __ddiv_rn(l, r);
    }
}

// ---- step 2: lengths, items, array offsets ---------------------------------
__global__ void __launch_bounds__(kExprThreads) expr_prepare(ExprPass P, ExprScratch S) {
    __shared__ unsigned long long carry[kMaxAggs + 1];
    __shared__ unsigned long long warp_tot[kMaxAggs + 1][kExprThreads / 32];
    const uint32_t C = P.n_chunks, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x <= kMaxAggs) carry[threadIdx.x] = 0;
    __syncthreads();
    for (uint32_t c0 = 0; c0 < C; c0 += kExprThreads) {
        const uint32_t c = c0 + threadIdx.x;
        unsigned long long mine[kMaxAggs + 1];
        unsigned long long items = 0;
#pragma unroll
        for (int a = 0; a < kMaxAggs; ++a) {
            mine[a] = 0;
            if (a < static_cast<int>(P.n_aggs) && c < C) {
                unsigned long long n = ~0ull;
                for (uint32_t j = 0; j < P.n_cols; ++j) {
                    if (!((P.cols[a] >> j) & 1u)) continue;
                    const unsigned long long* o = S.off + uint64_t(j) * (C + 1);
                    const unsigned long long k = o[c + 1] - o[c];
                    n = k < n ? k : n;
                }
                mine[a] = n == ~0ull ? 0 : n;
                S.len[uint64_t(a) * C + c] = mine[a];
                const unsigned long long it = (mine[a] + kExprItem - 1) / kExprItem;
                items = it > items ? it : items;
            }
        }
        mine[kMaxAggs] = items;
        // exclusive scans across the block, in chunk order
#pragma unroll
        for (int a = 0; a <= kMaxAggs; ++a) {
            unsigned long long x = mine[a];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
                if (static_cast<int>(lane) >= o) x += y;
            }
            if (lane == 31) warp_tot[a][wid] = x;
            mine[a] = x - mine[a];  // exclusive within the warp
        }
        __syncthreads();
#pragma unroll
        for (int a = 0; a <= kMaxAggs; ++a) {
            unsigned long long before = carry[a];
            for (uint32_t w = 0; w < wid; ++w) before += warp_tot[a][w];
            mine[a] += before;
        }
        if (c < C) {
            for (uint32_t a = 0; a < P.n_aggs; ++a) S.aoff[uint64_t(a) * C + c] = mine[a];
            S.item0[c] = mine[kMaxAggs];
        }
        __syncthreads();
        if (threadIdx.x <= kMaxAggs) {
            unsigned long long t = 0;
            for (int w = 0; w < kExprThreads / 32; ++w) t += warp_tot[threadIdx.x][w];
            carry[threadIdx.x] += t;
        }
        __syncthreads();
    }
    if (threadIdx.x < P.n_aggs) S.totals[threadIdx.x] = carry[threadIdx.x];
    if (threadIdx.x == 0) {
        S.totals[P.n_aggs] = carry[kMaxAggs];
        S.item0[C] = carry[kMaxAggs];
    }
}

// ---- step 3: evaluation ---------------------------------------------------
// GB300's FP64 pipe is a small fraction of its integer throughput, so FP64
// work is kept to the expression's own operations: a thread sums its values
// of an item plainly and adds that subtotal to a compensated running sum kept
// across all its items (its error stays far below the 1e-12 bound), min and
// max are ordered keys on the integer pipes, and the CTA reduces once.

// Per-thread running aggregate of one aggregation (shared memory).
struct RunAcc {
    double hi, lo;
    unsigned long long mn, mx;
};

__device__ __forceinline__ void run_init(RunAcc* runs, uint32_t n_aggs) {
    for (uint32_t a = 0; a < n_aggs; ++a)
        runs[a * blockDim.x + threadIdx.x] = RunAcc{0.0, 0.0, kKeyPosInf, kKeyNegInf};
}

// Adds the values v[i] with bit i of ok set.
template <int N>
__device__ __forceinline__ void run_add(RunAcc& r, const double (&v)[N], uint32_t ok, uint32_t kind) {
    if (!ok) return;
    if (kind == EBI_AGGR_SUM) {
        double s = 0.0;
        bool any = false;
#pragma unroll
        for (int i = 0; i < N; ++i)
            if ((ok >> i) & 1u) { s = any ? __dadd_rn(s, v[i]) : v[i]; any = true; }
        neumaier_add(r.hi, r.lo, s);
        return;
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
        const uint64_t b = static_cast<uint64_t>(__double_as_longlong(v[i]));
        if (((ok >> i) & 1u) && !is_nan_bits(b)) {
            const unsigned long long k = order_key(b);
            r.mn = k < r.mn ? k : r.mn;
            r.mx = k > r.mx ? k : r.mx;
        }
    }
}

// The CTA's partial of every scalar aggregation: part[a * gridDim.x + blockIdx.x].
__device__ void cta_partials(const ExprPass& P, const ExprScratch& S, const RunAcc* runs) {
    __shared__ double red_h[32], red_l[32];
    __shared__ unsigned long long red_mn[32], red_mx[32];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x / 32;
    for (uint32_t a = 0; a < P.n_aggs; ++a) {
        if (P.kind[a] == EBI_AGGR_NONE) continue;
        const RunAcc r = runs[a * blockDim.x + threadIdx.x];
        double hi = r.hi, lo = r.lo;
        unsigned long long mn = r.mn, mx = r.mx;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double oh = __shfl_down_sync(0xffffffffu, hi, o), ol = __shfl_down_sync(0xffffffffu, lo, o);
            if ((lane & (2 * o - 1)) == 0) dd_add(hi, lo, oh, ol);
        }
        mn = warp_min_u64(mn);
        mx = warp_max_u64(mx);
        if (lane == 0) { red_h[wid] = hi; red_l[wid] = lo; red_mn[wid] = mn; red_mx[wid] = mx; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double th = 0.0, tl = 0.0;
            unsigned long long tmn = kKeyPosInf, tmx = kKeyNegInf;
            for (uint32_t w = 0; w < nw; ++w) {
                dd_add(th, tl, red_h[w], red_l[w]);
                tmn = red_mn[w] < tmn ? red_mn[w] : tmn;
                tmx = red_mx[w] > tmx ? red_mx[w] : tmx;
            }
            Quad q;
            q.x = th;
            q.y = tl;
            q.z = __longlong_as_double(static_cast<long long>(tmn));
            q.w = __longlong_as_double(static_cast<long long>(tmx));
            S.part[a * uint64_t(gridDim.x) + blockIdx.x] = q;
        }
        __syncthreads();
    }
}

__device__ __forceinline__ double operand(uint8_t src, uint16_t col, double lit, double acc_e,
                                          const double (&st)[kMaxStack][kExprPerThread], int sp, int e,
                                          const double* const* base, uint64_t k, bool ok) {
    switch (src) {
    case S_ACC: return acc_e;
    case S_POP: return st[sp - 1][e];
    case S_LIT: return lit;
    default: return ok ? __ldg(base[col] + k) : 0.0;
    }
}

__global__ void __launch_bounds__(kExprThreads) expr_eval(ExprPass P, ExprScratch S) {
    extern __shared__ RunAcc runs[];  // [n_aggs][kExprThreads]
    __shared__ Instr prog[kPassInstr];
    __shared__ const double* base[kMaxCols];
    __shared__ uint32_t s_c;
    const uint32_t n_instr = P.first[P.n_aggs];
    for (uint32_t i = threadIdx.x; i < n_instr; i += kExprThreads) prog[i] = S.prog[i];
    run_init(runs, P.n_aggs);
    const uint32_t C = P.n_chunks;
    const unsigned long long n_items = S.totals[P.n_aggs];
    for (unsigned long long item = blockIdx.x; item < n_items; item += gridDim.x) {
        __syncthreads();  // the previous item's shared values are consumed
        if (threadIdx.x == 0) {
            // the chunk of the item: the last c with item0[c] <= item
            uint32_t lo = 0, hi = C;
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) / 2;
                if (S.item0[mid] <= item) lo = mid; else hi = mid;
            }
            s_c = lo;
        }
        __syncthreads();
        // column values of the chunk start at the column's chunk offset
        if (threadIdx.x < P.n_cols) base[threadIdx.x] = P.vals[threadIdx.x] + S.off[uint64_t(threadIdx.x) * (C + 1) + s_c];
        __syncthreads();
        const uint32_t c = s_c;
        const uint64_t k0 = (item - S.item0[c]) * kExprItem;
        for (uint32_t a = 0; a < P.n_aggs; ++a) {
            const uint64_t len = S.len[uint64_t(a) * C + c];
            double acc[kExprPerThread];
            double st[kMaxStack][kExprPerThread];
            int sp = 0;
#pragma unroll
            for (int e = 0; e < kExprPerThread; ++e) acc[e] = 0.0;
            for (uint32_t i = P.first[a]; i < P.first[a + 1]; ++i) {
                const Instr I = prog[i];
                if (I.op == I_PUSH) {
#pragma unroll
                    for (int e = 0; e < kExprPerThread; ++e) st[sp][e] = acc[e];
                    ++sp;
                    continue;
                }
#pragma unroll
                for (int e = 0; e < kExprPerThread; ++e) {
                    const uint64_t k = k0 + uint64_t(e) * kExprThreads + threadIdx.x;
                    const bool ok = k < len;
                    const double x = operand(I.a, I.ca, I.la, acc[e], st, sp, e, base, k, ok);
                    if (I.op == I_LOAD) { acc[e] = x; continue; }
                    const double y = operand(I.b, I.cb, I.lb, acc[e], st, sp, e, base, k, ok);
                    acc[e] = op_doit(I.op, x, y);
                }
                if (I.a == S_POP || I.b == S_POP) --sp;
            }
            uint32_t ok = 0;
#pragma unroll
            for (int e = 0; e < kExprPerThread; ++e)
                if (k0 + uint64_t(e) * kExprThreads + threadIdx.x < len) ok |= 1u << e;
            const uint32_t kind = P.kind[a];
            if (kind == EBI_AGGR_NONE) {
                double* out = P.out[a];
                const uint64_t o = S.aoff[uint64_t(a) * C + c], cap = P.out_cap[a];
#pragma unroll
                for (int e = 0; e < kExprPerThread; ++e) {
                    const uint64_t k = k0 + uint64_t(e) * kExprThreads + threadIdx.x;
                    if (((ok >> e) & 1u) && o + k < cap) out[o + k] = acc[e];
                }
                continue;
            }
            run_add(runs[a * kExprThreads + threadIdx.x], acc, ok, kind);
        }
    }
    __syncthreads();
    cta_partials(P, S, runs);
}

// One CTA per aggregation: the CTAs' partials in CTA order.
__global__ void __launch_bounds__(kExprThreads) expr_fold(ExprPass P, ExprScratch S, uint32_t n_parts) {
    __shared__ double sh_h[kExprThreads / 32], sh_l[kExprThreads / 32];
    __shared__ unsigned long long sh_mn[kExprThreads / 32], sh_mx[kExprThreads / 32];
    const uint32_t a = blockIdx.x;
    if (a >= P.n_aggs || P.kind[a] == EBI_AGGR_NONE) return;
    const Quad* part = S.part + uint64_t(a) * n_parts;
    double hi = 0.0, lo = 0.0;
    unsigned long long mn = kKeyPosInf, mx = kKeyNegInf;
    for (uint32_t i = threadIdx.x; i < n_parts; i += kExprThreads) {
        const Quad p = part[i];
        dd_add(hi, lo, p.x, p.y);
        const unsigned long long pm = static_cast<unsigned long long>(__double_as_longlong(p.z));
        const unsigned long long px = static_cast<unsigned long long>(__double_as_longlong(p.w));
        mn = pm < mn ? pm : mn;
        mx = px > mx ? px : mx;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double oh = __shfl_down_sync(0xffffffffu, hi, o), ol = __shfl_down_sync(0xffffffffu, lo, o);
        if ((lane & (2 * o - 1)) == 0) dd_add(hi, lo, oh, ol);
    }
    mn = warp_min_u64(mn);
    mx = warp_max_u64(mx);
    if (lane == 0) { sh_h[wid] = hi; sh_l[wid] = lo; sh_mn[wid] = mn; sh_mx[wid] = mx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double th = 0.0, tl = 0.0;
        unsigned long long tmn = kKeyPosInf, tmx = kKeyNegInf;
        for (int w = 0; w < kExprThreads / 32; ++w) {
            dd_add(th, tl, sh_h[w], sh_l[w]);
            tmn = sh_mn[w] < tmn ? sh_mn[w] : tmn;
            tmx = sh_mx[w] > tmx ? sh_mx[w] : tmx;
        }
        Quad r;
        r.x = neumaier_value(th, tl);
        r.y = __longlong_as_double(static_cast<long long>(key_bits(tmn)));
        r.z = __longlong_as_double(static_cast<long long>(key_bits(tmx)));
        r.w = 0.0;
        S.res[a] = r;
    }
}

// ---- fused path: BUFF columns with aligned chunks ---------------------------
// When every column of a pass is BUFF, read at full precision, and its first
// C chunks cover the same rows as the other columns', element k of a chunk is
// the same row in every column: the zip is row-wise and the values need not
// be materialized.  The walk over the planes is expr_fused.cuh's; the
// program objects below interpret the pass's programs, on the fixed-point
// integers (exact programs) or on the f64 values.  Exact passes may instead
// run the same walk compiled at run time with the programs written out
// (expr_jit.cu).
constexpr int kFuseThreads = ebi_fx::kThreads;
constexpr int kFuseWarps = ebi_fx::kWarps;
constexpr int kFuseRows = ebi_fx::kRows;
constexpr uint32_t kFuseUnit = ebi_fx::kUnit;
constexpr int kFuseStride = ebi_fx::kStride;
constexpr int kFuseCols = ebi_fx::kCols;
constexpr int kFuseStack = 2;  // accumulators a fused program may push

static_assert(sizeof(ebi_fx::ChunkInfo) == sizeof(BuffChunkInfo) &&
                  offsetof(ebi_fx::ChunkInfo, planes) == offsetof(BuffChunkInfo, planes) &&
                  offsetof(ebi_fx::ChunkInfo, tail) == offsetof(BuffChunkInfo, tail) &&
                  offsetof(ebi_fx::ChunkInfo, base) == offsetof(BuffChunkInfo, base) &&
                  offsetof(ebi_fx::ChunkInfo, bits) == offsetof(BuffChunkInfo, bits) &&
                  offsetof(ebi_fx::ChunkInfo, frac) == offsetof(BuffChunkInfo, frac) &&
                  offsetof(ebi_fx::ChunkInfo, status) == offsetof(BuffChunkInfo, status) &&
                  offsetof(ebi_fx::ChunkInfo, stride) == offsetof(BuffChunkInfo, stride),
              "ebi_fx::ChunkInfo is BuffChunkInfo's layout twin");
static_assert(sizeof(ebi_fx::Chunk) == sizeof(ChunkDesc) &&
                  offsetof(ebi_fx::Chunk, row_off) == offsetof(ChunkDesc, row_off) &&
                  offsetof(ebi_fx::Chunk, n_rows) == offsetof(ChunkDesc, n_rows),
              "ebi_fx::Chunk is ChunkDesc's layout twin");
static_assert(ebi_fx::kSum == EBI_AGGR_SUM && ebi_fx::kMin == EBI_AGGR_MIN && ebi_fx::kMax == EBI_AGGR_MAX,
              "aggregation kinds");
static_assert(sizeof(ebi_fx::Acc) == sizeof(Quad) && sizeof(RunAcc) == sizeof(ebi_fx::Acc), "partials");

// (base + delta) / 2^frac exactly as the BUFF materialize kernel computes it
// (int64 -> f64, then * 2^-frac or / 2^frac); when the integer is below 2^53
// and the result normal the conversion is exact and its bits are built on
// the integer pipes.  inv_ok: frac <= 1022 (the materialize kernel's inv != 0).
__device__ __forceinline__ double fuse_value(long long fixed, uint32_t frac, bool inv_ok, double inv, double scale) {
    const unsigned long long u = fixed < 0 ? 0ull - static_cast<unsigned long long>(fixed)
                                           : static_cast<unsigned long long>(fixed);
    if (u == 0) return 0.0;
    const int msb = 63 - __clzll(static_cast<long long>(u));
    const int e = msb - static_cast<int>(frac) + 1023;
    if (msb <= 52 && e >= 1 && inv_ok) {
        const unsigned long long bits = (fixed < 0 ? 0x8000000000000000ull : 0ull) |
                                        (static_cast<unsigned long long>(e) << 52) |
                                        ((u << (52 - msb)) & 0x000fffffffffffffull);
        return __longlong_as_double(static_cast<long long>(bits));
    }
    return inv_ok ? static_cast<double>(fixed) * inv : static_cast<double>(fixed) / scale;
}

// The program interpreter of a fused pass.  kExact: the program runs on the
// fixed-point integers (each value is fixed * 2^-frac; the host proved every
// intermediate below 2^53, where each IEEE operation is exact and equals the
// integer one); else on the f64 values.  Running aggregates live in shared
// memory: ebi_fx::Acc (exact) or RunAcc (f64) per thread and aggregation.
template <bool kExact>
struct FuseInterp {
    static constexpr bool kPacked = true;
    const Instr* __restrict__ prog;  // every lane reads the same instruction: one L1 line
    const uint32_t* first;           // shared: [n_aggs + 1]
    const uint32_t* kind;            // shared: [n_aggs]
    void* runs;                      // shared: [n_aggs][kFuseThreads]
    uint32_t n;

    __device__ uint32_t n_aggs() const { return n; }
    __device__ void begin() {
        for (uint32_t a = 0; a < n; ++a) {
            if (kExact) static_cast<ebi_fx::Acc*>(runs)[a * kFuseThreads + threadIdx.x] = ebi_fx::acc_rest();
            else static_cast<RunAcc*>(runs)[a * kFuseThreads + threadIdx.x] = RunAcc{0.0, 0.0, kKeyPosInf, kKeyNegInf};
        }
    }
    __device__ long long pack(const ebi_fx::ChunkInfo& ci, long long fixed) const {
        if (kExact) return fixed;
        const bool inv_ok = ci.frac <= 1022;
        const double scale = ci.frac <= 1023 ? __longlong_as_double(static_cast<long long>(uint64_t(1023 + ci.frac) << 52))
                                             : __longlong_as_double(0x7ff0000000000000ll);
        const double inv = inv_ok ? __longlong_as_double(static_cast<long long>(uint64_t(1023 - ci.frac) << 52)) : 0.0;
        return __double_as_longlong(fuse_value(fixed, ci.frac, inv_ok, inv, scale));
    }
    __device__ ebi_fx::Acc result(uint32_t a) const { return static_cast<ebi_fx::Acc*>(runs)[a * kFuseThreads + threadIdx.x]; }

    __device__ void unit(const long long* islot, uint32_t lane, uint32_t ok) {
        const double* wslot = reinterpret_cast<const double*>(islot);
        for (uint32_t a = 0; a < n; ++a) {
            using V = typename std::conditional<kExact, long long, double>::type;
            // accumulator and a two-deep stack, all in registers: the operand
            // kinds are the same for every lane, so each instruction branches
            // once and then runs over the lane's values
            V acc[kFuseRows], st0[kFuseRows], st1[kFuseRows];
            int sp = 0;
#pragma unroll
            for (int k = 0; k < kFuseRows; ++k) acc[k] = st0[k] = st1[k] = 0;
            for (uint32_t q = first[a]; q < first[a + 1]; ++q) {
                const uint8_t op = prog[q].op, src_a = prog[q].a, src_b = prog[q].b;
                if (op == I_PUSH) {
                    if (sp == 0) {
#pragma unroll
                        for (int k = 0; k < kFuseRows; ++k) st0[k] = acc[k];
                    } else {
#pragma unroll
                        for (int k = 0; k < kFuseRows; ++k) st1[k] = acc[k];
                    }
                    ++sp;
                    continue;
                }
                V x[kFuseRows], y[kFuseRows];
                auto fetch = [&](uint8_t src, uint16_t col, double lit_bits, uint32_t sh, V (&out)[kFuseRows]) {
                    if (src == S_COL) {
                        // slots past the packed count hold stale values of the warp's own region:
                        // read anyway (in bounds), their rows are dropped when aggregating
#pragma unroll
                        for (int k = 0; k < kFuseRows; ++k) {
                            const uint32_t at = col * kFuseStride + ebi_fx::pad(lane + uint32_t(k) * 32);
                            if constexpr (kExact) out[k] = islot[at];
                            else out[k] = wslot[at];
                        }
                    } else if (src == S_LIT) {
                        V l;
                        if constexpr (kExact) l = __double_as_longlong(lit_bits);
                        else l = lit_bits;
#pragma unroll
                        for (int k = 0; k < kFuseRows; ++k) out[k] = l;
                    } else if (src == S_ACC) {
#pragma unroll
                        for (int k = 0; k < kFuseRows; ++k) out[k] = acc[k];
                    } else if (sp == 1) {
#pragma unroll
                        for (int k = 0; k < kFuseRows; ++k) out[k] = st0[k];
                    } else {
#pragma unroll
                        for (int k = 0; k < kFuseRows; ++k) out[k] = st1[k];
                    }
                    if constexpr (kExact) {
                        if (sh) {  // the same for every lane
#pragma unroll
                            for (int k = 0; k < kFuseRows; ++k)
                                out[k] = static_cast<long long>(static_cast<unsigned long long>(out[k]) << sh);
                        }
                    }
                };
                fetch(src_a, prog[q].ca, prog[q].la, prog[q].sa, x);
                if (op == I_LOAD) {
#pragma unroll
                    for (int k = 0; k < kFuseRows; ++k) acc[k] = x[k];
                    continue;
                }
                fetch(src_b, prog[q].cb, prog[q].lb, prog[q].sb, y);
                if (src_a == S_POP || src_b == S_POP) --sp;
                if constexpr (kExact) {
                    // wrapping (unsigned) arithmetic: exact for the rows aggregated, whose
                    // intermediates stay below 2^53; defined for the stale ones dropped later
                    using U = unsigned long long;
                    if (op == I_ADD) {
#pragma unroll
                        for (int k = 0; k < kFuseRows; ++k) acc[k] = static_cast<long long>(U(x[k]) + U(y[k]));
                    } else if (op == I_SUB) {
#pragma unroll
                        for (int k = 0; k < kFuseRows; ++k) acc[k] = static_cast<long long>(U(x[k]) - U(y[k]));
                    } else {
#pragma unroll
                        for (int k = 0; k < kFuseRows; ++k) acc[k] = static_cast<long long>(U(x[k]) * U(y[k]));
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < kFuseRows; ++k)
                        if ((ok >> k) & 1u) acc[k] = op_doit(op, x[k], y[k]);
                }
            }
            if constexpr (kExact) {
                ebi_fx::acc_add(static_cast<ebi_fx::Acc*>(runs)[a * kFuseThreads + threadIdx.x], kind[a], acc, ok);
            } else {
                run_add(static_cast<RunAcc*>(runs)[a * kFuseThreads + threadIdx.x], acc, ok, kind[a]);
            }
        }
    }
};

// Dynamic shared memory of an interpreted fused pass: the packed values, then
// the running aggregates.
__host__ __device__ constexpr size_t fuse_smem(uint32_t n_cols, uint32_t n_aggs) {
    return size_t(kFuseWarps) * n_cols * kFuseStride * sizeof(double) + size_t(n_aggs) * kFuseThreads * sizeof(RunAcc);
}

template <bool kExact>
__global__ void __launch_bounds__(kFuseThreads, 3) expr_buff_fused(ExprPass P, ExprScratch S, ebi_fx::Params F) {
    extern __shared__ double dyn[];  // [warp][n_cols][kFuseStride] packed values, then the running aggregates
    __shared__ uint32_t s_kind[kMaxAggs], s_first[kMaxAggs + 1];
    if (threadIdx.x < kMaxAggs) s_kind[threadIdx.x] = P.kind[threadIdx.x];
    if (threadIdx.x <= kMaxAggs) s_first[threadIdx.x] = P.first[threadIdx.x];
    FuseInterp<kExact> I{S.prog, s_first, s_kind, dyn + kFuseWarps * P.n_cols * kFuseStride, P.n_aggs};
    ebi_fx::fused_walk(F, I, reinterpret_cast<long long*>(dyn));  // synchronises after s_kind, s_first
    if constexpr (kExact) ebi_fx::fused_finish_exact(F, I);
    else cta_partials(P, S, static_cast<RunAcc*>(I.runs));
}

// Exact programs: the CTAs' 128-bit sums and keys, added in CTA order (res
// bits: sum lo, sum hi, min key, max key; the host scales them).
__global__ void __launch_bounds__(kExprThreads) expr_fold_exact(ExprPass P, ExprScratch S, uint32_t n_parts) {
    __shared__ unsigned long long r_lo[kExprThreads / 32], r_hi[kExprThreads / 32], r_mn[kExprThreads / 32],
        r_mx[kExprThreads / 32];
    const uint32_t a = blockIdx.x;
    if (a >= P.n_aggs) return;
    const Quad* part = S.part + uint64_t(a) * n_parts;
    unsigned long long lo = 0, hi = 0, mn = ~0ull, mx = 0;
    for (uint32_t i = threadIdx.x; i < n_parts; i += kExprThreads) {
        const Quad p = part[i];
        ebi_fx::add128(lo, hi, static_cast<unsigned long long>(__double_as_longlong(p.x)),
               static_cast<unsigned long long>(__double_as_longlong(p.y)));
        const unsigned long long pm = static_cast<unsigned long long>(__double_as_longlong(p.z));
        const unsigned long long px = static_cast<unsigned long long>(__double_as_longlong(p.w));
        mn = pm < mn ? pm : mn;
        mx = px > mx ? px : mx;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ebi_fx::add128(lo, hi, __shfl_xor_sync(0xffffffffu, lo, o), __shfl_xor_sync(0xffffffffu, hi, o));
        const unsigned long long omn = __shfl_xor_sync(0xffffffffu, mn, o), omx = __shfl_xor_sync(0xffffffffu, mx, o);
        mn = omn < mn ? omn : mn;
        mx = omx > mx ? omx : mx;
    }
    if (lane == 0) { r_lo[wid] = lo; r_hi[wid] = hi; r_mn[wid] = mn; r_mx[wid] = mx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long tl = 0, th = 0, tmn = ~0ull, tmx = 0;
        for (int w = 0; w < kExprThreads / 32; ++w) {
            ebi_fx::add128(tl, th, r_lo[w], r_hi[w]);
            tmn = r_mn[w] < tmn ? r_mn[w] : tmn;
            tmx = r_mx[w] > tmx ? r_mx[w] : tmx;
        }
        Quad r;
        r.x = __longlong_as_double(static_cast<long long>(tl));
        r.y = __longlong_as_double(static_cast<long long>(th));
        r.z = __longlong_as_double(static_cast<long long>(tmn));
        r.w = __longlong_as_double(static_cast<long long>(tmx));
        S.res[a] = r;
    }
}

// Output offsets of a column's chunks 0..n: its tile offsets at each chunk's first tile.
__global__ void gather_chunk_offsets(const unsigned long long* tile_offsets, const uint32_t* first_tile, uint32_t n,
                                     unsigned long long* off) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x)
        off[i] = tile_offsets[first_tile[i]];
}

// ---- host -------------------------------------------------------------------
int fail(int code, const std::string& msg) {
    set_last_error(msg);
    return code;
}
int cuda_fail(cudaError_t e, const char* what) {
    return fail(EBI_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(expr)                                              \
    do {                                                      \
        cudaError_t _e = (expr);                              \
        if (_e != cudaSuccess) return cuda_fail(_e, #expr);   \
    } while (0)

struct Node {
    int32_t kind;
    uint32_t index;
    double lit;
    int lhs, rhs;
};

// Postfix -> tree; the root, or -1 for a malformed program.
int build_tree(const ebi_aggregation& g, uint32_t n_cols, std::vector<Node>& t) {
    if (!g.nodes || g.n_nodes == 0 || g.n_nodes > EBI_EXPR_MAX_NODES) return -1;
    t.resize(g.n_nodes);
    std::vector<int> st;
    for (uint32_t i = 0; i < g.n_nodes; ++i) {
        const ebi_expr_node& n = g.nodes[i];
        t[i] = Node{n.kind, n.index, n.literal, -1, -1};
        if (n.kind == EBI_EXPR_INDEX || n.kind == EBI_EXPR_LITERAL) {
            if (n.kind == EBI_EXPR_INDEX && n.index >= n_cols) return -1;
            st.push_back(static_cast<int>(i));
            continue;
        }
        if (n.kind < EBI_EXPR_ADD || n.kind > EBI_EXPR_DIV || st.size() < 2) return -1;
        t[i].rhs = st.back(); st.pop_back();
        t[i].lhs = st.back(); st.pop_back();
        st.push_back(static_cast<int>(i));
    }
    return st.size() == 1 ? st[0] : -1;
}

// Accumulator code of one expression tree: leaves are operands of the
// operator above them, a non-leaf right operand pushes the left result.
// S_COL operands carry the column index (slots are assigned per pass).
struct Compiler {
    const std::vector<Node>& t;
    std::vector<Instr> out;
    int depth = 0, max_depth = 0;
    bool precondition = false;

    static bool is_leaf(const Node& n) { return n.kind == EBI_EXPR_INDEX || n.kind == EBI_EXPR_LITERAL; }
    static void leaf(const Node& n, uint8_t& src, uint16_t& col, double& lit) {
        if (n.kind == EBI_EXPR_LITERAL) { src = S_LIT; lit = n.lit; return; }
        src = S_COL;
        col = static_cast<uint16_t>(n.index);
    }
    // Leaves acc = value of node k.
    void gen(int k) {
        const Node& n = t[k];
        Instr I{};
        if (n.kind == EBI_EXPR_LITERAL) { precondition = true; return; }  // a Literal has no chunk values
        if (n.kind == EBI_EXPR_INDEX) {
            I.op = I_LOAD;
            leaf(n, I.a, I.ca, I.la);
            out.push_back(I);
            return;
        }
        const Node &L = t[n.lhs], &R = t[n.rhs];
        I.op = static_cast<uint8_t>(I_ADD + (n.kind - EBI_EXPR_ADD));
        if (L.kind == EBI_EXPR_LITERAL && R.kind == EBI_EXPR_LITERAL) { precondition = true; return; }
        if (is_leaf(L) && is_leaf(R)) {
            leaf(L, I.a, I.ca, I.la);
            leaf(R, I.b, I.cb, I.lb);
        } else if (is_leaf(R)) {
            gen(n.lhs);
            I.a = S_ACC;
            leaf(R, I.b, I.cb, I.lb);
        } else if (is_leaf(L)) {
            gen(n.rhs);
            leaf(L, I.a, I.ca, I.la);
            I.b = S_ACC;
        } else {
            gen(n.lhs);
            Instr push{};
            push.op = I_PUSH;
            out.push_back(push);
            if (++depth > max_depth) max_depth = depth;
            gen(n.rhs);
            --depth;
            I.a = S_POP;
            I.b = S_ACC;
        }
        out.push_back(I);
    }
};

// The columns an instruction list reads.
std::vector<uint32_t> program_columns(const std::vector<Instr>& prog) {
    std::vector<uint32_t> c;
    for (const Instr& I : prog) {
        if (I.a == S_COL) c.push_back(I.ca);
        if (I.b == S_COL) c.push_back(I.cb);
    }
    std::sort(c.begin(), c.end());
    c.erase(std::unique(c.begin(), c.end()), c.end());
    return c;
}

int aggregate_index(ebi_column* col, ebi_aggregation& g, const uint64_t* d_mask, void* stream) {
    switch (g.kind) {
    case EBI_AGGR_SUM: return ebi_sum(col, d_mask, -1, &g.scalar, stream);
    case EBI_AGGR_MIN: return ebi_min(col, d_mask, -1, &g.scalar, stream);
    case EBI_AGGR_MAX: return ebi_max(col, d_mask, -1, &g.scalar, stream);
    default: return fail(EBI_E_UNSUPPORTED, "Aggregation of kind None over a bare Index (todo!() in the reference)");
    }
}

// Materializes column col under d_mask into a fresh device array (*vals, *n)
// and writes the output offsets of its chunks 0..C to d_off (C + 1 values).
int materialize_column(ebi_column* col, const uint64_t* d_mask, uint32_t C, unsigned long long* d_off,
                       uint32_t* d_first_tile, double** vals, uint64_t* n, cudaStream_t s) {
    uint64_t cap = std::max<uint64_t>(col->n_records, 1);
    for (int attempt = 0; attempt < 2; ++attempt) {
        double* v = nullptr;
        CK(cudaMallocAsync(reinterpret_cast<void**>(&v), cap * sizeof(double), s));
        uint64_t got = 0;
        const int st = ebi_materialize(col, d_mask, -1, v, cap, &got, s);
        if (st == EBI_E_INVALID && got > cap && attempt == 0) {  // chunks decoded more values than their row counts
            cudaFreeAsync(v, s);
            cap = got;
            continue;
        }
        if (st) { cudaFreeAsync(v, s); return st; }
        *vals = v;
        *n = got;
        break;
    }
    if (col->scheme == EBI_BUFF && !d_mask) {
        // BUFF without a mask writes chunk c's rows at its first row
        std::vector<unsigned long long> off(C + 1);
        for (uint32_t c = 0; c < C; ++c) off[c] = col->chunks[c].row_off;
        off[C] = C < col->n_chunks ? col->chunks[C].row_off : col->n_records;
        CK(cudaMemcpyAsync(d_off, off.data(), off.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));  // off is host memory
        return EBI_OK;
    }
    std::vector<uint32_t> ft(col->tiles.first_tile.begin(), col->tiles.first_tile.begin() + C + 1);
    CK(cudaMemcpyAsync(d_first_tile, ft.data(), ft.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    gather_chunk_offsets<<<(C + 256) / 256, 256, 0, s>>>(col->d_tile_offsets, d_first_tile, C, d_off);
    count_launch();
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));  // the next query on this column reuses its tile offsets; ft is host memory
    return EBI_OK;
}

// ---- exact BUFF programs ------------------------------------------------------
// Every value of a BUFF column is fixed * 2^-frac.  A program of +, -, * over
// such values and dyadic literals runs on the integers when every
// intermediate stays below 2^53 at its scale: each IEEE operation then
// returns its exact result, which the integer operation also gives.
struct Scale {
    int f;     // value = n * 2^-f
    int bits;  // |n| < 2^bits
};

int bitlen(unsigned long long v) { return v ? 64 - __builtin_clzll(v) : 0; }

// x = n * 2^-f with |n| < 2^53 and the least f >= 0.
bool dyadic(double x, long long* n, Scale* sc) {
    if (x == 0.0) { *n = 0; *sc = Scale{0, 0}; return true; }
    if (!std::isfinite(x)) return false;
    int e = 0;
    const double m = std::frexp(std::fabs(x), &e);  // |x| = m * 2^e, m in [0.5, 1)
    unsigned long long M = static_cast<unsigned long long>(std::ldexp(m, 53));
    int k = e - 53;
    while (!(M & 1ull)) { M >>= 1; ++k; }
    if (k >= 0) {
        if (bitlen(M) + k > 53) return false;
        M <<= k;
        k = 0;
    }
    *n = x < 0 ? -static_cast<long long>(M) : static_cast<long long>(M);
    *sc = Scale{-k, bitlen(M)};
    return true;
}

// Rewrites the pass's program for integer evaluation (shifts, integer
// literals) and gives each aggregation's result scale; false when a step is
// not provably exact.
bool exact_program(std::vector<Instr>& prog, const ExprPass& P, const std::vector<Scale>& col, std::vector<int>& f_out) {
    f_out.assign(P.n_aggs, 0);
    for (uint32_t a = 0; a < P.n_aggs; ++a) {
        Scale acc{0, 0};
        std::vector<Scale> stack;
        for (uint32_t q = P.first[a]; q < P.first[a + 1]; ++q) {
            Instr& I = prog[q];
            if (I.op == I_PUSH) { stack.push_back(acc); continue; }
            if (I.op == I_DIV) return false;
            auto operand = [&](uint8_t src, uint16_t c, double& lit, Scale& sc) -> bool {
                if (src == S_ACC) { sc = acc; return true; }
                if (src == S_POP) { sc = stack.back(); return true; }
                if (src == S_COL) { sc = col[c]; return true; }
                long long n = 0;
                if (!dyadic(lit, &n, &sc)) return false;
                std::memcpy(&lit, &n, sizeof n);
                return true;
            };
            Scale x{}, y{};
            if (!operand(I.a, I.ca, I.la, x)) return false;
            I.sa = I.sb = 0;
            if (I.op == I_LOAD) {
                acc = x;
            } else {
                if (!operand(I.b, I.cb, I.lb, y)) return false;
                if (I.a == S_POP || I.b == S_POP) stack.pop_back();
                if (I.op == I_MUL) {
                    acc = Scale{x.f + y.f, x.bits + y.bits};
                } else {
                    const int f = std::max(x.f, y.f);
                    I.sa = static_cast<uint8_t>(f - x.f);
                    I.sb = static_cast<uint8_t>(f - y.f);
                    if (x.bits + I.sa > 62 || y.bits + I.sb > 62) return false;
                    acc = Scale{f, std::max(x.bits + I.sa, y.bits + I.sb) + 1};
                }
            }
            if (acc.bits > 53 || acc.f > 1000) return false;
        }
        f_out[a] = acc.f;
    }
    return true;
}

// n * 2^-f for a two's complement 128-bit n, rounded to nearest even once.
double scaled_i128(unsigned long long lo, unsigned long long hi, int f) {
    const __int128 v = static_cast<__int128>((static_cast<unsigned __int128>(hi) << 64) | lo);
    const bool neg = v < 0;
    unsigned __int128 m = neg ? -static_cast<unsigned __int128>(v) : static_cast<unsigned __int128>(v);
    if (m == 0) return 0.0;
    const unsigned long long mh = static_cast<unsigned long long>(m >> 64);
    const int p = mh ? 127 - __builtin_clzll(mh) : 63 - __builtin_clzll(static_cast<unsigned long long>(m));
    double d;
    if (p <= 52) {
        d = static_cast<double>(static_cast<unsigned long long>(m));
    } else {
        int sh = p - 52;
        unsigned __int128 top = m >> sh;
        const unsigned __int128 rem = m & ((static_cast<unsigned __int128>(1) << sh) - 1);
        const unsigned __int128 half = static_cast<unsigned __int128>(1) << (sh - 1);
        if (rem > half || (rem == half && (top & 1))) {
            ++top;
            if (top >> 53) { top >>= 1; ++sh; }
        }
        d = std::ldexp(static_cast<double>(static_cast<unsigned long long>(top)), sh);
    }
    d = std::ldexp(d, -f);
    return neg ? -d : d;
}

// The fused path applies: scalar results only, programs at most kFuseStack
// deep, at most kFuseCols BUFF columns at full precision whose first C
// chunks cover the same rows.
bool fusable(ebi_column* const* cols, const std::vector<uint32_t>& slot_cols, const ebi_aggregation* aggs,
             const std::vector<uint32_t>& idx, const std::vector<std::vector<Instr>>& progs, uint32_t C) {
    if (slot_cols.empty() || slot_cols.size() > static_cast<size_t>(kFuseCols)) return false;
    for (uint32_t a : idx)
        if (aggs[a].kind == EBI_AGGR_NONE) return false;
    for (uint32_t a : idx) {  // the fused kernels keep a two-deep stack in registers
        int depth = 0;
        for (const Instr& I : progs[a]) {
            if (I.op == I_PUSH && ++depth > kFuseStack) return false;
            if (I.a == S_POP || I.b == S_POP) --depth;
        }
    }
    const ebi_column* r = cols[slot_cols[0]];
    for (uint32_t j : slot_cols) {
        const ebi_column* c = cols[j];
        if (c->scheme != EBI_BUFF || c->precision >= 0 || !c->d_buff) return false;
        for (uint32_t k = 0; k < C; ++k)
            if (c->chunks[k].n_rows != r->chunks[k].n_rows || c->chunks[k].row_off != r->chunks[k].row_off) return false;
    }
    return true;
}

// Runs a fusable pass.  *fell_back: a chunk is unreadable, the caller runs
// the general path (which reports the chunk's error in chunk order).
int run_fused(ebi_column* const* cols, ebi_aggregation* aggs, const std::vector<uint32_t>& idx, const ExprPass& P,
              const std::vector<Instr>& prog, const std::vector<uint32_t>& slot_cols, const uint64_t* d_mask,
              uint32_t C, cudaStream_t s, bool* fell_back) {
    const ebi_column* r = cols[slot_cols[0]];
    std::vector<uint32_t> unit0(C + 1);
    uint64_t units = 0;
    for (uint32_t c = 0; c < C; ++c) {
        unit0[c] = static_cast<uint32_t>(units);
        units += (r->chunks[c].n_rows + kFuseUnit - 1) / kFuseUnit;
    }
    if (units > 0xffffffffull) return fail(EBI_E_INVALID, "too many rows");
    unit0[C] = static_cast<uint32_t>(units);
    const uint32_t n_units = static_cast<uint32_t>(units);
    // integer evaluation when every column has one scale and the program is provably exact
    std::vector<Instr> iprog = prog;
    std::vector<int> f_out;
    std::vector<Scale> col_scale;
    bool exact = true;
    for (uint32_t j : slot_cols) {
        const ebi_column* c = cols[j];
        if (!c->buff_same_frac || c->buff_fixed_bits > 53) exact = false;
        col_scale.push_back(Scale{static_cast<int>(c->buff_frac), static_cast<int>(c->buff_fixed_bits)});
    }
    exact = exact && exact_program(iprog, P, col_scale, f_out);
    // exact passes: the walk compiled with these programs written out, when
    // the run-time compiler is there; else (and for f64 programs) interpreted
    cudaKernel_t jit = nullptr;
    bool narrow = true;  // the compiled walk decodes in 32-bit arithmetic
    for (uint32_t j : slot_cols) narrow = narrow && cols[j]->buff_max_bits <= 32;
    if (exact && narrow) {
        std::string why;
        bool required = false;
        uint32_t widths[kFuseCols] = {};
        for (uint32_t j = 0; j < P.n_cols; ++j) widths[j] = cols[slot_cols[j]]->stream_bits;
        jit = fused_jit_kernel(iprog, P.first, P.kind, P.n_aggs, P.n_cols, widths, &why, &required);
        if (!jit && required) return fail(EBI_E_CUDA, "run-time compiled expression pass: " + why);
    }
    const void* kernel = jit ? reinterpret_cast<const void*>(jit)
                             : exact ? reinterpret_cast<const void*>(expr_buff_fused<true>)
                                     : reinterpret_cast<const void*>(expr_buff_fused<false>);
    // grid: the CTAs that fit the device at once (each keeps running sums);
    // the compiled walk decodes and aggregates in registers
    const size_t smem = jit ? 0 : fuse_smem(P.n_cols, P.n_aggs);
    if (!jit) {
        const cudaError_t attr = allow_dynamic_smem(kernel, smem);
        if (attr != cudaSuccess) return cuda_fail(attr, "expr_buff_fused shared memory");
    }
    int dev = 0, sms = 0, per_sm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kFuseThreads, smem));
    const uint32_t grid = std::max<uint32_t>(
        1, std::min<uint32_t>((n_units + kFuseWarps - 1) / kFuseWarps, static_cast<uint32_t>(sms * std::max(per_sm, 1))));
    // device: unit0, bad flag, program, partials + results
    uint32_t* d_unit0 = nullptr;
    unsigned long long* d_tot = nullptr;
    Instr* d_prog = nullptr;
    Quad* d_part = nullptr;
    auto done = [&](int code) {
        if (d_unit0) cudaFreeAsync(d_unit0, s);
        if (d_tot) cudaFreeAsync(d_tot, s);
        if (d_prog) cudaFreeAsync(d_prog, s);
        if (d_part) cudaFreeAsync(d_part, s);
        return code;
    };
    if (cudaMallocAsync(reinterpret_cast<void**>(&d_unit0), (C + 1) * sizeof(uint32_t), s) != cudaSuccess ||
        cudaMallocAsync(reinterpret_cast<void**>(&d_tot), 8, s) != cudaSuccess ||
        cudaMallocAsync(reinterpret_cast<void**>(&d_prog), prog.size() * sizeof(Instr), s) != cudaSuccess ||
        cudaMallocAsync(reinterpret_cast<void**>(&d_part), (uint64_t(grid) + 1) * P.n_aggs * sizeof(Quad), s) !=
            cudaSuccess)
        return done(fail(EBI_E_OOM, "expression scratch"));
    ExprScratch S{};
    S.part = d_part;
    S.res = d_part + uint64_t(grid) * P.n_aggs;
    S.prog = d_prog;
    ebi_fx::Params F{};
    for (uint32_t j = 0; j < P.n_cols; ++j) {
        F.file[j] = cols[slot_cols[j]]->d_file;
        F.info[j] = reinterpret_cast<const ebi_fx::ChunkInfo*>(cols[slot_cols[j]]->d_buff);
    }
    F.chunks = reinterpret_cast<const ebi_fx::Chunk*>(r->d_chunks);
    F.in_mask = reinterpret_cast<const uint32_t*>(d_mask);
    F.n_records = r->n_records;
    F.unit0 = d_unit0;
    F.n_units = n_units;
    F.n_chunks = C;
    F.n_cols = P.n_cols;
    F.n_aggs = P.n_aggs;
    F.bad = reinterpret_cast<unsigned int*>(d_tot);
    F.part = reinterpret_cast<ebi_fx::Acc*>(d_part);
    std::vector<Quad> res(P.n_aggs);
    unsigned long long bad = 0;
    CK(cudaMemcpyAsync(d_unit0, unit0.data(), unit0.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(d_tot, 0, 8, s));
    CK(cudaMemcpyAsync(d_prog, (exact ? iprog : prog).data(), prog.size() * sizeof(Instr), cudaMemcpyHostToDevice, s));
    // every CTA writes its partials (identities when it gets no tile)
    if (jit) {
        void* args[] = {&F};
        CK(cudaLaunchKernel(kernel, dim3(grid), dim3(kFuseThreads), args, smem, s));
    } else if (exact) {
        expr_buff_fused<true><<<grid, kFuseThreads, smem, s>>>(P, S, F);
    } else {
        expr_buff_fused<false><<<grid, kFuseThreads, smem, s>>>(P, S, F);
    }
    if (exact) expr_fold_exact<<<P.n_aggs, kExprThreads, 0, s>>>(P, S, grid);
    else expr_fold<<<P.n_aggs, kExprThreads, 0, s>>>(P, S, grid);
    count_launch(2);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(res.data(), S.res, res.size() * sizeof(Quad), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, d_tot, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // unit0 and prog are host memory
    if (e != cudaSuccess) return done(cuda_fail(e, "fused expression evaluation"));
    if (bad) {
        *fell_back = true;
        return done(EBI_OK);
    }
    for (uint32_t a = 0; a < P.n_aggs; ++a) {
        ebi_aggregation& g = aggs[idx[a]];
        if (!exact) {
            g.scalar = g.kind == EBI_AGGR_SUM ? res[a].x : g.kind == EBI_AGGR_MIN ? res[a].y : res[a].z;
            continue;
        }
        unsigned long long w[4];
        std::memcpy(w, &res[a], sizeof w);
        const unsigned long long sign = 0x8000000000000000ull;
        if (g.kind == EBI_AGGR_SUM) {
            g.scalar = scaled_i128(w[0], w[1], f_out[a]);
        } else if (g.kind == EBI_AGGR_MIN) {
            g.scalar = w[2] == (static_cast<unsigned long long>(LLONG_MAX) ^ sign)
                           ? HUGE_VAL : std::ldexp(static_cast<double>(static_cast<long long>(w[2] ^ sign)), -f_out[a]);
        } else {
            g.scalar = w[3] == (static_cast<unsigned long long>(LLONG_MIN) ^ sign)
                           ? -HUGE_VAL : std::ldexp(static_cast<double>(static_cast<long long>(w[3] ^ sign)), -f_out[a]);
        }
    }
    return done(EBI_OK);
}

// One evaluation pass: aggregations idx (at most kMaxAggs, kPassInstr
// instructions and kMaxCols columns together) with their programs.
int run_pass(ebi_column* const* cols, ebi_aggregation* aggs, const std::vector<uint32_t>& idx,
             const std::vector<std::vector<Instr>>& progs, const uint64_t* d_mask, uint32_t C, cudaStream_t s) {
    ExprPass P{};
    P.n_aggs = static_cast<uint32_t>(idx.size());
    P.n_chunks = C;
    std::vector<Instr> prog;
    std::vector<uint32_t> slot_cols;  // slot -> column index
    auto slot = [&](uint16_t col) -> uint16_t {
        for (size_t j = 0; j < slot_cols.size(); ++j)
            if (slot_cols[j] == col) return static_cast<uint16_t>(j);
        slot_cols.push_back(col);
        return static_cast<uint16_t>(slot_cols.size() - 1);
    };
    for (uint32_t a = 0; a < P.n_aggs; ++a) {
        ebi_aggregation& g = aggs[idx[a]];
        P.kind[a] = static_cast<uint32_t>(g.kind);
        P.first[a] = static_cast<uint32_t>(prog.size());
        for (Instr I : progs[idx[a]]) {
            if (I.a == S_COL) { I.ca = slot(I.ca); P.cols[a] |= 1u << I.ca; }
            if (I.b == S_COL) { I.cb = slot(I.cb); P.cols[a] |= 1u << I.cb; }
            prog.push_back(I);
        }
        P.out[a] = g.d_array;
        P.out_cap[a] = g.d_array ? g.array_cap : 0;
    }
    P.first[P.n_aggs] = static_cast<uint32_t>(prog.size());
    P.n_cols = static_cast<uint32_t>(slot_cols.size());
    if (fusable(cols, slot_cols, aggs, idx, progs, C)) {
        bool fell_back = false;
        if (int st = run_fused(cols, aggs, idx, P, prog, slot_cols, d_mask, C, s, &fell_back)) return st;
        if (!fell_back) return EBI_OK;
    }

    // scratch: chunk offsets, lengths, array offsets, items, totals; the
    // columns' values; the item partials; the program
    const uint64_t n_off = uint64_t(P.n_cols) * (C + 1);
    const uint64_t n_u64 = n_off + 2ull * P.n_aggs * C + (C + 1) + (P.n_aggs + 1);
    std::vector<double*> vals(P.n_cols, nullptr);
    unsigned long long* d_u64 = nullptr;
    uint32_t* d_ft = nullptr;
    Instr* d_prog = nullptr;
    Quad* d_part = nullptr;
    auto done = [&](int code) {
        for (double* v : vals) if (v) cudaFreeAsync(v, s);
        if (d_u64) cudaFreeAsync(d_u64, s);
        if (d_ft) cudaFreeAsync(d_ft, s);
        if (d_prog) cudaFreeAsync(d_prog, s);
        if (d_part) cudaFreeAsync(d_part, s);
        return code;
    };
    if (cudaMallocAsync(reinterpret_cast<void**>(&d_u64), n_u64 * 8, s) != cudaSuccess ||
        cudaMallocAsync(reinterpret_cast<void**>(&d_ft), (C + 1) * sizeof(uint32_t), s) != cudaSuccess ||
        cudaMallocAsync(reinterpret_cast<void**>(&d_prog), prog.size() * sizeof(Instr), s) != cudaSuccess)
        return done(fail(EBI_E_OOM, "expression scratch"));
    ExprScratch S{};
    S.off = d_u64;
    S.len = S.off + n_off;
    S.aoff = S.len + uint64_t(P.n_aggs) * C;
    S.item0 = S.aoff + uint64_t(P.n_aggs) * C;
    S.totals = S.item0 + (C + 1);
    S.prog = d_prog;
    uint64_t total_vals = 0;
    for (uint32_t j = 0; j < P.n_cols; ++j) {
        uint64_t n = 0;
        const int st = materialize_column(cols[slot_cols[j]], d_mask, C, S.off + uint64_t(j) * (C + 1), d_ft,
                                          &vals[j], &n, s);
        if (st) return done(st);
        P.vals[j] = vals[j];
        total_vals += n;
    }
    // items: at most sum over chunks of ceil(longest run / kExprItem); the
    // grid: the CTAs that fit the device at once (each keeps running sums)
    const uint64_t items_cap = total_vals / kExprItem + C + 1;
    const size_t smem = size_t(P.n_aggs) * kExprThreads * sizeof(RunAcc);
    const cudaError_t attr = allow_dynamic_smem(reinterpret_cast<const void*>(expr_eval), smem);
    if (attr != cudaSuccess) return done(cuda_fail(attr, "expr_eval shared memory"));
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, expr_eval, kExprThreads, smem);
    const uint32_t grid = static_cast<uint32_t>(
        std::max<uint64_t>(1, std::min<uint64_t>(items_cap, uint64_t(sms) * std::max(per_sm, 1))));
    if (cudaMallocAsync(reinterpret_cast<void**>(&d_part), (uint64_t(grid) + 1) * P.n_aggs * sizeof(Quad), s) !=
        cudaSuccess)
        return done(fail(EBI_E_OOM, "expression partials"));
    S.part = d_part;
    S.res = d_part + uint64_t(grid) * P.n_aggs;
    std::vector<unsigned long long> totals(P.n_aggs + 1);
    std::vector<Quad> res(P.n_aggs);
    cudaError_t e = cudaMemcpyAsync(d_prog, prog.data(), prog.size() * sizeof(Instr), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        expr_prepare<<<1, kExprThreads, 0, s>>>(P, S);
        expr_eval<<<grid, kExprThreads, smem, s>>>(P, S);
        expr_fold<<<P.n_aggs, kExprThreads, 0, s>>>(P, S, grid);
        count_launch(3);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(totals.data(), S.totals, totals.size() * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(res.data(), S.res, res.size() * sizeof(Quad), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return done(cuda_fail(e, "expression evaluation"));
    int st = EBI_OK;
    for (uint32_t a = 0; a < P.n_aggs; ++a) {
        ebi_aggregation& g = aggs[idx[a]];
        if (g.kind == EBI_AGGR_NONE) {
            g.n_array = totals[a];
            if (totals[a] > P.out_cap[a] && !st) st = fail(EBI_E_INVALID, "array output smaller than the values to write");
        } else {
            g.scalar = g.kind == EBI_AGGR_SUM ? res[a].x : g.kind == EBI_AGGR_MIN ? res[a].y : res[a].z;
        }
    }
    return done(st);
}

// Bare Index aggregations that may join the fused pass of the others.  The
// column's own query (exact integer partials for an exact BUFF column) and the
// fused exact pass agree bit for bit when every partial sum in either is
// exactly representable: the column's sum of |value| bounds every partial sum
// of a subset, and buff_exact holds it below 2^52; min and max are exact in
// both.  Folded only when the whole set then fits one fused pass compiled at
// run time (at most kFuseCols BUFF columns, every one readable, exact, at
// most 32 bits wide and chunked like the first column, at most kMaxAggs
// aggregations), so the fold never trades a scan for a slower pass.
std::vector<bool> fold_index_aggregations(ebi_column* const* cols, const ebi_aggregation* aggs, uint32_t n_aggs,
                                          const std::vector<std::vector<Node>>& trees, const std::vector<int>& roots) {
    std::vector<bool> fold(n_aggs, false);
    const ebi_column* r = cols[0];
    auto eligible = [&](const ebi_column* c) {
        if (c->scheme != EBI_BUFF || c->precision >= 0 || !c->d_buff || !c->buff_exact || !c->buff_all_readable ||
            c->buff_max_bits > 32 || c->n_chunks != r->n_chunks || c->n_records != r->n_records || c->n_chunks == 0)
            return false;
        for (uint64_t k = 0; k < c->n_chunks; ++k)
            if (c->chunks[k].n_rows != r->chunks[k].n_rows || c->chunks[k].row_off != r->chunks[k].row_off) return false;
        return true;
    };
    std::vector<uint32_t> used;  // columns of the pass
    uint32_t n_pass = 0, n_index = 0;
    for (uint32_t a = 0; a < n_aggs; ++a) {
        const bool index = trees[a][roots[a]].kind == EBI_EXPR_INDEX;
        if (index && aggs[a].kind == EBI_AGGR_NONE) continue;  // stays an error of its own
        if (!index && aggs[a].kind == EBI_AGGR_NONE) return fold;  // an array result: no fused pass
        for (const Node& n : trees[a])
            if (n.kind == EBI_EXPR_INDEX && std::find(used.begin(), used.end(), n.index) == used.end())
                used.push_back(n.index);
        ++n_pass;
        n_index += index ? 1 : 0;
    }
    if (n_index == 0 || n_index == n_pass || n_pass > static_cast<uint32_t>(kMaxAggs) ||
        used.size() > static_cast<size_t>(kFuseCols) || !fused_jit_enabled())
        return fold;
    for (uint32_t j : used)
        if (!eligible(cols[j])) return fold;
    for (uint32_t a = 0; a < n_aggs; ++a)
        fold[a] = trees[a][roots[a]].kind == EBI_EXPR_INDEX && aggs[a].kind != EBI_AGGR_NONE;
    return fold;
}

}  // namespace
}  // namespace ebi

using namespace ebi;

extern "C" int ebi_aggregate(ebi_column* const* cols, uint32_t n_cols, ebi_aggregation* aggs, uint32_t n_aggs,
                             const uint64_t* d_mask, void* stream) {
    if (!cols || n_cols == 0 || (!aggs && n_aggs)) return fail(EBI_E_INVALID, "no columns or no aggregations");
    for (uint32_t i = 0; i < n_cols; ++i)
        if (!cols[i]) return fail(EBI_E_INVALID, "null column");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::vector<std::vector<Node>> trees(n_aggs);
    std::vector<int> roots(n_aggs);
    for (uint32_t a = 0; a < n_aggs; ++a) {
        if (aggs[a].kind < EBI_AGGR_NONE || aggs[a].kind > EBI_AGGR_SUM) return fail(EBI_E_INVALID, "bad aggregation kind");
        roots[a] = build_tree(aggs[a], n_cols, trees[a]);
        if (roots[a] < 0) return fail(EBI_E_INVALID, "malformed expression (or an index past the columns)");
        aggs[a].n_array = 0;
    }
    // bare Index expressions first, in order (Aggregation::compute_multiple),
    // each through its column's own query -- unless fold_index_aggregations
    // shows that the pass compiled for the other aggregations gives the same
    // results while reading those columns anyway
    const std::vector<bool> folded = fold_index_aggregations(cols, aggs, n_aggs, trees, roots);
    std::vector<uint32_t> rest;
    for (uint32_t a = 0; a < n_aggs; ++a) {
        if (trees[a][roots[a]].kind != EBI_EXPR_INDEX || folded[a]) { rest.push_back(a); continue; }
        if (int st = aggregate_index(cols[trees[a][roots[a]].index], aggs[a], d_mask, stream)) return st;
    }
    if (rest.empty()) return EBI_OK;
    const uint64_t C64 = cols[0]->n_chunks;
    if (C64 == 0) {
        // no chunk is visited: AggregationResult::zero (api/decoder.rs:773-780)
        for (uint32_t a : rest) {
            const int k = aggs[a].kind;
            aggs[a].scalar = k == EBI_AGGR_MAX ? -HUGE_VAL : k == EBI_AGGR_MIN ? HUGE_VAL : 0.0;
        }
        return EBI_OK;
    }
    for (uint32_t i = 0; i < n_cols; ++i)
        if (cols[i]->n_chunks < C64) return fail(EBI_E_INVALID, "a column has fewer chunks than the first");
    if (C64 > (1ull << 30)) return fail(EBI_E_INVALID, "too many chunks");
    const uint32_t C = static_cast<uint32_t>(C64);
    // compile, then pack the programs into passes
    std::vector<std::vector<Instr>> progs(n_aggs);
    for (uint32_t a : rest) {
        Compiler cp{trees[a]};
        cp.gen(roots[a]);
        if (cp.precondition) return fail(EBI_E_PRECONDITION, "Expr::Literal, or an Op over two literals");
        if (cp.max_depth > kMaxStack || cp.out.size() > static_cast<size_t>(kMaxInstr) ||
            program_columns(cp.out).size() > static_cast<size_t>(kMaxCols))
            return fail(EBI_E_INVALID, "expression too large");
        progs[a] = std::move(cp.out);
    }
    // greedy passes in aggregation order
    std::vector<uint32_t> pass, pass_cols;
    size_t instr = 0;
    for (uint32_t a : rest) {
        const std::vector<uint32_t> pc = program_columns(progs[a]);
        std::vector<uint32_t> merged = pass_cols;
        merged.insert(merged.end(), pc.begin(), pc.end());
        std::sort(merged.begin(), merged.end());
        merged.erase(std::unique(merged.begin(), merged.end()), merged.end());
        if (!pass.empty() && (pass.size() == static_cast<size_t>(kMaxAggs) ||
                              instr + progs[a].size() > static_cast<size_t>(kPassInstr) ||
                              merged.size() > static_cast<size_t>(kMaxCols))) {
            if (int st = run_pass(cols, aggs, pass, progs, d_mask, C, s)) return st;
            pass.clear();
            instr = 0;
            merged = pc;
        }
        pass.push_back(a);
        instr += progs[a].size();
        pass_cols = merged;
    }
    if (int st = run_pass(cols, aggs, pass, progs, d_mask, C, s)) return st;
    return EBI_OK;
}
