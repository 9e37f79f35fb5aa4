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
#include <cmath>
#include <vector>

#include "column.h"
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

// One instruction: acc = a OP b (LOAD: acc = a; PUSH: push acc).
enum : uint8_t { I_LOAD = 0, I_PUSH = 1, I_ADD = 2, I_SUB = 3, I_MUL = 4, I_DIV = 5 };
enum : uint8_t { S_ACC = 0, S_POP = 1, S_COL = 2, S_LIT = 3 };
struct Instr {
    uint8_t op, a, b, pad;
    uint16_t ca, cb;    // column slot of an S_COL operand (a column index until a pass assigns slots)
    double la, lb;      // literal of an S_LIT operand
};

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
    Quad* part;             // [n_aggs][items_cap]: sum hi, sum lo, min key, max key
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
    __shared__ Instr prog[kPassInstr];
    __shared__ const double* base[kMaxCols];
    __shared__ double red_h[kExprThreads / 32], red_l[kExprThreads / 32];
    __shared__ unsigned long long red_mn[kExprThreads / 32], red_mx[kExprThreads / 32];
    __shared__ uint32_t s_c;
    const uint32_t n_instr = P.first[P.n_aggs];
    for (uint32_t i = threadIdx.x; i < n_instr; i += kExprThreads) prog[i] = S.prog[i];
    const uint32_t C = P.n_chunks, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
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
            const uint32_t kind = P.kind[a];
            if (kind == EBI_AGGR_NONE) {
                double* out = P.out[a];
                const uint64_t o = S.aoff[uint64_t(a) * C + c], cap = P.out_cap[a];
#pragma unroll
                for (int e = 0; e < kExprPerThread; ++e) {
                    const uint64_t k = k0 + uint64_t(e) * kExprThreads + threadIdx.x;
                    if (k < len && o + k < cap) out[o + k] = acc[e];
                }
                continue;
            }
            ValAgg g = val_agg_init(kind == EBI_AGGR_SUM ? AGG_SUM : (AGG_MIN | AGG_MAX));
#pragma unroll
            for (int e = 0; e < kExprPerThread; ++e) {
                const uint64_t k = k0 + uint64_t(e) * kExprThreads + threadIdx.x;
                if (k < len) val_agg_add1(g, static_cast<uint64_t>(__double_as_longlong(acc[e])));
            }
            // fixed-order tree: lanes, then warps
            double hi = g.hi, lo = g.lo;
            unsigned long long mn = g.mnk, mx = g.mxk;
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
                for (int w = 0; w < kExprThreads / 32; ++w) {
                    dd_add(th, tl, red_h[w], red_l[w]);
                    tmn = red_mn[w] < tmn ? red_mn[w] : tmn;
                    tmx = red_mx[w] > tmx ? red_mx[w] : tmx;
                }
                Quad p;
                p.x = th;
                p.y = tl;
                p.z = __longlong_as_double(static_cast<long long>(tmn));
                p.w = __longlong_as_double(static_cast<long long>(tmx));
                S.part[a * n_items + item] = p;
            }
            __syncthreads();
        }
    }
}

// One CTA per aggregation: the items' partials in item (= chunk) order.
__global__ void __launch_bounds__(kExprThreads) expr_fold(ExprPass P, ExprScratch S) {
    __shared__ double sh_h[kExprThreads / 32], sh_l[kExprThreads / 32];
    __shared__ unsigned long long sh_mn[kExprThreads / 32], sh_mx[kExprThreads / 32];
    const uint32_t a = blockIdx.x;
    if (a >= P.n_aggs || P.kind[a] == EBI_AGGR_NONE) return;
    const unsigned long long n = S.totals[P.n_aggs];
    const Quad* part = S.part + a * n;
    const unsigned long long per = (n + kExprThreads - 1) / kExprThreads;
    const unsigned long long i0 = min(n, threadIdx.x * per), i1 = min(n, i0 + per);
    double hi = 0.0, lo = 0.0;
    unsigned long long mn = kKeyPosInf, mx = kKeyNegInf;
    for (unsigned long long i = i0; i < i1; ++i) {
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
    // items: at most sum over chunks of ceil(longest run / kExprItem)
    const uint64_t items_cap = total_vals / kExprItem + C + 1;
    if (cudaMallocAsync(reinterpret_cast<void**>(&d_part), (items_cap + 1) * P.n_aggs * sizeof(Quad), s) !=
        cudaSuccess)
        return done(fail(EBI_E_OOM, "expression partials"));
    S.part = d_part;
    S.res = d_part + items_cap * P.n_aggs;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t grid = static_cast<uint32_t>(std::max<uint64_t>(1, std::min<uint64_t>(items_cap, uint64_t(sms) * 4)));
    std::vector<unsigned long long> totals(P.n_aggs + 1);
    std::vector<Quad> res(P.n_aggs);
    cudaError_t e = cudaMemcpyAsync(d_prog, prog.data(), prog.size() * sizeof(Instr), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        expr_prepare<<<1, kExprThreads, 0, s>>>(P, S);
        expr_eval<<<grid, kExprThreads, 0, s>>>(P, S);
        expr_fold<<<P.n_aggs, kExprThreads, 0, s>>>(P, S);
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
    // bare Index expressions first, in order (Aggregation::compute_multiple)
    std::vector<uint32_t> rest;
    for (uint32_t a = 0; a < n_aggs; ++a) {
        if (trees[a][roots[a]].kind != EBI_EXPR_INDEX) { rest.push_back(a); continue; }
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
