// expr_fused.cuh -- the fused Expr pass over BUFF columns whose chunks cover
// the same rows, one source for two compilers: nvcc builds it into the
// library with the program interpreters (expr.cu: any program, on the
// fixed-point integers or on the f64 values), and NVRTC builds it at run
// time with an exact pass's programs written out as straight-line code
// (expr_jit.cu).  Self-contained -- no includes -- so that NVRTC
// compiles the text as it is.
//
// Each warp walks its own contiguous range of units (256 rows of one chunk):
// a lane reads its 8 consecutive rows of every column straight from the BUFF
// planes, the fixed-point integers of the selected rows are packed into the
// warp's shared-memory slots (row order, warp shuffles for the offsets), and
// the program object evaluates every aggregation on the packed values and
// adds them to its running aggregates (128-bit sums, order keys of the
// extremes).  Warps synchronise only with themselves until the CTA's final
// reduction, so each one's memory latency overlaps the others' work.
//
// A program object provides
//   kPacked                       true: the walk packs the selected rows
//   n_aggs()                      aggregations of the pass
//   begin()                       sets the thread's running aggregates at rest
//   result(a)                     the thread's running aggregate of aggregation
//                                 a (exact passes: fused_finish_exact)
// and, when kPacked,
//   pack(ci, fixed)               the slot bits of a row's fixed-point integer
//                                 (the integer itself, or its f64 value's bits)
//   unit(slots, lane, ok)         evaluates packed values lane + 32 k (k with
//                                 bit k of ok) and adds them
// else
//   rows(ci, file, g, sel, bad)   decodes rows 8 g .. 8 g + 7 of the warp's
//                                 chunk (headers ci, planes file) itself and
//                                 adds those with bit k of sel set; sets *bad
//                                 when a header carries an error
#pragma once

namespace ebi_fx {

typedef unsigned long long u64;
typedef long long i64;
typedef unsigned int u32;

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kRows = 8;                    // rows per lane
constexpr u32 kUnit = 32 * kRows;           // rows per warp unit
constexpr int kStride = kUnit + kUnit / 8;  // slots per column (one pad every 8: conflict-free)
constexpr int kCols = 4;
constexpr u32 kMax = 1, kMin = 2, kSum = 3;  // aggregation kinds (the C ABI's EBI_AGGR_*)

// Layout twins of the engine's BuffChunkInfo and ChunkDesc (checked where
// nvcc compiles both).
struct ChunkInfo {
    u64 planes, tail;
    i64 base;
    u32 n, bits, frac, status;
    u64 stride;
};
struct Chunk {
    u64 byte_off, byte_len, row_off;
    u32 n_rows, flags;
};

// A running aggregate: a two's complement 128-bit sum and the order keys
// (sign bit flipped) of the least and greatest values.
struct Acc {
    u64 lo, hi, mn, mx;
};

struct Params {
    const unsigned char* file[kCols];
    const ChunkInfo* info[kCols];
    const Chunk* chunks;  // row ranges (identical in every column)
    const u32* in_mask;   // u32 view of the bitmask, or null
    u64 n_records;        // rows the mask covers
    const u32* unit0;     // [n_chunks + 1]: first unit of each chunk
    u32 n_units, n_chunks, n_cols, n_aggs;
    u32* bad;   // set when a chunk's status is not 0
    Acc* part;  // [n_aggs][gridDim.x]: every CTA's aggregates
};

__device__ __forceinline__ u32 umin(u32 a, u32 b) { return a < b ? a : b; }
__device__ __forceinline__ u32 pad(u32 p) { return p + (p >> 3); }
__device__ __forceinline__ u64 skey(i64 v) { return static_cast<u64>(v) ^ 0x8000000000000000ull; }
__device__ __forceinline__ void add128(u64& lo, u64& hi, u64 blo, u64 bhi) {
    const u64 o = lo;
    lo += blo;
    hi += bhi + (lo < o ? 1ull : 0ull);
}
__device__ __forceinline__ Acc acc_rest() {
    return Acc{0, 0, skey(0x7fffffffffffffffll), skey(-0x7fffffffffffffffll - 1)};
}
// The values v[k] with bit k of ok set, added to a running aggregate.
__device__ __forceinline__ void acc_sum(Acc& A, const i64 (&v)[kRows], u32 ok) {
    i64 s = 0;  // at most 8 values below 2^53: no overflow
#pragma unroll
    for (int k = 0; k < kRows; ++k)
        if ((ok >> k) & 1u) s += v[k];
    add128(A.lo, A.hi, static_cast<u64>(s), s < 0 ? ~0ull : 0ull);
}
__device__ __forceinline__ void acc_min(Acc& A, const i64 (&v)[kRows], u32 ok) {
#pragma unroll
    for (int k = 0; k < kRows; ++k) {
        const u64 kk = skey(v[k]);
        if (((ok >> k) & 1u) && kk < A.mn) A.mn = kk;
    }
}
__device__ __forceinline__ void acc_max(Acc& A, const i64 (&v)[kRows], u32 ok) {
#pragma unroll
    for (int k = 0; k < kRows; ++k) {
        const u64 kk = skey(v[k]);
        if (((ok >> k) & 1u) && kk > A.mx) A.mx = kk;
    }
}
__device__ __forceinline__ void acc_add(Acc& A, u32 kind, const i64 (&v)[kRows], u32 ok) {
    if (kind == kSum) acc_sum(A, v, ok);
    else if (kind == kMin) acc_min(A, v, ok);
    else acc_max(A, v, ok);
}

// Bits [r, r + 32) of a u32-word bitmask over n_records rows (0 past the end).
__device__ __forceinline__ u32 mask_bits(const u32* m, u64 r, u64 n_records) {
    if (r >= n_records) return 0;
    const u64 w = r >> 5;
    const u32 sh = static_cast<u32>(r & 31);
    const u32 lo = m[w];
    const u32 hi = (sh && ((w + 1) << 5) < n_records) ? m[w + 1] : 0u;
    u32 v = __funnelshift_r(lo, hi, sh);
    const u64 left = n_records - r;
    if (left < 32) v &= (1u << left) - 1u;
    return v;
}

// The 8 deltas of rows [8 g, 8 g + 8) of a chunk (byte planes, most
// significant first, then the tail bits).
__device__ __forceinline__ void deltas(const unsigned char* file, const ChunkInfo& ci, u32 g, u64 (&d)[kRows]) {
    const u32 np = ci.bits / 8, tb = ci.bits % 8;
#pragma unroll
    for (int i = 0; i < kRows; ++i) d[i] = 0;
    for (u32 p = 0; p < np; ++p) {
        const u64 w = *reinterpret_cast<const u64*>(file + ci.planes + p * ci.stride + u64(g) * 8);
#pragma unroll
        for (int i = 0; i < kRows; ++i) d[i] = (d[i] << 8) | (((w >> (8 * i)) & 0xffull) ^ 0x80ull);
    }
    if (tb) {
        // bits [64 g tb, 64 g tb + 8 tb) of the tail plane: bytes [g tb, g tb + tb)
        const u64 b0 = u64(g) * tb, w0 = b0 & ~3ull;
        const u32* t = reinterpret_cast<const u32*>(file + ci.tail + w0);
        const u32 sh = static_cast<u32>(b0 & 3) * 8;
        const u64 last = b0 + tb - 1;  // the words read end inside the (4-byte aligned) tail plane
        const u32 x0 = t[0];
        const u32 x1 = w0 + 4 <= last ? t[1] : 0u;
        const u32 x2 = w0 + 8 <= last ? t[2] : 0u;
        const u64 lo = static_cast<u64>(x0) | (static_cast<u64>(x1) << 32);
        const u64 bits = sh ? (lo >> sh) | (static_cast<u64>(x2) << (64 - sh)) : lo;
        const u64 m = (1ull << tb) - 1ull;
#pragma unroll
        for (int i = 0; i < kRows; ++i) d[i] = (d[i] << tb) | ((bits >> (i * tb)) & m);
    }
}

// deltas for a chunk NP * 8 + TB <= 32 bits wide, in 32-bit arithmetic
// (the same values).
template <int NP, int TB>
__device__ __forceinline__ void deltas32(const unsigned char* file, const ChunkInfo& ci, u32 g, u32 (&d)[kRows]) {
#pragma unroll
    for (int i = 0; i < kRows; ++i) d[i] = 0;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const u64 w = *reinterpret_cast<const u64*>(file + ci.planes + u64(p) * ci.stride + u64(g) * 8) ^
                      0x8080808080808080ull;
        const u32 lo = static_cast<u32>(w), hi = static_cast<u32>(w >> 32);
#pragma unroll
        for (int i = 0; i < kRows; ++i) d[i] = (d[i] << 8) | (((i < 4 ? lo : hi) >> (8 * (i & 3))) & 0xffu);
    }
    if (TB) {
        const u64 b0 = u64(g) * TB, w0 = b0 & ~3ull;
        const u32* t = reinterpret_cast<const u32*>(file + ci.tail + w0);
        const u32 sh = static_cast<u32>(b0 & 3) * 8;
        const u64 last = b0 + TB - 1;
        const u32 x0 = t[0];
        const u32 x1 = w0 + 4 <= last ? t[1] : 0u;
        const u32 x2 = w0 + 8 <= last ? t[2] : 0u;
        const u64 lo = static_cast<u64>(x0) | (static_cast<u64>(x1) << 32);
        const u64 bits = sh ? (lo >> sh) | (static_cast<u64>(x2) << (64 - sh)) : lo;
#pragma unroll
        for (int i = 0; i < kRows; ++i)
            d[i] = (d[i] << (TB & 7)) | static_cast<u32>((bits >> (i * TB)) & ((1ull << TB) - 1ull));
    }
}

// The walk over the units.  slots (packing program objects): the dynamic
// shared memory, kWarps * n_cols * kStride values first (more after them is
// the program object's).  Ends with the CTA synchronised.
template <class Prog>
__device__ __forceinline__ void fused_walk(const Params& F, Prog& prog, i64* slots) {
    __shared__ ChunkInfo s_ci[kWarps][kCols];
    __shared__ const unsigned char* s_file[kCols];
    __shared__ const ChunkInfo* s_info[kCols];
    const u32 lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    i64* islot = Prog::kPacked ? slots + wid * F.n_cols * kStride : nullptr;
#pragma unroll
    for (int j = 0; j < kCols; ++j)  // constant indices: the parameter arrays stay in the parameter bank
        if (threadIdx.x == j) {
            s_file[j] = F.file[j];
            s_info[j] = F.info[j];
        }
    prog.begin();
    __syncthreads();
    // the warp's units: a contiguous share of all units, in column order
    const u32 C = F.n_chunks, n_warps = gridDim.x * kWarps, gw = blockIdx.x * kWarps + wid;
    const u32 per = (F.n_units + n_warps - 1) / n_warps;
    const u32 u_begin = umin(F.n_units, gw * per), u_end = umin(F.n_units, u_begin + per);
    u32 c = 0xffffffffu, c_end = 0, c_first = 0, n_rows = 0;
    u64 row_off = 0;
    for (u32 u = u_begin; u < u_end; ++u) {
        if (c == 0xffffffffu || u >= c_end) {
            // the chunk of unit u (searched once, then stepped)
            if (c == 0xffffffffu) {
                u32 lo = 0, hi = C;
                while (hi - lo > 1) {
                    const u32 mid = (lo + hi) / 2;
                    if (F.unit0[mid] <= u) lo = mid; else hi = mid;
                }
                c = lo;
            } else {
                do { ++c; } while (F.unit0[c + 1] <= u);
            }
            c_first = F.unit0[c];
            c_end = F.unit0[c + 1];
            n_rows = F.chunks[c].n_rows;
            row_off = F.chunks[c].row_off;
            __syncwarp();
            if (lane < F.n_cols) s_ci[wid][lane] = s_info[lane][c];
            __syncwarp();
        }
        const u32 r = (u - c_first) * kUnit + lane * kRows;  // the lane's first row (in the chunk)
        u32 sel = 0;
        if (r < n_rows) {
            const u32 left = n_rows - r;
            sel = left >= kRows ? 0xffu : ((1u << left) - 1u);
            if (F.in_mask) sel &= mask_bits(F.in_mask, row_off + r, F.n_records);
        }
        if constexpr (!Prog::kPacked) {
            if (sel) prog.rows(s_ci[wid], s_file, r / kRows, sel, F.bad);
        } else {
            // pack position of the lane's first selected row: warp-exclusive prefix of the counts
            const u32 cnt = __popc(sel);
            u32 inc = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const u32 y = __shfl_up_sync(0xffffffffu, inc, o);
                if (static_cast<int>(lane) >= o) inc += y;
            }
            const u32 n_sel = __shfl_sync(0xffffffffu, inc, 31);
            if (n_sel == 0) continue;
            // the lane's rows of every column (no loads without selected rows)
            if (sel) {
                for (u32 j = 0; j < F.n_cols; ++j) {
                    const ChunkInfo ci = s_ci[wid][j];
                    if (ci.status) { atomicOr(F.bad, 1u); continue; }
                    u64 d[kRows];
                    deltas(s_file[j], ci, r / kRows, d);
                    u32 p = inc - cnt;
#pragma unroll
                    for (int i = 0; i < kRows; ++i) {
                        if (!((sel >> i) & 1u)) continue;
                        islot[j * kStride + pad(p++)] = prog.pack(ci, static_cast<i64>(static_cast<u64>(ci.base) + d[i]));
                    }
                }
            }
            __syncwarp();
            // the packed values p = lane + 32 k, k < 8; slots past n_sel hold
            // stale values of the warp's own region, read but not aggregated
            u32 ok = 0;
#pragma unroll
            for (int k = 0; k < kRows; ++k)
                if (lane + u32(k) * 32 < n_sel) ok |= 1u << k;
            prog.unit(islot, lane, ok);
            __syncwarp();  // the slots are rewritten by the next unit
        }
    }
    __syncthreads();
}

// An exact pass's CTA aggregates (per warp, then across warps) into F.part.
template <class Prog>
__device__ __forceinline__ void fused_finish_exact(const Params& F, Prog& prog) {
    __shared__ u64 r_lo[kWarps], r_hi[kWarps], r_mn[kWarps], r_mx[kWarps];
    const u32 lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (u32 a = 0; a < prog.n_aggs(); ++a) {
        const Acc R = prog.result(a);
        u64 lo = R.lo, hi = R.hi, mn = R.mn, mx = R.mx;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            add128(lo, hi, __shfl_xor_sync(0xffffffffu, lo, o), __shfl_xor_sync(0xffffffffu, hi, o));
            const u64 omn = __shfl_xor_sync(0xffffffffu, mn, o), omx = __shfl_xor_sync(0xffffffffu, mx, o);
            mn = omn < mn ? omn : mn;
            mx = omx > mx ? omx : mx;
        }
        if (lane == 0) { r_lo[wid] = lo; r_hi[wid] = hi; r_mn[wid] = mn; r_mx[wid] = mx; }
        __syncthreads();
        if (threadIdx.x == 0) {
            u64 tl = 0, th = 0, tmn = ~0ull, tmx = 0;
            for (int w = 0; w < kWarps; ++w) {
                add128(tl, th, r_lo[w], r_hi[w]);
                tmn = r_mn[w] < tmn ? r_mn[w] : tmn;
                tmx = r_mx[w] > tmx ? r_mx[w] : tmx;
            }
            F.part[a * u64(gridDim.x) + blockIdx.x] = Acc{tl, th, tmn, tmx};
        }
        __syncthreads();
    }
}

}  // namespace ebi_fx
