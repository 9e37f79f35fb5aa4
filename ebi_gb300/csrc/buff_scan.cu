// buff_scan.cu -- the pipelined BUFF scan: filter / filter+aggregate / aggregate
// in one launch.  Bulk copies (cp.async.bulk) stream each tile's byte planes
// into a ring of shared-memory stages; consumer warps decode and test 8 rows
// per lane; the last CTA folds the query result.
#include "buff_query_dev.cuh"
#include "tma.cuh"

namespace ebi {
namespace {
using namespace buff;

// ---------------------------------------------------------------------------
// Pipelined scan: a persistent CTA streams its contiguous range of tiles
// through a ring of shared-memory stages.  Warp 8 is the producer: for every
// tile it reads the chunk's header facts, compiles the predicate and issues
// one bulk copy (cp.async.bulk, the TMA unit) per byte plane plus one for
// the tail plane, all completing on the stage's `full` mbarrier.  Warps 0-7
// consume: each thread decodes 32 rows from shared memory, evaluates the
// predicate, writes its 32-bit bitmask word and accumulates exact per-chunk
// partials in registers, flushed with one atomic per warp when the chunk
// changes.  Consumers release a stage through its `empty` mbarrier.
// ---------------------------------------------------------------------------
constexpr int kScanConsumers = 256;
constexpr int kScanThreads = kScanConsumers + 32;

struct ScanMeta {
    int64_t base;       // the chunk's fixed-point base
    uint64_t row0;      // global row of the tile's first row
    uint32_t chunk, rows, ok, np, tb, bits;
    uint32_t mis[8];    // offset of the tile's first byte inside each plane slot
    uint32_t mis_tail;  // offset of the tile's first tail byte inside the tail slot
    BuffPred pred;
    RangeProg prog;
};

__device__ __forceinline__ uint4 lds16(const uint8_t* p) { return *reinterpret_cast<const uint4*>(p); }

// 32 bytes at an arbitrary shared-memory address as 8 little-endian words.
__device__ __forceinline__ void load32_smem(const uint8_t* p, uint32_t (&w)[8]) {
    const uint32_t a = smem_addr(p);
    const uint32_t s = a & 15;
    const uint8_t* q = p - s;
    uint4 x0 = lds16(q), x1 = lds16(q + 16), x2 = s ? lds16(q + 32) : make_uint4(0, 0, 0, 0);
    uint32_t v[12] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w, x2.x, x2.y, x2.z, x2.w};
    const bool s8 = s & 8, s4 = s & 4;
#pragma unroll
    for (int j = 0; j < 10; ++j) v[j] = s8 ? v[j + 2] : v[j];
#pragma unroll
    for (int j = 0; j < 9; ++j) v[j] = s4 ? v[j + 1] : v[j];
    const uint32_t bs = (s & 3) * 8;
#pragma unroll
    for (int j = 0; j < 8; ++j) w[j] = __funnelshift_r(v[j], v[j + 1], bs);
}

template <int TB, typename D>
__device__ __forceinline__ void scan_rows(const QueryParams& q, const ScanMeta& m, const uint8_t* stage,
                                          const StageLayout& L, Partial& part) {
    const uint32_t t = threadIdx.x;
    const uint32_t lr = 32 * t;
    const bool has_mask = q.in_mask != nullptr;
    const bool want_agg = q.op == OP_FILTER_AGG || q.op == OP_AGG;
    const bool in_tile = lr < m.rows;
    uint32_t sel = 0;
    if (in_tile && m.ok) {
        const uint32_t left = m.rows - lr;
        const uint32_t valid = left >= 32 ? ~0u : ((1u << left) - 1u);
        const uint32_t mw = has_mask ? (mask_word(q.in_mask, m.row0 + lr, q.n_records) & valid) : valid;
        D d[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) d[i] = 0;
        for (uint32_t p = 0; p < m.np; ++p) {
            uint32_t w[8];
            load32_smem(stage + p * L.plane_stride + m.mis[p] + lr, w);
#pragma unroll
            for (int j = 0; j < 8; ++j) w[j] ^= 0x80808080u;
#pragma unroll
            for (int i = 0; i < 32; ++i) d[i] = (d[i] << 8) | static_cast<D>((w[i >> 2] >> (8 * (i & 3))) & 0xffu);
        }
        if constexpr (TB > 0) {
            uint32_t w[8];
            load32_smem(stage + L.np_max * L.plane_stride + m.mis_tail + 4 * TB * t, w);
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                constexpr uint32_t msk = (1u << TB) - 1u;
                const int pos = i * TB, wi = pos >> 5, sh = pos & 31;
                const uint32_t f = (sh + TB <= 32) ? (w[wi] >> sh) : __funnelshift_r(w[wi], w[wi + 1], sh);
                d[i] = static_cast<D>((d[i] << TB) | static_cast<D>(f & msk));
            }
        }
        const BuffPred& k = m.pred;
        if (q.op == OP_AGG) {
            sel = mw;
        } else if (q.pred.kind == EBI_PRED_RANGE) {
            const bool la = k.lmode == SIDE_ABSENT, ra = k.rmode == SIDE_ABSENT;
            uint32_t Lw = 0, Rw = 0;
            if (k.lmode == SIDE_ALL) Lw = valid;
            else if (k.lmode == SIDE_CMP) Lw = cmp_word<D>(d, k.lthr, true, k.lincl) & mw;
            if (k.rmode == SIDE_ALL) Rw = valid;
            else if (k.rmode == SIDE_CMP) Rw = cmp_word<D>(d, k.rthr, false, k.rincl) & mw;
            sel = (la && ra) ? mw : la ? Rw : ra ? Lw : (Lw & Rw);
        } else {
            uint32_t e = 0;
            if (k.emode == SIDE_ALL) e = valid;
            else if (k.emode == SIDE_CMP) e = eq_word<D>(d, k.etgt) & mw;
            sel = q.pred.kind == EBI_PRED_EQ ? e : (mw & ~e);
        }
        if (want_agg && sel) {
            unsigned long long s64 = 0;
            D mx = 0, mn = static_cast<D>(~D(0));
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                const bool on = (sel >> i) & 1u;
                s64 += on ? static_cast<unsigned long long>(d[i]) : 0ull;
                mx = (on && d[i] > mx) ? d[i] : mx;
                mn = (on && d[i] < mn) ? d[i] : mn;
            }
            part.sum += s64;
            part.cnt += __popc(sel);
            part.mx = static_cast<unsigned long long>(mx) > part.mx ? static_cast<unsigned long long>(mx) : part.mx;
            part.mn = static_cast<unsigned long long>(mn) < part.mn ? static_cast<unsigned long long>(mn) : part.mn;
        }
    }
    if ((q.op == OP_FILTER || q.op == OP_FILTER_AGG) && in_tile && q.out_mask) {
        if (!q.out_atomic || sel) store_mask_word(q.out_mask, m.row0 + lr, sel, q.out_atomic);
    }
}


// Fast path for chunks of 8 to 32 bits.  Each lane handles quads of 4
// consecutive rows; quad j * 256 + t of the tile belongs to thread t, so the
// 32 lanes of a warp read consecutive words of every plane (no shared-memory
// bank conflicts).  Deltas are u32, assembled with byte permutes; the
// predicate is one unsigned range test per row; the loop is straight-line.
template <int NP, int TB, bool SUM, bool MINMAX, bool FAST>
__device__ __forceinline__ void scan_quads(const QueryParams& q, const ScanMeta& m, const uint8_t* stage,
                                           const StageLayout& L, Partial& part) {
    static_assert(NP >= 1 && NP <= 4 && NP * 8 + TB <= 32, "u32 deltas");
    constexpr bool kSum32 = NP * 8 + TB <= 27;  // 32 rows of deltas fit a u32 sum
    const uint32_t t = threadIdx.x, lane = t & 31;
    const bool has_mask = q.in_mask != nullptr;
    const bool store = (q.op == OP_FILTER || q.op == OP_FILTER_AGG) && q.out_mask;
    const RangeProg& g = m.prog;
    const uint32_t lo = static_cast<uint32_t>(g.lo), span = static_cast<uint32_t>(g.hi - g.lo);
    const bool test = !(g.empty || g.full);
    const uint32_t fixed_cw = g.full ? 0xfu : 0u;
    const uint32_t neg = g.negate ? 0xfu : 0u;
    const bool use_mask = g.use_mask && has_mask;
    const uint32_t* slot[NP];
    uint32_t rsh[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        slot[p] = reinterpret_cast<const uint32_t*>(stage + p * L.plane_stride + (m.mis[p] & ~3u));
        rsh[p] = 8 * (m.mis[p] & 3);
    }
    const uint32_t* tslot = reinterpret_cast<const uint32_t*>(stage + L.np_max * L.plane_stride);
    const uint32_t tbit0 = 8 * m.mis_tail;
    uint32_t cnt = 0, mx = 0, mn = ~0u;
    uint32_t s32 = 0;
    unsigned long long s64 = 0;
#pragma unroll 2
    for (int j = 0; j < 8; ++j) {
        const uint32_t qd = j * kScanConsumers + t;  // quad index in the tile
        const uint32_t r = 4 * qd;                   // first row of the quad in the tile
        uint32_t nib = 0;
        if (FAST || r < m.rows) {
            const uint32_t left = m.rows - r;
            const uint32_t valid = FAST ? 0xfu : (left >= 4 ? 0xfu : ((1u << left) - 1u));
            uint32_t w[NP];
#pragma unroll
            for (int p = 0; p < NP; ++p) w[p] = __funnelshift_r(slot[p][qd], slot[p][qd + 1], rsh[p]) ^ 0x80808080u;
            uint32_t v[4];
            if constexpr (NP == 1) {
#pragma unroll
                for (int k = 0; k < 4; ++k) v[k] = __byte_perm(w[0], 0u, 0x4440u | k);
            } else if constexpr (NP == 2) {
                const uint32_t P = __byte_perm(w[1], w[0], 0x5140u), Q = __byte_perm(w[1], w[0], 0x7362u);
                v[0] = P & 0xffffu; v[1] = P >> 16; v[2] = Q & 0xffffu; v[3] = Q >> 16;
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    uint32_t x = 0;
#pragma unroll
                    for (int p = 0; p < NP; ++p) x = (x << 8) | ((w[p] >> (8 * k)) & 0xffu);
                    v[k] = x;
                }
            }
            uint32_t d[4];
            if constexpr (TB > 0) {
                const uint32_t b = tbit0 + 4 * TB * qd;
                const uint32_t f = __funnelshift_r(tslot[b >> 5], tslot[(b >> 5) + 1], b & 31);
#pragma unroll
                for (int k = 0; k < 4; ++k) d[k] = (v[k] << TB) | ((f >> (TB * k)) & ((1u << TB) - 1u));
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) d[k] = v[k];
            }
            if constexpr (FAST) {
                // full tile, no input bitmask, predicate not negated: the range
                // test itself drives the bitmask bit and the accumulators
                if (test) {
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const bool in = d[k] - lo <= span;
                        nib |= static_cast<uint32_t>(in) << k;
                        if constexpr (SUM) { if (in) { if constexpr (kSum32) s32 += d[k]; else s64 += d[k]; } }
                        if constexpr (MINMAX) { if (in) { mx = max(mx, d[k]); mn = min(mn, d[k]); } }
                    }
                } else if (g.full) {
                    nib = 0xfu;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        if constexpr (SUM) { if constexpr (kSum32) s32 += d[k]; else s64 += d[k]; }
                        if constexpr (MINMAX) { mx = max(mx, d[k]); mn = min(mn, d[k]); }
                    }
                }
                cnt += __popc(nib);
            } else {
            uint32_t cw = fixed_cw;
            if (test) {
#pragma unroll
                for (int k = 0; k < 4; ++k) cw |= static_cast<uint32_t>(d[k] - lo <= span) << k;
            }
            uint32_t base_set = valid;
            if (use_mask) base_set &= mask_word(q.in_mask, m.row0 + r, q.n_records);
            nib = (cw ^ neg) & base_set;
            cnt += __popc(nib);
            if constexpr (SUM) {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const uint32_t x = ((nib >> k) & 1u) ? d[k] : 0u;
                    if constexpr (kSum32) s32 += x; else s64 += x;
                }
            }
            if constexpr (MINMAX) {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const bool on = (nib >> k) & 1u;
                    mx = max(mx, on ? d[k] : 0u);
                    mn = min(mn, on ? d[k] : ~0u);
                }
            }
            }
        }
        if (store) {
            // 8 lanes hold the 32 rows of one bitmask word: gather their nibbles
            uint32_t x = nib << (4 * (lane & 7));
            x |= __shfl_xor_sync(0xffffffffu, x, 1);
            x |= __shfl_xor_sync(0xffffffffu, x, 2);
            x |= __shfl_xor_sync(0xffffffffu, x, 4);
            const uint32_t r0 = 4 * (j * kScanConsumers + (t & ~7u));  // first row of the word in the tile
            if ((lane & 7) == 0 && r0 < m.rows && (!q.out_atomic || x))
                store_mask_word(q.out_mask, m.row0 + r0, x, q.out_atomic);
        }
    }
    if (q.op == OP_FILTER_AGG || q.op == OP_AGG) {
        part.cnt += cnt;
        part.sum += kSum32 ? s32 : s64;
        part.mx = mx > part.mx ? mx : part.mx;
        part.mn = mn < part.mn ? mn : part.mn;
    }
}


// Fastest path: a full tile, no input bitmask, a predicate that is not
// negated, chunks of 8..32 bits.  Each lane decodes 8 consecutive rows per
// step (oct j * 256 + t of the tile), so a plane contributes 8 bytes and the
// tail exactly TB bytes per lane; everything is unrolled with constant
// offsets.  Four lanes assemble one 32-bit bitmask word.
template <int NP, int TB, bool SUM, bool MINMAX>
__device__ __forceinline__ void scan_octs(const QueryParams& q, const ScanMeta& m, const uint8_t* stage,
                                          const StageLayout& L, Partial& part) {
    constexpr bool kSum32 = NP * 8 + TB <= 27;
    const uint32_t t = threadIdx.x, lane = t & 31;
    const bool store = (q.op == OP_FILTER || q.op == OP_FILTER_AGG) && q.out_mask;
    const RangeProg& g = m.prog;
    const uint32_t lo = static_cast<uint32_t>(g.lo), span = static_cast<uint32_t>(g.hi - g.lo);
    const bool test = !(g.empty || g.full), all = g.full;
    const uint32_t* slot[NP];
    uint32_t rsh[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        slot[p] = reinterpret_cast<const uint32_t*>(stage + p * L.plane_stride + (m.mis[p] & ~3u)) + 2 * t;
        rsh[p] = 8 * (m.mis[p] & 3);
    }
    const uint8_t* tail = stage + L.np_max * L.plane_stride + m.mis_tail + TB * t;
    uint32_t cnt = 0, mx = 0, mn = ~0u, s32 = 0;
    unsigned long long s64 = 0;
    uint32_t* out = store ? q.out_mask + ((m.row0 >> 5) + (t >> 2)) : nullptr;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        // two words (8 rows) of each plane
        uint32_t lo_w[NP], hi_w[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            const uint32_t* sp = slot[p] + 512 * j;
            const uint32_t a = sp[0], b = sp[1], c = sp[2];
            lo_w[p] = __funnelshift_r(a, b, rsh[p]) ^ 0x80808080u;
            hi_w[p] = __funnelshift_r(b, c, rsh[p]) ^ 0x80808080u;
        }
        uint32_t v[8];
        if constexpr (NP == 1) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                v[k] = __byte_perm(lo_w[0], 0u, 0x4440u | k);
                v[k + 4] = __byte_perm(hi_w[0], 0u, 0x4440u | k);
            }
        } else if constexpr (NP == 2) {
            const uint32_t P0 = __byte_perm(lo_w[1], lo_w[0], 0x5140u), Q0 = __byte_perm(lo_w[1], lo_w[0], 0x7362u);
            const uint32_t P1 = __byte_perm(hi_w[1], hi_w[0], 0x5140u), Q1 = __byte_perm(hi_w[1], hi_w[0], 0x7362u);
            v[0] = P0 & 0xffffu; v[1] = P0 >> 16; v[2] = Q0 & 0xffffu; v[3] = Q0 >> 16;
            v[4] = P1 & 0xffffu; v[5] = P1 >> 16; v[6] = Q1 & 0xffffu; v[7] = Q1 >> 16;
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                uint32_t x = 0;
#pragma unroll
                for (int p = 0; p < NP; ++p) x = (x << 8) | (((k < 4 ? lo_w[p] : hi_w[p]) >> (8 * (k & 3))) & 0xffu);
                v[k] = x;
            }
        }
        uint32_t d[8];
        if constexpr (TB > 0) {
            // TB bytes of tail bits for these 8 rows, at byte offset TB * (j * 256 + t)
            const uint8_t* tp = tail + TB * 256 * j;
            const uint32_t ba = static_cast<uint32_t>(reinterpret_cast<uintptr_t>(tp)) & 3u;
            const uint32_t* tw = reinterpret_cast<const uint32_t*>(tp - ba);
            const uint32_t t0 = tw[0], t1 = tw[1], t2 = tw[2];
            const uint32_t f0 = __funnelshift_r(t0, t1, 8 * ba), f1 = __funnelshift_r(t1, t2, 8 * ba);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                constexpr uint32_t msk = (1u << TB) - 1u;
                const int pos = k * TB;
                const uint32_t f = pos + TB <= 32 ? (f0 >> pos) : (pos >= 32 ? (f1 >> (pos - 32)) : __funnelshift_r(f0, f1, pos));
                d[k] = (v[k] << TB) | (f & msk);
            }
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k) d[k] = v[k];
        }
        uint32_t bits = 0;
        if (test) {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const bool in = d[k] - lo <= span;
                bits |= in ? (1u << k) : 0u;
                if constexpr (SUM) { if (in) { if constexpr (kSum32) s32 += d[k]; else s64 += d[k]; } }
                if constexpr (MINMAX) { if (in) { mx = max(mx, d[k]); mn = min(mn, d[k]); } }
            }
        } else if (all) {
            bits = 0xffu;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if constexpr (SUM) { if constexpr (kSum32) s32 += d[k]; else s64 += d[k]; }
                if constexpr (MINMAX) { mx = max(mx, d[k]); mn = min(mn, d[k]); }
            }
        }
        cnt += __popc(bits);
        if (store) {
            uint32_t x = bits << (8 * (lane & 3));
            x |= __shfl_xor_sync(0xffffffffu, x, 1);
            x |= __shfl_xor_sync(0xffffffffu, x, 2);
            if ((lane & 3) == 0) out[64 * j] = x;
        }
    }
    if (q.op == OP_FILTER_AGG || q.op == OP_AGG) {
        part.cnt += cnt;
        part.sum += kSum32 ? s32 : s64;
        part.mx = mx > part.mx ? mx : part.mx;
        part.mn = mn < part.mn ? mn : part.mn;
    }
}

template <int NP, int TB>
__device__ __forceinline__ void scan_quads_agg(const QueryParams& q, const ScanMeta& m, const uint8_t* st,
                                               const StageLayout& L, Partial& part) {
    const bool agg = q.op == OP_FILTER_AGG || q.op == OP_AGG;
    const bool sum = agg && (q.agg & AGG_SUM), mm = agg && (q.agg & (AGG_MIN | AGG_MAX));
    const bool fast = m.rows == kBuffTileRows && !(m.prog.use_mask && q.in_mask) && !m.prog.negate;
    if (fast && !q.out_atomic) {
        if (mm) scan_octs<NP, TB, true, true>(q, m, st, L, part);
        else scan_octs<NP, TB, true, false>(q, m, st, L, part);
    } else {
        (void)sum;
        scan_quads<NP, TB, true, true, false>(q, m, st, L, part);
    }
}

#define EBI_Q(NP, TB) case NP * 8 + TB: scan_quads_agg<NP, TB>(q, m, st, L, part); return true;
// Chunks of 8..32 bits; false for the others (they take the generic path).
__device__ bool scan_fast_dispatch(const QueryParams& q, const ScanMeta& m, const uint8_t* st, const StageLayout& L,
                                   Partial& part) {
    switch (m.bits) {
        EBI_Q(1, 0) EBI_Q(1, 1) EBI_Q(1, 2) EBI_Q(1, 3) EBI_Q(1, 4) EBI_Q(1, 5) EBI_Q(1, 6) EBI_Q(1, 7)
        EBI_Q(2, 0) EBI_Q(2, 1) EBI_Q(2, 2) EBI_Q(2, 3) EBI_Q(2, 4) EBI_Q(2, 5) EBI_Q(2, 6) EBI_Q(2, 7)
        EBI_Q(3, 0) EBI_Q(3, 1) EBI_Q(3, 2) EBI_Q(3, 3) EBI_Q(3, 4) EBI_Q(3, 5) EBI_Q(3, 6) EBI_Q(3, 7)
        EBI_Q(4, 0)
        default: return false;
    }
}
#undef EBI_Q

template <typename D>
__device__ __forceinline__ void scan_dispatch(const QueryParams& q, const ScanMeta& m, const uint8_t* stage,
                                              const StageLayout& L, Partial& part) {
    switch (m.ok ? m.tb : 0) {
        case 0: scan_rows<0, D>(q, m, stage, L, part); break;
        case 1: scan_rows<1, D>(q, m, stage, L, part); break;
        case 2: scan_rows<2, D>(q, m, stage, L, part); break;
        case 3: scan_rows<3, D>(q, m, stage, L, part); break;
        case 4: scan_rows<4, D>(q, m, stage, L, part); break;
        case 5: scan_rows<5, D>(q, m, stage, L, part); break;
        case 6: scan_rows<6, D>(q, m, stage, L, part); break;
        default: scan_rows<7, D>(q, m, stage, L, part); break;
    }
}

// A tile's metadata and copy plan, prepared by one producer lane.
struct PreTile {
    ScanMeta m;
    uint64_t planes, tail;  // device offsets of the chunk's first plane and tail plane
    uint64_t stride;        // bytes from one plane to the next
    uint32_t begin;         // the tile's first row
    uint32_t bytes;         // bytes the tile's copies deliver
};

__device__ __forceinline__ void prepare_tile(const QueryParams& q, const BuffChunkInfo* info, ScanTotals* T,
                                             uint32_t tile, bool has_mask, PreTile& pt) {
    const Tile tl = q.tiles[tile];
    const uint32_t c = tl.chunk;
    const ChunkDesc cd = q.chunks[c];
    const BuffChunkInfo ci = info[c];
    ScanMeta& m = pt.m;
    const bool selected = has_mask ? q.acc[c].selected != 0
                                   : (q.chunk_id < 0 || static_cast<uint64_t>(q.chunk_id) == c);
    if (selected && tl.begin == 0) {
        if (!has_mask) q.acc[c].selected = 1;
        if (ci.status) chunk_error(q, T, c, ci.status);
    }
    m.chunk = c;
    m.base = ci.base;
    m.row0 = cd.row_off + tl.begin;
    m.rows = min(kBuffTileRows, cd.n_rows - tl.begin);
    m.ok = selected && ci.status == 0;
    pt.planes = ci.planes;
    pt.tail = ci.tail;
    pt.stride = ci.stride;
    pt.begin = tl.begin;
    uint32_t bytes = 0;
    if (m.ok) {
        m.np = ci.bits / 8;
        m.tb = ci.bits % 8;
        m.bits = ci.bits;
        compile_pred(q.pred, ci.base, ci.bits, ci.frac, has_mask, m.pred);
        m.prog = compile_prog(q, m.pred, ci.bits, has_mask);
        for (uint32_t p = 0; p < m.np; ++p) {
            const uintptr_t src = reinterpret_cast<uintptr_t>(q.file + ci.planes + uint64_t(p) * ci.stride + tl.begin);
            const uintptr_t a = src & ~uintptr_t(15);
            m.mis[p] = static_cast<uint32_t>(src - a);
            bytes += static_cast<uint32_t>(((src + m.rows + 15) & ~uintptr_t(15)) - a);
        }
        if (m.tb) {
            const uintptr_t src = reinterpret_cast<uintptr_t>(q.file + ci.tail + uint64_t(tl.begin / 8) * m.tb);
            const uintptr_t a = src & ~uintptr_t(15);
            m.mis_tail = static_cast<uint32_t>(src - a);
            bytes += static_cast<uint32_t>(((src + (uint64_t(m.rows) * m.tb + 7) / 8 + 15) & ~uintptr_t(15)) - a);
        }
    } else {
        m.np = 0;
        m.tb = 0;
    }
    pt.bytes = bytes;
}

__global__ void __launch_bounds__(kScanThreads, 2)
buff_scan_kernel(QueryParams q, const BuffChunkInfo* info, uint32_t tile_base, uint32_t n_tiles, StageLayout L,
                 ScanTotals* T, QueryResult* res, uint32_t frac, uint32_t fast_ok) {
    extern __shared__ __align__(128) uint8_t smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem);
    uint64_t* empty = full + L.stages;
    ScanMeta* meta = reinterpret_cast<ScanMeta*>(smem + 128);
    uint8_t* stages = smem + L.data_offset;
    // contiguous tile range of this CTA
    const uint32_t t_first = static_cast<uint32_t>((uint64_t(n_tiles) * blockIdx.x) / gridDim.x);
    const uint32_t t_end = static_cast<uint32_t>((uint64_t(n_tiles) * (blockIdx.x + 1)) / gridDim.x);
    const uint32_t count = t_end - t_first;
    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < L.stages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kScanConsumers / 32);
        }
        fence_mbar_init();
    }
    __syncthreads();
    const bool has_mask = q.in_mask != nullptr;

    if (threadIdx.x >= kScanConsumers) {
        // ---- producer warp.  Its lanes prepare the next 32 tiles' metadata in
        // parallel (the chunk-table loads of different tiles overlap instead of
        // queueing behind one lane); lane 0 then runs the ring in tile order:
        // wait for a free stage, publish the tile's metadata, issue its copies.
        const uint32_t lane = threadIdx.x - kScanConsumers;
        __shared__ PreTile pre[32];
        bool stop = false;
        uint32_t issued = 0;  // tiles whose copies lane 0 issued
        for (uint32_t i0 = 0; i0 < count && !stop; i0 += 32) {
            const uint32_t nb = count - i0 < 32 ? count - i0 : 32u;
            if (lane < nb) prepare_tile(q, info, T, tile_base + t_first + i0 + lane, has_mask, pre[lane]);
            __syncwarp();
            if (lane == 0) {
                for (uint32_t j = 0; j < nb; ++j) {
                    const uint32_t i = i0 + j, s = i % L.stages, k = i / L.stages;
                    if (k > 0 && !mbar_wait(&empty[s], (k - 1) & 1, q.copy_wait)) {
                        chunk_error(q, T, 0, EBI_E_CUDA);
                        stop = true;  // consumers stopped; nothing of this stage is in flight
                        break;
                    }
                    const PreTile& pt = pre[j];
                    meta[s] = pt.m;
                    uint8_t* st = stages + size_t(s) * L.stage_bytes;
                    fence_proxy_async_smem();
                    mbar_arrive_expect_tx(&full[s], pt.bytes);
                    if (pt.m.ok) {
                        for (uint32_t p = 0; p < pt.m.np; ++p) {
                            const uintptr_t src = reinterpret_cast<uintptr_t>(q.file + pt.planes + uint64_t(p) * pt.stride + pt.begin);
                            const uintptr_t a = src & ~uintptr_t(15);
                            const uint32_t len = static_cast<uint32_t>(((src + pt.m.rows + 15) & ~uintptr_t(15)) - a);
                            bulk_g2s(st + p * L.plane_stride, reinterpret_cast<const void*>(a), len, &full[s]);
                        }
                        if (pt.m.tb) {
                            const uintptr_t src = reinterpret_cast<uintptr_t>(q.file + pt.tail + uint64_t(pt.begin / 8) * pt.m.tb);
                            const uintptr_t a = src & ~uintptr_t(15);
                            const uint32_t len = static_cast<uint32_t>(
                                ((src + (uint64_t(pt.m.rows) * pt.m.tb + 7) / 8 + 15) & ~uintptr_t(15)) - a);
                            bulk_g2s(st + L.np_max * L.plane_stride, reinterpret_cast<const void*>(a), len, &full[s]);
                        }
                    }
                    issued = i + 1;
                }
            }
            stop = __shfl_sync(0xffffffffu, stop, 0);
            __syncwarp();  // pre[] is rewritten only after lane 0 consumed it
        }
        // drain (full limit whatever q.copy_wait): the copies of the last stages
        // issued complete before this warp leaves
        if (lane == 0)
            for (uint32_t i = issued > L.stages ? issued - L.stages : 0; i < issued; ++i)
                if (!mbar_wait(&full[i % L.stages], (i / L.stages) & 1)) { chunk_error(q, T, 0, EBI_E_CUDA); break; }
    }
    __shared__ WarpTot wtot[kScanConsumers / 32];
    if (threadIdx.x < kScanConsumers) {
    // ---- consumer warps ----
    Partial part{0, 0, 0, ~0ull};
    WarpTot wt{0, 0, 0, LLONG_MIN, LLONG_MAX, 0};
    uint32_t cur = 0xffffffffu;
    int64_t cur_base = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const uint32_t s = i % L.stages, k = i / L.stages;
        if (!mbar_wait(&full[s], k & 1, q.copy_wait)) {
            chunk_error(q, T, 0, EBI_E_CUDA);
            break;
        }
        const ScanMeta& m = meta[s];
        if (m.chunk != cur) {
            if (cur != 0xffffffffu) flush_partial(q, cur, cur_base, part, wt);
            cur = m.chunk;
            cur_base = m.base;
        }
        const uint8_t* st = stages + size_t(s) * L.stage_bytes;
        if (!m.ok) scan_dispatch<uint32_t>(q, m, st, L, part);  // writes zero words only
        else if (m.bits > 32) scan_dispatch<unsigned long long>(q, m, st, L, part);
        else if (!scan_fast_dispatch(q, m, st, L, part)) scan_dispatch<uint32_t>(q, m, st, L, part);
        __syncwarp();
        if ((threadIdx.x & 31) == 0) mbar_arrive(&empty[s]);
    }
    if (cur != 0xffffffffu) flush_partial(q, cur, cur_base, part, wt);
    if ((threadIdx.x & 31) == 0) wtot[threadIdx.x >> 5] = wt;
    }
    cta_finish(q, info, T, res, frac, fast_ok != 0, wtot, kScanConsumers / 32);
}

}  // namespace

StageLayout buff_stage_layout(uint32_t np_max, uint32_t tb_max, uint32_t* ctas_per_sm) {
    StageLayout L{};
    L.plane_stride = kBuffTileRows + 32;
    L.np_max = np_max;
    L.tail_stride = ((kBuffTileRows / 8) * tb_max + 48 + 15) & ~15u;
    L.stage_bytes = (np_max * L.plane_stride + L.tail_stride + 127) & ~127u;
    const uint32_t meta = 128 + 8 * static_cast<uint32_t>(sizeof(ScanMeta));  // barriers + up to 8 stages
    L.data_offset = (meta + 127) & ~127u;
    const uint32_t budget2 = 110 * 1024, budget1 = 220 * 1024;
    uint32_t st = (budget2 - L.data_offset) / L.stage_bytes;
    *ctas_per_sm = 2;
    if (st < 3) {
        st = (budget1 - L.data_offset) / L.stage_bytes;
        *ctas_per_sm = 1;
    }
    L.stages = st > 8 ? 8 : (st < 2 ? 2 : st);
    if (L.stages > 4 && *ctas_per_sm == 2) L.stages = 4;
    return L;
}

cudaError_t launch_buff_scan(const QueryParams& q, const BuffChunkInfo* info, uint32_t tile_begin, uint32_t n_tiles,
                            const StageLayout& L, uint32_t grid, ScanTotals* T, QueryResult* res, uint32_t frac,
                            bool fast_ok, cudaStream_t s) {
    if (n_tiles == 0) return cudaSuccess;
    const size_t smem = L.data_offset + size_t(L.stages) * L.stage_bytes;
    const cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void*>(buff_scan_kernel), smem);
    if (e != cudaSuccess) return e;
    if ((grid < n_tiles ? grid : n_tiles) > kScanSlots) return cudaErrorInvalidConfiguration;
    buff_scan_kernel<<<grid < n_tiles ? grid : n_tiles, kScanThreads, smem, s>>>(q, info, tile_begin, n_tiles, L, T,
                                                                               res, frac, fast_ok ? 1u : 0u);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ebi
