// xor_dev.cuh -- Gorilla, Chimp, Chimp128, Elf and ElfOnChimp chunks: XOR
// bitstreams decoded on the device and queried in the same kernel (one CTA
// per chunk).
//
// Formats (big-endian bit order, MSB of the first byte first):
//   Gorilla   decoder/chunk_reader/gorilla.rs:90-157: 64 raw bits, then per
//             value '0' (repeat), '10' + payload in the inherited window, or
//             '11' + 5-bit leading + 6-bit (significant - 1) + payload.
//   Chimp     decoder/chunk_reader/chimp.rs:58-124: 2-bit flags; '01' carries
//             a 3-bit leading code (LEADING_REPR) and 6 significant bits.
//   Chimp128  decoder/chunk_reader/chimp_n.rs:160-285: as Chimp, but '00' and
//             '01' name one of the last 128 values by a 7-bit ring index.
//   Elf       decoder/chunk_reader/elf.rs: per value a wrapper prefix ('0'
//             restore, '10' as is, '11' + 4-bit beta* and restore) and an
//             ElfXor record; ElfOnChimp: the same prefix over Chimp records.
//             The XOR chain runs over the erased values v'; a restored value
//             is v' rounded up at the digits beta* names (elf_dev.cuh).
// A stream ends at the first value equal to f64::NAN's bits (Chimp128: not
// for a '00' copy); a read past the chunk raises UnexpectedEndOfChunk first.
//
// Decoding is split in three parallel steps:
//   1. control parse.  The chunk's bits (read through L1 from the resident
//      file) are cut into one segment per thread.  Thread 0 starts at the true first record;
//      every other thread guesses a start and parses its segment.  Each round
//      a thread whose start differs from its predecessor's end adopts that end
//      and parses again.  The segments agree with the sequential parse once
//      every start equals its predecessor's end up to the first failing
//      segment; by induction from thread 0 that takes at most one round per
//      segment, and far fewer when misaligned parses fall back into step with
//      the true record boundaries (Chimp and Chimp128 do within ~100 records).
//   2. extraction.  Record offsets come from a block scan of the segment
//      record counts; each thread re-parses its segment and writes every
//      record's XOR delta (and, for Chimp128, the record its value refers to).
//   3. values.  Gorilla, Chimp and Elf values are the prefix XOR of the deltas
//      (warp-shuffle scans); Chimp128 values resolve by pointer jumping over
//      the references (ceil(log2 n) rounds).  The first NaN ends the chunk.
//      Elf: each record takes the beta* of the last '11' prefix at or before
//      it (a block max-scan over record indices) and restores its value.
// The query then runs row-parallel over the values in shared memory.
//
// A chunk with more records than kRcap (only for chunks far above 8,192
// values) is decoded by one thread in order.
#pragma once

#include "bitstream.cuh"
#include "values.cuh"
#include "xor_parse.cuh"

namespace ebi {
namespace {

using namespace xorp;

constexpr int kXorThreads = 256;
constexpr uint32_t kRcap = 8448;         // records (values) held in shared memory
__device__ __forceinline__ uint32_t block_min_u32(uint32_t v, uint32_t* sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    uint32_t m = sh[0];
#pragma unroll
    for (int w = 1; w < kXorThreads / 32; ++w) m = min(m, sh[w]);
    return m;
}

struct Smem {
    uint64_t* vals;   // kRcap: deltas, then values
    uint16_t* refs;   // kRcap (Chimp128)
    uint32_t* nanok;  // kRcap / 32 (Chimp128)
    uint8_t* meta;    // kRcap (Elf): wrapper prefix flags and beta*
};

// Row sink of the query: one call per decoded row, in row order within the
// calling thread.  Used by the sequential path (thread 0 alone).
struct SerialSink {
    const QueryParams* q;
    uint64_t row_off;
    int mode;
    bool has_mask, pred_on, store;
    KeyPred kp;
    ValAgg agg;
    unsigned long long pos;
    uint64_t word_idx;
    uint32_t word;
    __device__ void flush() {
        if (word) atomicOr(&q->out_mask[word_idx], word);
        word = 0;
    }
    __device__ void row(uint64_t i, uint64_t vb) {
        const uint64_t g = row_off + i;
        const bool in = !has_mask || mask_row(q->in_mask, q->n_records, g);
        const bool pass = in && (!pred_on || kp.pass(vb));
        if (!pass) return;
        if (mode == VAL_MATERIALIZE) {
            if (pos < q->out_cap) q->out_vals[pos] = __longlong_as_double(static_cast<long long>(vb));
            ++pos;
            return;
        }
        if (mode == VAL_COUNT) { ++agg.cnt; return; }
        if (store && g < q->n_records) {
            if ((g >> 5) != word_idx) { flush(); word_idx = g >> 5; }
            word |= 1u << (g & 31);
        }
        val_agg_add1(agg, vb);
    }
};

// Sequential decode of a whole chunk by one thread (the reader's own loop).
// Returns 0 or the chunk's error.
template <int CODEC>
__device__ uint32_t decode_serial(const uint32_t* fw, uint64_t bit0, uint64_t B, uint64_t* ring, SerialSink& sink) {
    auto peek = [fw, bit0](uint64_t p) { return peek64_file(fw, bit0 + p); };
    if (is_elf(CODEC)) {
        PState s{0, CODEC == CODEC_ELF ? kNoWin : kNoLead};
        uint64_t v = 0;
        int32_t beta = INT32_MAX;
        for (uint64_t i = 0;; ++i) {
            Rec r;
            const uint32_t e = parse_rec<CODEC>(peek, B, s, r);
            if (e) return e;
            v ^= r.delta;
            if (v == kNanBits) return 0;
            if (r.meta & kElfBeta) beta = r.meta & 15;
            const uint64_t out = (r.meta & kElfRestore)
                ? static_cast<uint64_t>(__double_as_longlong(elf_recover(__longlong_as_double(static_cast<long long>(v)), beta, sink.q->dec_tab)))
                : v;
            sink.row(i, out);
        }
    }
    if (B < 64) return EBI_E_UNEXPECTED_END;
    uint64_t v = peek(0);
    PState s{64, CODEC == CODEC_GORILLA ? 0u : kNoLead};
    uint32_t cur = 0;
    if (CODEC == CODEC_CHIMP128) {
        for (int k = 0; k < 128; ++k) ring[k] = 0;
        ring[0] = v;
    }
    bool check = true;
    for (uint64_t i = 0;; ++i) {
        if (check && v == kNanBits) return 0;
        sink.row(i, v);
        Rec r;
        const uint32_t e = parse_rec<CODEC>(peek, B, s, r);
        if (e) return e;
        if (CODEC == CODEC_CHIMP128) {
            v = (r.ring == kRefPrev ? v : ring[r.ring]) ^ r.delta;
            cur = (cur + 1) & 127u;
            ring[cur] = v;
        } else {
            v ^= r.delta;
        }
        check = r.nan_ok;
    }
}

// Elf: vals[0, end) hold the erased values v'; each record flagged
// kElfRestore is replaced by its decimal, with the beta* of the last record
// at or before it that carries kElfBeta (i32::MAX when none does).  Thread t
// takes a contiguous range of records; the block max-scan of "last beta
// record + 1" over the ranges gives each thread the beta* it starts with.
__device__ __noinline__ void elf_restore(Smem sm, uint32_t end, const double* __restrict__ tab, uint32_t* s_red) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t per = (end + kXorThreads - 1) / kXorThreads;
    const uint32_t b = min(end, tid * per), e = min(end, b + per);
    uint32_t last = 0;  // index + 1 of the range's last beta record
    for (uint32_t i = b; i < e; ++i)
        if (sm.meta[i] & kElfBeta) last = i + 1;
    uint32_t inc = last;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc = max(inc, y);
    }
    __syncthreads();  // s_red's previous readers are done
    if (lane == 31) s_red[wid] = inc;
    __syncthreads();
    uint32_t before = __shfl_up_sync(0xffffffffu, inc, 1);
    if (lane == 0) before = 0;
    for (int w = 0; w < wid; ++w) before = max(before, s_red[w]);
    int32_t beta = before ? (sm.meta[before - 1] & 15) : INT32_MAX;
    for (uint32_t i = b; i < e; ++i) {
        const uint8_t m = sm.meta[i];
        if (m & kElfBeta) beta = m & 15;
        if (m & kElfRestore)
            sm.vals[i] = static_cast<uint64_t>(__double_as_longlong(
                elf_recover(__longlong_as_double(static_cast<long long>(sm.vals[i])), beta, tab)));
    }
    __syncthreads();
}

// The control parse of a chunk of B bits by a CTA of kXorThreads threads:
// thread t's segment of the bits starts at a guess (thread 0 at the true first
// record), and each round a thread whose start differs from its predecessor's
// end adopts that end and parses again, until no start up to the first
// failing segment changes.  Out: this thread's converged start, its records
// and first error from there, and the first failing segment (kXorThreads:
// none).  s_in / s_out: kXorThreads words each, s_red: the block reductions'.
template <int CODEC, typename Peek>
__device__ __forceinline__ void converge_segments(Peek peek, uint64_t B, uint64_t* s_in, uint64_t* s_out,
                                                  uint32_t* s_red, PState& in, uint32_t& n, uint32_t& fail,
                                                  uint32_t& first_fail) {
    const int tid = threadIdx.x;
    constexpr uint64_t kFirst = is_elf(CODEC) ? 0 : 64;  // bits before the first parsed record
    const uint64_t span = B - kFirst;
    const uint64_t seg = (span + kXorThreads - 1) / kXorThreads;
    const uint64_t sbeg = kFirst + seg * tid;
    const uint64_t send =
        tid == kXorThreads - 1 ? B : (kFirst + seg * (tid + 1) < B ? kFirst + seg * (tid + 1) : B);
    const bool last = tid == kXorThreads - 1;
    const uint32_t win0 = CODEC == CODEC_GORILLA ? 0u : CODEC == CODEC_ELF ? kNoWin : kNoLead;
    in = PState{tid == 0 ? kFirst : (sbeg < B ? sbeg : B), tid == 0 ? win0 : 0u};
    PState out = parse_segment<CODEC>(peek, B, in, send, last, &n, &fail);
    s_in[tid] = pack_state(in);
    s_out[tid] = pack_state(out);
    first_fail = kXorThreads;
    for (int round = 0; round < kXorThreads; ++round) {
        __syncthreads();
        first_fail = block_min_u32(fail ? static_cast<uint32_t>(tid) : kXorThreads, s_red);
        const bool stale = tid > 0 && s_in[tid] != s_out[tid - 1];
        const uint64_t want = tid > 0 ? s_out[tid - 1] : 0;
        if (!__syncthreads_or(stale && static_cast<uint32_t>(tid) <= first_fail)) break;
        if (stale) {
            in = unpack_state(want);
            out = parse_segment<CODEC>(peek, B, in, send, last, &n, &fail);
            s_in[tid] = want;
            s_out[tid] = pack_state(out);
        }
    }
}


// One Chimp / Chimp128 chunk c by a CTA of kXorThreads threads with
// xor_smem_bytes(CODEC) bytes of dynamic shared memory; li indexes the pass's
// per-chunk counts / offsets.  qs[0, nq) (nq <= 32) are queries over the same
// column: the chunk is decoded once and each query that selects it runs its
// own query phase over the decoded values (a batch's requests on one column
// share the decode).
template <int CODEC>
__device__ __forceinline__ void xor_chunk(const QueryParams* qs, uint32_t nq, uint32_t li, uint32_t c, int mode,
                                          const unsigned long long* chunk_offsets, const SegState* segs = nullptr) {
    static_assert(kSegsPerChunk == kXorThreads, "one converged segment per thread");
    const QueryParams& q = qs[0];  // the column (file, chunk table, tables) of every query
    extern __shared__ __align__(16) uint8_t smem_raw[];
    Smem sm;
    sm.vals = reinterpret_cast<uint64_t*>(smem_raw);
    sm.refs = reinterpret_cast<uint16_t*>(sm.vals + kRcap);
    sm.nanok = reinterpret_cast<uint32_t*>(sm.refs + kRcap);
    sm.meta = reinterpret_cast<uint8_t*>(sm.vals + kRcap);  // Elf (no refs there)
    __shared__ uint64_t s_in[kXorThreads], s_out[kXorThreads];
    __shared__ uint32_t s_red[kXorThreads / 32];
    __shared__ uint64_t s_x[kXorThreads / 32];
    __shared__ ValAgg sh_agg[kXorThreads / 32];
    __shared__ uint32_t s_ok;  // bit k: query k selects the chunk
    __shared__ uint32_t s_status;

    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const ChunkDesc cd = q.chunks[c];
    if (tid == 0) {
        uint32_t okm = 0;
        for (uint32_t k = 0; k < nq; ++k) {
            const QueryParams& qk = qs[k];
            ChunkAcc* ak = qk.acc + c;
            const bool hm = qk.in_mask != nullptr;
            int ok = 1;
            if (mode == VAL_SCAN) {
                ok = hm ? ak->selected != 0 : (qk.chunk_id < 0 || static_cast<uint64_t>(qk.chunk_id) == c);
                if (ok && !hm) ak->selected = 1;
            } else if (mode == VAL_MATERIALIZE) {
                ok = chunk_offsets[li + 1] != chunk_offsets[li];
            } else if (hm) {
                uint32_t any = 0;
                for (uint64_t r = 0; r < cd.n_rows && !any; r += 32) {
                    uint32_t w = mask_word(qk.in_mask, cd.row_off + r, qk.n_records);
                    if (cd.n_rows - r < 32) w &= (1u << (cd.n_rows - r)) - 1u;
                    any = w;
                }
                ok = any != 0;
            }
            if (ok && (cd.flags & kChunkBadGeometry)) { set_status(ak, EBI_E_IO); ok = 0; }
            if (!ok && mode == VAL_COUNT) qk.tile_counts[li] = 0;
            if (ok) okm |= 1u << k;
        }
        s_ok = okm;
        s_status = 0;
    }
    __syncthreads();
    const uint32_t okm = s_ok;
    if (!okm) return;

    const uint64_t B = cd.byte_len * 8;
    const uint32_t* fw = reinterpret_cast<const uint32_t*>(q.file);
    const uint64_t bit0 = cd.byte_off * 8;
    // well-formed chunks hold n_rows + 1 records (the end marker included)
    constexpr bool kElf = is_elf(CODEC);
    constexpr uint64_t kFirst = kElf ? 0 : 64;  // bits before the first parsed record
    const bool parallel = (kElf || B >= 64) && cd.n_rows + 1 < kRcap;

    uint32_t end = 0;         // decoded values (the NaN end marker's index)
    bool serial = !parallel;
    if (parallel) {
        auto peek = [fw, bit0](uint64_t p) { return peek64_file(fw, bit0 + p); };
        PState in;
        uint32_t n, fail, first_fail;
        if (segs) {
            // converged by xor_converge_kernel (the same rounds, run ahead at high occupancy)
            const SegState g = segs[uint64_t(li) * kSegsPerChunk + tid];
            in = unpack_state(g.in);
            n = g.n;
            fail = g.fail;
            first_fail = block_min_u32(fail ? static_cast<uint32_t>(tid) : kXorThreads, s_red);
        } else {
            // The convergence rounds re-read the chunk and each read depends on the
            // previous one: stage the chunk's words (big-endian) in the values
            // array, unused until the extraction, when it fits; else warm L2.
            const uint64_t w0 = cd.byte_off >> 2;
            const uint64_t nwords = ((cd.byte_off + cd.byte_len + 3) >> 2) - w0 + 3;
            const bool staged = nwords <= uint64_t(kRcap) * 2;
            uint32_t* stage = reinterpret_cast<uint32_t*>(sm.vals);
            if (staged) {
                for (uint64_t i = tid; i < nwords; i += kXorThreads) stage[i] = bswap32(__ldg(fw + w0 + i));
                __syncthreads();
            } else {
                for (uint64_t a = (cd.byte_off & ~uint64_t(127)) + uint64_t(tid) * 128; a < cd.byte_off + cd.byte_len;
                     a += uint64_t(kXorThreads) * 128)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(q.file + a));
            }
            const uint64_t sbit0 = (cd.byte_off & 3) * 8;
            auto peek_staged = [stage, sbit0](uint64_t p) { return peek64_be(stage, sbit0 + p); };
            // ---- 1. control parse: segments converge to the sequential parse ---
            if (staged) converge_segments<CODEC>(peek_staged, B, s_in, s_out, s_red, in, n, fail, first_fail);
            else converge_segments<CODEC>(peek, B, s_in, s_out, s_red, in, n, fail, first_fail);
            __syncthreads();  // the staged words are overwritten by the extraction
        }
        // Segments past the first failure hold no records of the stream.
        if (static_cast<uint32_t>(tid) > first_fail) n = 0;
        uint32_t total;
        constexpr uint32_t kHead = kElf ? 0 : 1;  // the first value, outside the segments
        const uint32_t off = kHead + block_excl_scan_u32<kXorThreads>(n, s_red, &total);
        const uint32_t R = kHead + total;  // records before the failure, the first value included
        if (tid == static_cast<int>(first_fail)) s_status = fail;
        // ---- 2. extraction -------------------------------------------------
        if (CODEC == CODEC_CHIMP128)
            for (uint32_t i = tid; i < kRcap / 32; i += kXorThreads) sm.nanok[i] = 0;
        __syncthreads();
        if (tid == 0 && !kElf) {
            sm.vals[0] = peek(0);
            if (CODEC == CODEC_CHIMP128) { sm.refs[0] = kNoRef; atomicOr(&sm.nanok[0], 1u); }
        }
        if (n && off < kRcap) {
            PState s = in;
            Rec r;
            uint32_t idx = off;
            for (uint32_t k = 0; k < n && idx < kRcap; ++k, ++idx) {
                parse_rec<CODEC>(peek, B, s, r);  // succeeds: these records precede the failure
                sm.vals[idx] = r.delta;
                if (kElf) sm.meta[idx] = r.meta;
                if (CODEC == CODEC_CHIMP128) {
                    sm.refs[idx] = static_cast<uint16_t>(r.ring == kRefPrev ? idx - 1 : ring_ref(idx, r.ring));
                    if (r.nan_ok) atomicOr(&sm.nanok[idx >> 5], 1u << (idx & 31));
                }
            }
        }
        __syncthreads();
        const uint32_t Rs = R < kRcap ? R : kRcap;
        // ---- 3. values ----------------------------------------------------
        if (CODEC != CODEC_CHIMP128) {
            // prefix XOR: warp w scans entries [w * per, (w + 1) * per)
            const uint32_t per = ((Rs + kXorThreads / 32 - 1) / (kXorThreads / 32) + 31) & ~31u;
            const uint32_t b = wid * per, e = min(Rs, b + per);
            uint64_t carry = 0;
            for (uint32_t i0 = b; i0 < e; i0 += 32) {
                const uint32_t i = i0 + lane;
                uint64_t v = i < e ? sm.vals[i] : 0;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint64_t y = __shfl_up_sync(0xffffffffu, v, o);
                    if (lane >= o) v ^= y;
                }
                v ^= carry;
                if (i < e) sm.vals[i] = v;
                carry = __shfl_sync(0xffffffffu, v, 31);
            }
            if (lane == 0) s_x[wid] = carry;
            __syncthreads();
            uint64_t pre = 0;
            for (int w = 0; w < wid; ++w) pre ^= s_x[w];
            if (pre)
                for (uint32_t i = b + lane; i < e; i += 32) sm.vals[i] ^= pre;
        } else {
            // pointer jumping: value(i) = acc(i) ^ value(ref(i)), value(kNoRef) = 0.
            // Entries jump in groups; a group reads (acc, ref) pairs between two
            // barriers and writes them between the next two, so every pair read
            // is a consistent jump state and the invariant above holds throughout.
            constexpr int kPer = (kRcap + kXorThreads - 1) / kXorThreads;
            constexpr int kGroup = 11;
            for (int round = 0; round < 20; ++round) {
                bool any = false;
                for (int g0 = 0; g0 < kPer; g0 += kGroup) {
                    uint64_t a[kGroup];
                    uint16_t p[kGroup];
#pragma unroll
                    for (int k = 0; k < kGroup; ++k) {
                        const uint32_t i = tid + (g0 + k) * kXorThreads;
                        p[k] = kNoRef;
                        a[k] = 0;
                        if (g0 + k < kPer && i < Rs) {
                            const uint32_t r = sm.refs[i];
                            if (r != kNoRef) {
                                a[k] = sm.vals[r];
                                p[k] = sm.refs[r];
                                any = true;
                            }
                        }
                    }
                    __syncthreads();
#pragma unroll
                    for (int k = 0; k < kGroup; ++k) {
                        const uint32_t i = tid + (g0 + k) * kXorThreads;
                        if (g0 + k < kPer && i < Rs && sm.refs[i] != kNoRef) {
                            sm.vals[i] ^= a[k];
                            sm.refs[i] = p[k];
                        }
                    }
                    __syncthreads();
                }
                if (!__syncthreads_or(any)) break;
            }
        }
        __syncthreads();
        // ---- end marker ---------------------------------------------------
        uint32_t nan_at = kRcap;
        for (uint32_t i = tid; i < Rs; i += kXorThreads) {
            const bool ok_i = CODEC != CODEC_CHIMP128 || ((sm.nanok[i >> 5] >> (i & 31)) & 1u);
            if (ok_i && sm.vals[i] == kNanBits) { nan_at = i; break; }
        }
        nan_at = block_min_u32(nan_at, s_red);
        if (nan_at < Rs) {
            end = nan_at;
            if (kElf) elf_restore(sm, end, q.dec_tab, s_red);
        } else if (R > kRcap) {
            serial = true;  // the end marker lies past the records held in shared memory
        } else {
            if (tid == 0)
                for (uint32_t k = 0; k < nq; ++k) {
                    if (!((okm >> k) & 1u)) continue;
                    set_status(qs[k].acc + c, s_status ? s_status : EBI_E_UNEXPECTED_END);
                    if (mode == VAL_COUNT) qs[k].tile_counts[li] = 0;
                }
            return;
        }
    }

    if (serial) {
        __syncthreads();
        if (tid == 0)
            for (uint32_t k = 0; k < nq; ++k) {  // each query decodes the chunk again (chunks past kRcap records)
                if (!((okm >> k) & 1u)) continue;
                const QueryParams& qk = qs[k];
                ChunkAcc* ak = qk.acc + c;
                const bool pk = qk.pred_on != 0, sk = mode == VAL_SCAN && pk && qk.out_mask != nullptr;
                SerialSink sink{&qk, cd.row_off, mode, qk.in_mask != nullptr, pk, sk, key_pred(qk.pred),
                                val_agg_init(qk.op == OP_FILTER_AGG || qk.op == OP_AGG ? qk.agg : 0u),
                                mode == VAL_MATERIALIZE ? chunk_offsets[li] : 0ull, 0, 0};
                const uint32_t e = decode_serial<CODEC>(fw, bit0, B, sm.vals, sink);
                if (e) {
                    set_status(ak, e);
                    if (mode == VAL_COUNT) qk.tile_counts[li] = 0;
                } else if (mode == VAL_COUNT) {
                    qk.tile_counts[li] = sink.agg.cnt;
                } else if (mode == VAL_SCAN) {
                    if (sk) sink.flush();
                    val_agg_store(ak, sink.agg);
                }
            }
        return;
    }

    // ---- each selecting query over vals[0, end) ------------------------------
    for (uint32_t k = 0; k < nq; ++k) {
        if (!((okm >> k) & 1u)) continue;
        __syncthreads();  // the previous query's block reduction is read
        const QueryParams& qk = qs[k];
        const bool has_mask = qk.in_mask != nullptr, pred_on = qk.pred_on != 0;
        const bool store = mode == VAL_SCAN && pred_on && qk.out_mask != nullptr;
        const KeyPred kp = key_pred(qk.pred);
        ValAgg agg = val_agg_init(qk.op == OP_FILTER_AGG || qk.op == OP_AGG ? qk.agg : 0u);
        unsigned long long pos = mode == VAL_MATERIALIZE ? chunk_offsets[li] : 0;
        for (uint32_t r0 = 0; r0 < end; r0 += kXorThreads) {
            const uint32_t i = r0 + tid;
            const uint64_t g = cd.row_off + i;
            const bool in = i < end && (!has_mask || mask_row(qk.in_mask, qk.n_records, g));
            const uint64_t vb = in ? sm.vals[i] : 0;
            const bool pass = in && (!pred_on || kp.pass(vb));
            if (mode == VAL_MATERIALIZE) {
                uint32_t total;
                const uint32_t before = block_excl_scan_u32<kXorThreads>(pass, s_red, &total);
                if (pass && pos + before < qk.out_cap) qk.out_vals[pos + before] = __longlong_as_double(static_cast<long long>(vb));
                pos += total;
                continue;
            }
            if (store) {
                const uint32_t word = __ballot_sync(0xffffffffu, pass && g < qk.n_records);
                if (lane == 0 && word) store_mask_word(qk.out_mask, g, word, true);
            }
            if (pass) val_agg_add1(agg, vb);
        }
        if (mode == VAL_MATERIALIZE) continue;
        const ValAgg a = val_agg_block(agg, sh_agg);
        if (tid == 0) {
            if (mode == VAL_COUNT) qk.tile_counts[li] = a.cnt;
            else val_agg_store(qk.acc + c, a);
        }
    }
}

constexpr size_t xor_smem_bytes(int codec) {
    return kRcap * 8 + (codec == CODEC_CHIMP128 ? kRcap * 2 + kRcap / 8 : is_elf(codec) ? kRcap : 0);
}

}  // namespace
}  // namespace ebi
