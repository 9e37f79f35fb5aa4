// gorilla.cu -- kernel and launcher of the Gorilla chunk pass (gorilla_dev.cuh).
//
// One CTA of three warps per chunk.  Warp 0 brings the chunk into shared
// memory by one bulk copy (cp.async.bulk, completed on an mbarrier with a
// bounded wait; chunks above the staging size are read through L1 from the
// resident file instead) and parses the stream; its parse steps' values (up
// to 32 per step, one per lane) go, kSub steps per slot, through a ring of
// kRing slots in shared memory to warps 1 and 2, which apply the query: warp 1
// the bitmask, counts, min / max and materialized values, warp 2 the
// compensated sums.  Neither the parse nor the FP64 sums wait for the rest of
// the query's work.  Both query warps give step values to lanes exactly as the
// one-warp walk does (value i of a step to lane i) and warp 1 takes warp 2's
// per-lane sums before the warp reduction, so every per-lane running value,
// and the result, is the same as the batched path's walk.  Slots are handed
// over with full / empty mbarriers (every lane arrives: each releases its own
// writes or reads); every wait is bounded and a wait that runs out ends the
// chunk with EBI_E_CUDA.
#include "internal.h"
#include "gorilla_dev.cuh"

namespace ebi {
namespace {

constexpr int kRing = 4;
constexpr int kSub = 8;             // parse steps per slot
constexpr uint32_t kEnd = 1u << 8;  // meta: the parse is over; status in bits 16..

struct __align__(16) GorillaRing {
    uint64_t full[kRing];
    uint64_t empty[kRing];
    uint64_t sums_ready;         // warp 2's per-lane sums are in hi / lo
    double hi[32], lo[32];
    uint32_t meta[kRing][kSub];  // k | kEnd | status << 16
    uint32_t nsub[kRing];        // steps in the slot
    uint32_t ok;                 // the chunk is read by this pass
    uint32_t pad[3];
    uint64_t vals[kRing][kSub][32];
};
constexpr size_t kRingOff = 16;  // after the bulk copy's mbarrier
constexpr size_t kStageOff = kRingOff + sizeof(GorillaRing);
static_assert(kStageOff % 16 == 0, "bulk copies land on 16-byte boundaries");

__global__ void __launch_bounds__(96) gorilla_kernel(QueryParams q, uint32_t chunk_base, int mode,
                                                     const unsigned long long* chunk_offsets) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t li = blockIdx.x;
    const uint32_t c = chunk_base + li;
    extern __shared__ __align__(16) uint8_t smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
    GorillaRing* R = reinterpret_cast<GorillaRing*>(smem + kRingOff);
    if (warp == 0) {
        const bool ok = gorilla_begin(q, li, c, mode, chunk_offsets);  // warp-collective
        if (lane == 0) {
            R->ok = ok ? 1u : 0u;
            for (int i = 0; i < kRing; ++i) {
                mbar_init(&R->full[i], 32);
                mbar_init(&R->empty[i], 64);
            }
            mbar_init(&R->sums_ready, 32);
            mbar_init(bar, 1);
            fence_mbar_init();
        }
    }
    __syncthreads();
    if (!R->ok) return;
    const ChunkDesc cd = q.chunks[c];

    if (warp == 0) {
        // ---- parse: kSub steps into each ring slot ---------------------------
        uint32_t n = 0;       // slots published
        uint32_t sub = 0;     // steps in the slot being filled
        uint32_t s = 0;       // that slot
        bool broken = false;  // a wait for a free slot ran out: the rest is dropped
        auto put = [&](uint32_t k, uint64_t v, uint32_t flags) {
            if (broken) return;
            if (sub == 0) {
                s = n % kRing;
                if (n >= kRing && !__all_sync(kFull, mbar_wait(&R->empty[s], ((n / kRing) - 1) & 1))) {
                    broken = true;
                    if (lane == 0) set_status(q.acc + c, EBI_E_CUDA);
                    return;
                }
            }
            R->vals[s][sub][lane] = v;
            if (lane == 0) R->meta[s][sub] = k | flags;
            if (++sub == kSub || (flags & kEnd)) {
                if (lane == 0) R->nsub[s] = sub;
                mbar_arrive(&R->full[s]);
                ++n;
                sub = 0;
            }
        };
        const uint64_t span = stage_span(cd.byte_off, cd.byte_len);
        uint32_t status;
        if (span <= q.stage_bytes) {
            const uint8_t* src = q.file + (cd.byte_off & ~uint64_t(15));
            if (lane == 0) {
                mbar_arrive_expect_tx(bar, static_cast<uint32_t>(span));
                bulk_g2s(smem + kStageOff, src, static_cast<uint32_t>(span), bar);
            }
            __syncwarp();
            if (!__all_sync(kFull, mbar_wait(bar, 0, q.copy_wait))) {
                mbar_wait(bar, 0);  // a second wait (full limit) before the CTA leaves
                status = EBI_E_CUDA;
            } else {
                const uint32_t* stage = reinterpret_cast<const uint32_t*>(smem + kStageOff);
                const uint64_t bit0 = (cd.byte_off & 15) * 8;
                status = parse_stream(cd.byte_len * 8, [stage, bit0](uint64_t p) { return peek64_le_smem(stage, bit0 + p); },
                                      [&](uint32_t k, uint64_t v) { put(k, v, 0u); });
            }
        } else {
            const uint32_t* fw = reinterpret_cast<const uint32_t*>(q.file);
            const uint64_t bit0 = cd.byte_off * 8;
            status = parse_stream(cd.byte_len * 8, [fw, bit0](uint64_t p) { return peek64_file(fw, bit0 + p); },
                                  [&](uint32_t k, uint64_t v) { put(k, v, 0u); });
        }
        put(0u, 0ull, kEnd | (status << 16));
        return;
    }

    // ---- query: the ring's steps in order (warp 1: all but the sums; warp 2: the sums)
    const bool sums = warp == 2;
    WalkSink<1, kPartNoSum> sink;
    WalkSink<1, kPartSum> sum_sink;
    if (sums) sum_sink.init(&q, 1, 1u, cd, li, mode, chunk_offsets);
    else sink.init(&q, 1, 1u, cd, li, mode, chunk_offsets);
    uint32_t status = 0;
    for (uint32_t n = 0;; ++n) {
        const uint32_t s = n % kRing;
        if (!__all_sync(kFull, mbar_wait(&R->full[s], (n / kRing) & 1))) {
            status = EBI_E_CUDA;
            break;
        }
        // the slot's steps into registers, then the slot goes back to the parse
        const uint32_t ns = R->nsub[s];
        uint32_t meta[kSub];
        uint64_t v[kSub];
#pragma unroll
        for (int j = 0; j < kSub; ++j) {
            meta[j] = R->meta[s][j];
            v[j] = R->vals[s][j][lane];
        }
        mbar_arrive(&R->empty[s]);
        bool end = false;
#pragma unroll
        for (int j = 0; j < kSub; ++j) {
            if (end || static_cast<uint32_t>(j) >= ns) break;
            if (meta[j] & kEnd) {
                status = meta[j] >> 16;
                end = true;
                break;
            }
            if (sums) sum_sink.apply(meta[j] & 0xffu, v[j]);
            else sink.apply(meta[j] & 0xffu, v[j]);
        }
        if (end) break;
    }
    if (sums) {
        // hand the per-lane sums to warp 1 (nothing to hand over after a failure)
        if (!status) {
            R->hi[lane] = sum_sink.agg[0].hi;
            R->lo[lane] = sum_sink.agg[0].lo;
            mbar_arrive(&R->sums_ready);
        }
        return;
    }
    if (!status && mode == VAL_SCAN) {
        if (__all_sync(kFull, mbar_wait(&R->sums_ready, 0))) {
            sink.agg[0].hi = R->hi[lane];
            sink.agg[0].lo = R->lo[lane];
        } else {
            status = EBI_E_CUDA;
        }
    }
    if (status) sink.fail(c, li, status);
    else sink.finish(c, li);
}

}  // namespace

uint32_t gorilla_stage_bytes(const ChunkDesc* chunks, uint64_t n) {
    uint64_t mx = 0;
    for (uint64_t i = 0; i < n; ++i) {
        if (chunks[i].flags & kChunkBadGeometry) continue;
        const uint64_t sp = stage_span(chunks[i].byte_off, chunks[i].byte_len);
        if (sp <= kGorillaStageCap && sp > mx) mx = sp;
    }
    return static_cast<uint32_t>(mx);
}

cudaError_t launch_gorilla(const QueryParams& q, uint32_t chunk_begin, uint32_t n_chunks, int mode,
                           const unsigned long long* chunk_offsets, cudaStream_t s) {
    if (n_chunks == 0) return cudaSuccess;
    const size_t smem = kStageOff + size_t(q.stage_bytes);
    const cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void*>(gorilla_kernel), smem);
    if (e != cudaSuccess) return e;
    gorilla_kernel<<<n_chunks, 96, smem, s>>>(q, chunk_begin, mode, chunk_offsets);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ebi
