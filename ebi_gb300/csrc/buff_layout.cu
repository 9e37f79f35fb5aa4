// buff_layout.cu -- the device layout of BUFF columns.
//
// In the file a chunk is a 20-byte header, bits/8 byte planes of n bytes and a
// tail plane, packed back to back from an arbitrary byte offset.  In HBM the
// engine keeps only the planes, each starting on a 128-byte boundary, planes
// of a chunk round_up(n, 128) bytes apart, the tail plane padded to whole
// 64-row groups (8 * tb bytes each) and to 16 bytes.  Every 16-byte load of
// a scan kernel is then aligned, and a group of 64 rows owns exactly 64 bytes
// of each plane and 8 * tb bytes of tail.  The header facts travel in
// BuffChunkInfo; chunks whose header or length is bad keep no bytes (reading
// them raises their status).  The repack runs once, on the device, at open.
#include "internal.h"

namespace ebi {
namespace {

constexpr uint64_t kAlign = 128;
inline uint64_t round_up(uint64_t x, uint64_t a) { return (x + a - 1) / a * a; }

constexpr uint32_t kRepackThreads = 256;
constexpr uint32_t kRepackUnroll = 4;  // source loads in flight per thread

// One CTA per repack block (at most kRepackWords 16-byte destination words
// of one segment).  Word i of a segment is 16 source bytes from an arbitrary
// offset: the bytes of two aligned 16-byte source blocks.  Each thread loads
// one block per word and takes the next from its neighbour lane (lane 31
// loads it itself), four words in flight at a time, so every source byte
// crosses the bus about once -- the source may be pinned host memory read
// over the host link, which then bounds the repack.
__global__ void __launch_bounds__(kRepackThreads) repack_kernel(const uint8_t* __restrict__ src,
                                                                uint8_t* __restrict__ dst,
                                                                const RepackSeg* __restrict__ blocks_in) {
    const RepackSeg g = blocks_in[blockIdx.x];  // src_off / dst_off of the block's first word, len in words
    const uint64_t words = g.len;
    const uintptr_t first = reinterpret_cast<uintptr_t>(src + g.src_off);
    const uint4* blocks = reinterpret_cast<const uint4*>(first & ~uintptr_t(15));
    const uint32_t q = static_cast<uint32_t>(first & 15) >> 2, sh = static_cast<uint32_t>(first & 3) * 8;
    const bool misaligned = (first & 15) != 0;
    const uint32_t lane = threadIdx.x & 31;
    uint4* dw = reinterpret_cast<uint4*>(dst + g.dst_off);
    for (uint64_t i0 = 0; i0 < words; i0 += kRepackThreads * kRepackUnroll) {
        uint4 lo[kRepackUnroll];
#pragma unroll
        for (uint32_t u = 0; u < kRepackUnroll; ++u) {
            const uint64_t i = i0 + u * kRepackThreads + threadIdx.x;
            lo[u] = i < words ? blocks[i] : make_uint4(0, 0, 0, 0);
        }
#pragma unroll
        for (uint32_t u = 0; u < kRepackUnroll; ++u) {
            const uint64_t i = i0 + u * kRepackThreads + threadIdx.x;
            uint4 hi;
            hi.x = __shfl_down_sync(0xffffffffu, lo[u].x, 1);
            hi.y = __shfl_down_sync(0xffffffffu, lo[u].y, 1);
            hi.z = __shfl_down_sync(0xffffffffu, lo[u].z, 1);
            hi.w = __shfl_down_sync(0xffffffffu, lo[u].w, 1);
            if (i >= words) continue;
            if (misaligned && (lane == 31 || i + 1 >= words)) hi = blocks[i + 1];
            const uint32_t w[8] = {lo[u].x, lo[u].y, lo[u].z, lo[u].w, hi.x, hi.y, hi.z, hi.w};
            uint32_t o[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t a = q == 0 ? w[j] : q == 1 ? w[j + 1] : q == 2 ? w[j + 2] : w[j + 3];
                const uint32_t b = q == 0 ? w[j + 1] : q == 1 ? w[j + 2] : q == 2 ? w[j + 3] : w[j + 4];
                o[j] = __funnelshift_r(a, b, sh);
            }
            dw[i] = make_uint4(o[0], o[1], o[2], o[3]);
        }
    }
}

}  // namespace

namespace {
constexpr uint64_t kRepackWords = 4096;  // 16-byte words per repack block (64 KB)

// Appends the copy of len bytes as blocks of whole 16-byte destination words.
void add_copy(std::vector<RepackSeg>& blocks, uint64_t src_off, uint64_t dst_off, uint64_t len) {
    const uint64_t words = (len + 15) / 16;
    for (uint64_t w = 0; w < words; w += kRepackWords)
        blocks.push_back({src_off + 16 * w, dst_off + 16 * w, words - w < kRepackWords ? words - w : kRepackWords});
}
}  // namespace

uint64_t buff_plan_layout(std::vector<BuffChunkInfo>& info, std::vector<RepackSeg>& segs) {
    uint64_t at = 0;
    for (BuffChunkInfo& b : info) {
        if (b.status || b.bits == 0) {  // nothing to read: a bad chunk, or a constant one (bits 0)
            b.planes = b.tail = 0;
            b.stride = 0;
            continue;
        }
        const uint64_t np = b.bits / 8, tb = b.bits % 8;
        const uint64_t src_planes = b.planes, src_tail = b.tail;  // file offsets, from the header parse
        b.stride = round_up(b.n, kAlign);
        b.planes = at;
        for (uint64_t p = 0; p < np; ++p) add_copy(segs, src_planes + p * b.n, at + p * b.stride, b.n);
        at += np * b.stride;
        b.tail = at;
        if (tb) {
            const uint64_t tail_len = (uint64_t(b.n) * tb + 7) / 8;
            add_copy(segs, src_tail, at, tail_len);
            at += round_up(round_up(b.n, 64) / 8 * tb, kAlign);
        }
    }
    return at;
}

cudaError_t launch_buff_repack(const uint8_t* src, uint8_t* dst, const RepackSeg* d_segs, uint32_t n_segs,
                               cudaStream_t s) {
    if (n_segs == 0) return cudaSuccess;
    repack_kernel<<<n_segs, kRepackThreads, 0, s>>>(src, dst, d_segs);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ebi
