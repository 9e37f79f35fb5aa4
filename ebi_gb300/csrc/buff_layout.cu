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

// One CTA per segment; every thread writes 16-byte words of the destination,
// assembled from the 4-byte words of the source around them.
__global__ void __launch_bounds__(256) repack_kernel(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst,
                                                     const RepackSeg* __restrict__ segs) {
    const RepackSeg g = segs[blockIdx.x];
    const uint64_t words = (g.len + 15) / 16;
    const uint64_t s0 = g.src_off & ~uint64_t(3);
    const uint32_t sh = static_cast<uint32_t>(g.src_off & 3) * 8;
    const uint32_t* sw = reinterpret_cast<const uint32_t*>(src + s0);
    uint4* dw = reinterpret_cast<uint4*>(dst + g.dst_off);
    for (uint64_t i = threadIdx.x; i < words; i += blockDim.x) {
        const uint32_t* p = sw + 4 * i;
        const uint32_t a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3), e = __ldg(p + 4);
        dw[i] = make_uint4(__funnelshift_r(a, b, sh), __funnelshift_r(b, c, sh), __funnelshift_r(c, d, sh),
                           __funnelshift_r(d, e, sh));
    }
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
        for (uint64_t p = 0; p < np; ++p) segs.push_back({src_planes + p * b.n, at + p * b.stride, b.n});
        at += np * b.stride;
        b.tail = at;
        if (tb) {
            const uint64_t tail_len = (uint64_t(b.n) * tb + 7) / 8;
            segs.push_back({src_tail, at, tail_len});
            at += round_up(round_up(b.n, 64) / 8 * tb, kAlign);
        }
    }
    return at;
}

cudaError_t launch_buff_repack(const uint8_t* src, uint8_t* dst, const RepackSeg* d_segs, uint32_t n_segs,
                               cudaStream_t s) {
    if (n_segs == 0) return cudaSuccess;
    repack_kernel<<<n_segs, 256, 0, s>>>(src, dst, d_segs);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ebi
