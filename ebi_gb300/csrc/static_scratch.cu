// static_scratch.cu -- fixed device scratch for ebi_materialize_static.
//
// The per-tile counts and offsets of a materialize live in one file-scope
// __device__ array instead of memory allocated on first use, so that entry
// point allocates nothing.  Its limit is kStaticTiles tiles per call.  The
// array's address is looked up once per device (cudaGetSymbolAddress with
// that device current) and cached.  Every call that uses it shares it: calls
// that overlap in time (other streams, other host threads) race on it.
#include <mutex>

#include "internal.h"

namespace ebi {
namespace {

// counts [0, kStaticTiles), offsets [kStaticTiles, 2 * kStaticTiles + 1)
static __device__ __align__(256) unsigned long long g_static_scratch[2 * kStaticTiles + 2];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned long long* g_addr[kMaxDevices] = {};

}  // namespace

cudaError_t static_scratch(unsigned long long** counts, unsigned long long** offsets) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = static_cast<unsigned long long*>(p);
    }
    *counts = g_addr[dev];
    *offsets = g_addr[dev] + kStaticTiles;
    return cudaSuccess;
}

}  // namespace ebi
