// elf_tables.cu -- the decimal tables of elf_dev.cuh, one copy per device.
//
// Built on the host once per process: powers of ten from the decimal strings
// the reference parses, and the boundaries of floor(log10(v)) found by
// bisection over the bit patterns of positive doubles with the host C
// library's log10 (the function the reference's get_sp calls).  Uploaded to a
// file-scope __device__ array on first use per device (at column open).
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "elf_dev.cuh"
#include "elf_host.h"
#include "internal.h"

namespace ebi {
namespace {

static __device__ __align__(16) double g_elf_tab[kElfTabLen];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
const double* g_addr[kMaxDevices] = {};

double from_bits(uint64_t b) {
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}

// floor(log10(v)) >= k for the positive double with bits b
bool at_least(uint64_t b, int32_t k) { return elf::sat_i32(std::floor(std::log10(from_bits(b)))) >= k; }

std::vector<double> build_table() {
    std::vector<double> t(kElfTabLen);
    for (uint32_t i = 0; i < kElfNP10; ++i) t[kElfP10 + i] = elf::pow10_pos(i);
    for (uint32_t i = 0; i < kElfNN10; ++i) t[kElfN10 + i] = elf::pow10_neg(i);
    const uint64_t kInf = 0x7ff0000000000000ull;
    for (int32_t k = kElfSpMin; k <= kElfSpMax; ++k) {
        uint64_t lo = 1, hi = kInf - 1;  // least b in [1, inf) with at_least(b, k)
        if (!at_least(lo, k)) {
            while (hi - lo > 1) {
                const uint64_t mid = lo + (hi - lo) / 2;
                if (at_least(mid, k)) hi = mid;
                else lo = mid;
            }
            lo = hi;
        }
        t[kElfSpB + (k - kElfSpMin)] = from_bits(lo);
    }
    return t;
}

}  // namespace

cudaError_t elf_tables(const double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        static const std::vector<double> host = build_table();
        e = cudaMemcpyToSymbol(g_elf_tab, host.data(), host.size() * sizeof(double));
        if (e != cudaSuccess) return e;
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_elf_tab);
        if (e != cudaSuccess) return e;
        g_addr[dev] = static_cast<const double*>(p);
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

}  // namespace ebi
