// Host harness of the value-codec fold's fixed-point helpers (finalize.cuh),
// driven by tests/test_cpu_fold.py.  stdin lines:
//   "s n b1 .. bn"   -> the fold of n f64 terms (hex bits) at their largest
//                       exponent field: result bits and that field
//   "r w0 w1 w2 n"   -> floor(W / 2^n) of the signed 192-bit W
#include <cstdio>
#include <vector>

#include "../ebi_gb300/csrc/finalize.cuh"

using namespace ebi;

int main() {
    char op;
    while (std::scanf(" %c", &op) == 1) {
        if (op == 'r') {
            unsigned long long w0, w1, w2;
            unsigned n;
            if (std::scanf("%llx %llx %llx %u", &w0, &w1, &w2, &n) != 4) return 1;
            const Wide r = wide_sar(Wide{w0, w1, w2}, n);
            std::printf("%016llx %016llx %016llx\n", r.w0, r.w1, r.w2);
            continue;
        }
        int n;
        if (std::scanf("%d", &n) != 1) return 1;
        std::vector<unsigned long long> b(n);
        for (auto& x : b)
            if (std::scanf("%llx", &x) != 1) return 1;
        uint32_t T = 0;
        for (auto x : b) T = T > term_top(x) ? T : term_top(x);
        Wide w{0, 0, 0};
        for (auto x : b) w = wide_add(w, term_wide(x, T));
        const double d = wide_to_f64(w, static_cast<int>(T) - 1172);
        unsigned long long o;
        std::memcpy(&o, &d, 8);
        std::printf("%016llx %u\n", o, T);
    }
    return 0;
}
