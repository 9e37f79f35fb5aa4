// Host harness of the XOR decoders' control parse (xor_parse.cuh compiled for
// the host), driven by tests/test_cpu_converge.py.  For each chunk file given
// as "<codec> <segments> <path>" on stdin it runs the record parse in order
// from the first record, and an emulation of the chunk kernel's convergence
// rounds (converge_segments in xor_dev.cuh: thread t of T guesses a start in
// its share of the bits; each round a start that differs from the previous
// segment's end adopts it and parses again).  Prints one line per chunk:
//   <records in order> <records over the converged segments> <starts off the true path> <rounds>
#include <cstdio>
#include <set>
#include <vector>

#include "../ebi_gb300/csrc/xor_parse.cuh"

using namespace ebi::xorp;

struct Peek {
    const uint8_t* b;
    uint64_t operator()(uint64_t p) const {  // 64 bits from bit p, MSB first
        const uint64_t byte = p >> 3;
        const uint32_t sh = p & 7;
        uint64_t hi = 0;
        for (int i = 0; i < 8; ++i) hi = (hi << 8) | b[byte + i];
        return sh ? (hi << sh) | (b[byte + 8] >> (8 - sh)) : hi;
    }
};

template <int CODEC>
uint32_t step(Peek& pk, uint64_t B, PState& s) {
    if (CODEC == CODEC_CHIMP || CODEC == CODEC_CHIMP128) return step_len<CODEC>(pk, B, s);
    Rec r;
    return parse_rec<CODEC>(pk, B, s, r);
}

template <int CODEC>
void run(const std::vector<uint8_t>& buf, uint64_t len, int T) {
    Peek peek{buf.data()};
    const uint64_t B = len * 8;
    const uint64_t kFirst = is_elf(CODEC) ? 0 : 64;
    const uint32_t win0 = CODEC == CODEC_ELF ? kNoWin : kNoLead;
    // the reader's order: every record start up to the first failing record
    std::set<uint64_t> path;
    uint64_t records = 0;
    for (PState s{kFirst, win0}; s.pos < B;) {
        path.insert(pack_state(s));
        if (step<CODEC>(peek, B, s)) break;
        ++records;
    }
    // the rounds
    const uint64_t span = B - kFirst, seg = (span + T - 1) / T;
    std::vector<PState> in(T), out(T);
    std::vector<uint32_t> n(T), fail(T);
    std::vector<uint64_t> send(T);
    for (int t = 0; t < T; ++t) {
        const uint64_t sb = kFirst + seg * t;
        send[t] = t == T - 1 ? B : (kFirst + seg * (t + 1) < B ? kFirst + seg * (t + 1) : B);
        in[t] = t == 0 ? PState{kFirst, win0} : PState{sb < B ? sb : B, 0u};
        out[t] = parse_segment<CODEC>(peek, B, in[t], send[t], t == T - 1, &n[t], &fail[t]);
    }
    int rounds = 0, first_fail = T;
    for (int r = 0; r < T; ++r) {
        first_fail = T;
        for (int t = 0; t < T; ++t)
            if (fail[t]) { first_fail = t; break; }
        std::vector<uint64_t> want(T);
        bool any = false;
        for (int t = 1; t < T; ++t) {
            want[t] = pack_state(out[t - 1]);
            if (pack_state(in[t]) != want[t] && t <= first_fail) any = true;
        }
        if (!any) break;
        ++rounds;
        for (int t = 1; t < T; ++t)
            if (pack_state(in[t]) != want[t]) {
                in[t] = unpack_state(want[t]);
                out[t] = parse_segment<CODEC>(peek, B, in[t], send[t], t == T - 1, &n[t], &fail[t]);
            }
    }
    uint64_t total = 0, off_path = 0;
    for (int t = 0; t <= first_fail && t < T; ++t) {
        total += n[t];
        if (in[t].pos < B && !path.count(pack_state(in[t]))) ++off_path;
    }
    std::printf("%llu %llu %llu %d\n", (unsigned long long)records, (unsigned long long)total,
                (unsigned long long)off_path, rounds);
}

int main() {
    int codec, T;
    char path[4096];
    while (std::scanf("%d %d %4095s", &codec, &T, path) == 3) {
        FILE* f = std::fopen(path, "rb");
        if (!f) return 1;
        std::vector<uint8_t> buf;
        for (int ch; (ch = std::fgetc(f)) != EOF;) buf.push_back(static_cast<uint8_t>(ch));
        std::fclose(f);
        const uint64_t len = buf.size();
        buf.resize(len + 32, 0);
        switch (codec) {
        case CODEC_CHIMP: run<CODEC_CHIMP>(buf, len, T); break;
        case CODEC_CHIMP128: run<CODEC_CHIMP128>(buf, len, T); break;
        case CODEC_ELF_CHIMP: run<CODEC_ELF_CHIMP>(buf, len, T); break;
        case CODEC_ELF: run<CODEC_ELF>(buf, len, T); break;
        default: return 2;
        }
        std::fflush(stdout);
    }
    return 0;
}
