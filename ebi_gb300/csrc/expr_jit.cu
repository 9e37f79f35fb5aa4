// expr_jit.cu -- the fused exact Expr pass compiled at run time for the
// programs of a pass.  The interpreter (expr.cu) decodes every instruction
// of every program for every unit of 256 rows, runs 64-bit shifts by
// amounts it learns at run time and reads its values back from shared
// memory; written out, a program is a few integer operations per row on
// registers with constant shifts and literals, expressions that several
// aggregations share (TPC-H Q1's price * (1 - discount)) are computed once,
// and the columns decode at their common widths in 32-bit arithmetic.  The
// walk itself is expr_fused.cuh's text, compiled as is.
//
// NVRTC is opened at first use (dlopen): the library itself does not
// depend on it, and without it the interpreter runs.
#include <dlfcn.h>

#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>

#include <nvrtc.h>

#include "expr_fused.cuh"
#include "expr_prog.h"

namespace ebi {
namespace {

// expr_fused.cuh as text (generated beside the objects at build time).
const char kFusedSource[] =
#include "expr_fused_src.inc"
    ;

constexpr const char* kKernelName = "ebi_expr_fused_jit";

// The C++ of a pass's program object.  It decodes the rows of the columns it
// reads itself, in registers (no packing), in 32-bit arithmetic (every chunk
// of the columns is at most 32 bits wide): at the columns' common chunk
// widths with the plane count and tail width constant, other chunks through
// the general decode.  Aggregation a's value of
// row k is v<a>[k], built from the columns' fixed-point integers c<j> with
// wrapping 64-bit arithmetic, exactly as the interpreter computes it.
std::string program_source(const std::vector<Instr>& prog, const uint32_t* first, const uint32_t* kind,
                           uint32_t n_aggs, uint32_t n_cols, const uint32_t* widths) {
    std::ostringstream body;
    std::vector<bool> used(n_cols, false);
    int tmp = 0;
    for (uint32_t a = 0; a < n_aggs; ++a) {
        std::string acc;
        std::vector<std::string> stack;
        auto operand = [&](uint8_t src, uint16_t col, double lit, uint8_t sh) {
            std::string e;
            if (src == S_COL) {
                e = "c" + std::to_string(col);
                if (col < n_cols) used[col] = true;
            } else if (src == S_LIT) {
                long long n = 0;
                std::memcpy(&n, &lit, sizeof n);
                char buf[32];
                std::snprintf(buf, sizeof buf, "0x%016llxull", static_cast<unsigned long long>(n));
                e = buf;
            } else if (src == S_ACC) {
                e = acc;
            } else {
                e = stack.back();
            }
            if (sh) e = "(" + e + " << " + std::to_string(sh) + ")";
            return e;
        };
        for (uint32_t q = first[a]; q < first[a + 1]; ++q) {
            const Instr& I = prog[q];
            if (I.op == I_PUSH) {
                stack.push_back(acc);
                continue;
            }
            const std::string x = operand(I.a, I.ca, I.la, I.sa);
            if (I.op == I_LOAD) {
                acc = x;
                continue;
            }
            const std::string y = operand(I.b, I.cb, I.lb, I.sb);
            if (I.a == S_POP || I.b == S_POP) stack.pop_back();
            const char* op = I.op == I_ADD ? " + " : I.op == I_SUB ? " - " : " * ";
            const std::string t = "t" + std::to_string(tmp++);
            body << "      const u64 " << t << " = " << x << op << y << ";\n";
            acc = t;
        }
        body << "      v" << a << "[k] = static_cast<i64>(" << acc << ");\n";
    }
    std::vector<uint32_t> U;  // the columns read
    for (uint32_t j = 0; j < n_cols; ++j)
        if (used[j]) U.push_back(j);
    bool fast = !U.empty();
    for (uint32_t j : U) fast = fast && widths[j] >= 1 && widths[j] <= 32;  // else every chunk decodes generally
    auto list = [&](const char* pre, const char* post) {
        std::string l;
        for (size_t i = 0; i < U.size(); ++i) l += (i ? ", " : "") + std::string(pre) + std::to_string(U[i]) + post;
        return l;
    };

    std::ostringstream o;
    o << "namespace ebi_fx {\nstruct Gen {\n  static constexpr bool kPacked = false;\n";
    for (uint32_t a = 0; a < n_aggs; ++a) o << "  Acc A" << a << ";\n";
    o << "  __device__ u32 n_aggs() const { return " << n_aggs << "u; }\n";
    o << "  __device__ void begin() {";
    for (uint32_t a = 0; a < n_aggs; ++a) o << " A" << a << " = acc_rest();";
    o << " }\n";
    o << "  __device__ Acc result(u32 a) const {";
    for (uint32_t a = 0; a + 1 < n_aggs; ++a) o << " if (a == " << a << "u) return A" << a << ";";
    o << " return A" << n_aggs - 1 << "; }\n";
    // eval over the decoded deltas (u32 or u64) and the chunks' bases
    o << "  template <" << list("class D", "") << ">\n";
    o << "  __device__ __forceinline__ void eval(";
    for (uint32_t j : U) o << "const D" << j << " (&d" << j << ")[kRows], i64 b" << j << ", ";
    o << "u32 sel) {\n";
    for (uint32_t a = 0; a < n_aggs; ++a) o << "    i64 v" << a << "[kRows];\n";
    o << "#pragma unroll\n    for (int k = 0; k < kRows; ++k) {\n";
    for (uint32_t j : U)
        o << "      const u64 c" << j << " = static_cast<u64>(b" << j << ") + static_cast<u64>(d" << j << "[k]);\n";
    o << body.str() << "    }\n";
    for (uint32_t a = 0; a < n_aggs; ++a) {
        const char* fn = kind[a] == ebi_fx::kSum ? "acc_sum" : kind[a] == ebi_fx::kMin ? "acc_min" : "acc_max";
        o << "    " << fn << "(A" << a << ", v" << a << ", sel);\n";
    }
    o << "  }\n";
    o << "  __device__ void rows(const ChunkInfo* ci, const unsigned char* const* file, u32 g, u32 sel, u32* bad) {\n";
    o << "    if (";
    for (size_t i = 0; i < U.size(); ++i) o << (i ? " | " : "") << "ci[" << U[i] << "].status";
    o << ") { atomicOr(bad, 1u); return; }\n";
    // every chunk is at most 32 bits wide (the host checks): the deltas fit u32
    auto decode = [&](bool common) {
        o << "      u32 " << list("d", "[kRows]") << ";\n";
        for (uint32_t j : U) {
            if (common)
                o << "      deltas32<" << widths[j] / 8 << ", " << widths[j] % 8 << ">(file[" << j << "], ci[" << j
                  << "], g, d" << j << ");\n";
            else
                o << "      { u64 w[kRows]; deltas(file[" << j << "], ci[" << j << "], g, w);"
                  << " for (int i = 0; i < kRows; ++i) d" << j << "[i] = static_cast<u32>(w[i]); }\n";
        }
        o << "      eval(";
        for (uint32_t j : U) o << "d" << j << ", ci[" << j << "].base, ";
        o << "sel);\n";
    };
    if (fast) {
        o << "    if (";
        for (size_t i = 0; i < U.size(); ++i)
            o << (i ? " && " : "") << "ci[" << U[i] << "].bits == " << widths[U[i]] << "u";
        o << ") {\n";
        decode(true);
        o << "    } else {\n";
        decode(false);
        o << "    }\n";
    } else {
        o << "    {\n";
        decode(false);
        o << "    }\n";
    }
    o << "  }\n};\n}  // namespace ebi_fx\n";
    // 4 CTAs per SM (64 registers) hold up to three columns' deltas and three
    // aggregations without spilling; larger passes take 80 registers
    const int min_blocks = U.size() <= 3 && n_aggs <= 3 ? 4 : 3;
    o << "extern \"C\" __global__ void __launch_bounds__(" << ebi_fx::kThreads << ", " << min_blocks << ") "
      << kKernelName
      << "(ebi_fx::Params F) {\n"
         "  ebi_fx::Gen g;\n"
         "  ebi_fx::fused_walk(F, g, nullptr);\n"
         "  ebi_fx::fused_finish_exact(F, g);\n"
         "}\n";
    return o.str();
}

// NVRTC entry points, resolved once.
struct Nvrtc {
    bool ok = false;
    std::string why;
    nvrtcResult (*create)(nvrtcProgram*, const char*, const char*, int, const char* const*, const char* const*);
    nvrtcResult (*compile)(nvrtcProgram, int, const char* const*);
    nvrtcResult (*log_size)(nvrtcProgram, size_t*);
    nvrtcResult (*log)(nvrtcProgram, char*);
    nvrtcResult (*cubin_size)(nvrtcProgram, size_t*);
    nvrtcResult (*cubin)(nvrtcProgram, char*);
    nvrtcResult (*destroy)(nvrtcProgram*);
};

const Nvrtc& nvrtc() {
    static const Nvrtc N = [] {
        Nvrtc n{};
        void* h = nullptr;
        for (const char* name : {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13"})
            if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL))) break;
        if (!h) {
            n.why = "NVRTC not found (libnvrtc.so.13)";
            return n;
        }
        auto sym = [&](const char* s) { return dlsym(h, s); };
        n.create = reinterpret_cast<decltype(n.create)>(sym("nvrtcCreateProgram"));
        n.compile = reinterpret_cast<decltype(n.compile)>(sym("nvrtcCompileProgram"));
        n.log_size = reinterpret_cast<decltype(n.log_size)>(sym("nvrtcGetProgramLogSize"));
        n.log = reinterpret_cast<decltype(n.log)>(sym("nvrtcGetProgramLog"));
        n.cubin_size = reinterpret_cast<decltype(n.cubin_size)>(sym("nvrtcGetCUBINSize"));
        n.cubin = reinterpret_cast<decltype(n.cubin)>(sym("nvrtcGetCUBIN"));
        n.destroy = reinterpret_cast<decltype(n.destroy)>(sym("nvrtcDestroyProgram"));
        n.ok = n.create && n.compile && n.log_size && n.log && n.cubin_size && n.cubin && n.destroy;
        if (!n.ok) n.why = "NVRTC lacks an entry point";
        return n;
    }();
    return N;
}

struct Compiled {
    cudaKernel_t kernel = nullptr;
    std::string why;  // the failure, when kernel is null
};

// The current device's architecture as an NVRTC option ("-arch=sm_103a"),
// or an empty string when no device answers.
std::string current_arch() {
    int dev = 0, major = 0, minor = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess)
        return std::string();
    return "-arch=sm_" + std::to_string(major * 10 + minor) + "a";
}

// Compiles the walk with a program object for the architecture `arch`.
Compiled compile(const std::string& program, const std::string& arch) {
    Compiled out;
    const Nvrtc& N = nvrtc();
    if (!N.ok) {
        out.why = N.why;
        return out;
    }
    if (arch.empty()) {
        out.why = "no device";
        return out;
    }
    const std::string src = std::string(kFusedSource) + "\n" + program;
    const char* opts[] = {arch.c_str(), "-std=c++17"};
    nvrtcProgram p = nullptr;
    if (N.create(&p, src.c_str(), "ebi_expr_fused_jit.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
        out.why = "nvrtcCreateProgram failed";
        return out;
    }
    std::vector<char> cubin;
    if (N.compile(p, 2, opts) != NVRTC_SUCCESS) {
        size_t n = 0;
        N.log_size(p, &n);
        std::string log(n, '\0');
        if (n) N.log(p, &log[0]);
        out.why = "NVRTC compile failed: " + log.substr(0, 2000);
    } else {
        size_t n = 0;
        if (N.cubin_size(p, &n) == NVRTC_SUCCESS && n) {
            cubin.resize(n);
            if (N.cubin(p, cubin.data()) != NVRTC_SUCCESS) cubin.clear();
        }
        if (cubin.empty()) out.why = "NVRTC produced no cubin";
    }
    N.destroy(&p);
    if (cubin.empty()) return out;
    cudaLibrary_t lib = nullptr;
    cudaError_t e = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&out.kernel, lib, kKernelName);
    if (e != cudaSuccess) {
        out.kernel = nullptr;
        out.why = std::string("loading the compiled pass: ") + cudaGetErrorString(e);
        cudaGetLastError();
    }
    return out;
}

}  // namespace

bool fused_jit_enabled() {
    const char* env = std::getenv("EBI_EXPR_JIT");
    return !(env && std::strcmp(env, "0") == 0) && nvrtc().ok;
}

cudaKernel_t fused_jit_kernel(const std::vector<Instr>& prog, const uint32_t* first, const uint32_t* kind,
                              uint32_t n_aggs, uint32_t n_cols, const uint32_t* widths, std::string* why,
                              bool* required) {
    const char* env = std::getenv("EBI_EXPR_JIT");
    *required = env && std::strcmp(env, "require") == 0;
    if (env && std::strcmp(env, "0") == 0) {
        *why = "off (EBI_EXPR_JIT=0)";
        return nullptr;
    }
    if (n_aggs == 0) {
        *why = "no aggregation";
        return nullptr;
    }
    const std::string program = program_source(prog, first, kind, n_aggs, n_cols, widths);
    // Compiled passes stay loaded for the process (a launch of one may still be
    // in flight on some stream), so the cache is bounded: past kMaxCompiled
    // distinct programs, new ones run on the interpreter.
    constexpr size_t kMaxCompiled = 256;
    static std::mutex mu;
    // keyed by the device architecture too: a cubin runs on the architecture it was built for
    static std::map<std::string, Compiled> cache;
    const std::string arch = current_arch();
    const std::string key = arch + "\n" + program;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it == cache.end()) {
        if (cache.size() >= kMaxCompiled) {
            *why = "compiled-pass cache full";
            return nullptr;
        }
        it = cache.emplace(key, compile(program, arch)).first;
    }
    if (!it->second.kernel) *why = it->second.why;
    return it->second.kernel;
}

}  // namespace ebi
