"""The fused Expr walk (ebi_gb300/csrc/expr_fused.cuh) is compiled twice: by
nvcc into the library, and by NVRTC at run time with a pass's programs written
out (expr_jit.cu).  NVRTC compiles without a GPU, so this CPU test checks that
the header stays self-contained and NVRTC-clean, with a program object of the
shape expr_jit.cu generates (register walk, common-width and general decode,
sum / min / max aggregates)."""
import ctypes as C
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "ebi_gb300" / "csrc" / "expr_fused.cuh"

# The program object for SUM(c0 * ((1 << 8) - c1)) and MAX(c2 - c0), as the
# generator writes it (columns 0..2 at common widths 25, 5 and 14 bits).
PROGRAM = r"""
namespace ebi_fx {
struct Gen {
  static constexpr bool kPacked = false;
  Acc A0;
  Acc A1;
  __device__ u32 n_aggs() const { return 2u; }
  __device__ void begin() { A0 = acc_rest(); A1 = acc_rest(); }
  __device__ Acc result(u32 a) const { if (a == 0u) return A0; return A1; }
  template <class D0, class D1, class D2>
  __device__ __forceinline__ void eval(const D0 (&d0)[kRows], i64 b0, const D1 (&d1)[kRows], i64 b1,
                                       const D2 (&d2)[kRows], i64 b2, u32 sel) {
    i64 v0[kRows];
    i64 v1[kRows];
#pragma unroll
    for (int k = 0; k < kRows; ++k) {
      const u64 c0 = static_cast<u64>(b0) + static_cast<u64>(d0[k]);
      const u64 c1 = static_cast<u64>(b1) + static_cast<u64>(d1[k]);
      const u64 c2 = static_cast<u64>(b2) + static_cast<u64>(d2[k]);
      const u64 t0 = (0x0000000000000001ull << 8) - c1;
      const u64 t1 = c0 * t0;
      v0[k] = static_cast<i64>(t1);
      const u64 t2 = c2 - c0;
      v1[k] = static_cast<i64>(t2);
    }
    acc_sum(A0, v0, sel);
    acc_max(A1, v1, sel);
  }
  __device__ void rows(const ChunkInfo* ci, const unsigned char* const* file, u32 g, u32 sel, u32* bad) {
    if (ci[0].status | ci[1].status | ci[2].status) { atomicOr(bad, 1u); return; }
    if (ci[0].bits == 25u && ci[1].bits == 5u && ci[2].bits == 14u) {
      u32 d0[kRows], d1[kRows], d2[kRows];
      deltas32<3, 1>(file[0], ci[0], g, d0);
      deltas32<0, 5>(file[1], ci[1], g, d1);
      deltas32<1, 6>(file[2], ci[2], g, d2);
      eval(d0, ci[0].base, d1, ci[1].base, d2, ci[2].base, sel);
    } else {
      u32 d0[kRows], d1[kRows], d2[kRows];
      { u64 w[kRows]; deltas(file[0], ci[0], g, w); for (int i = 0; i < kRows; ++i) d0[i] = static_cast<u32>(w[i]); }
      { u64 w[kRows]; deltas(file[1], ci[1], g, w); for (int i = 0; i < kRows; ++i) d1[i] = static_cast<u32>(w[i]); }
      { u64 w[kRows]; deltas(file[2], ci[2], g, w); for (int i = 0; i < kRows; ++i) d2[i] = static_cast<u32>(w[i]); }
      eval(d0, ci[0].base, d1, ci[1].base, d2, ci[2].base, sel);
    }
  }
};
}  // namespace ebi_fx
extern "C" __global__ void __launch_bounds__(256, 4) ebi_expr_fused_jit(ebi_fx::Params F) {
  ebi_fx::Gen g;
  ebi_fx::fused_walk(F, g, nullptr);
  ebi_fx::fused_finish_exact(F, g);
}
"""


def _nvrtc():
    for name in ("libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    return None


def test_fused_walk_compiles_with_nvrtc():
    lib = _nvrtc()
    if lib is None:
        pytest.skip("NVRTC is not installed here")
    src = (HEADER.read_text() + "\n" + PROGRAM).encode()
    prog = C.c_void_p()
    assert lib.nvrtcCreateProgram(C.byref(prog), src, b"ebi_expr_fused_jit.cu", 0, None, None) == 0
    opts = (C.c_char_p * 2)(b"-arch=sm_103a", b"-std=c++17")
    rc = lib.nvrtcCompileProgram(prog, 2, opts)
    n = C.c_size_t()
    lib.nvrtcGetProgramLogSize(prog, C.byref(n))
    log = C.create_string_buffer(n.value + 1)
    lib.nvrtcGetProgramLog(prog, log)
    size = C.c_size_t()
    lib.nvrtcGetCUBINSize(prog, C.byref(size))
    lib.nvrtcDestroyProgram(C.byref(prog))
    assert rc == 0, log.value.decode(errors="replace")
    assert size.value > 0, "NVRTC produced no cubin"
