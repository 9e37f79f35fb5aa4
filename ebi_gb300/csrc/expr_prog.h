// expr_prog.h -- the accumulator code an Expr compiles to (expr.cu), and the
// run-time compiled form of the fused exact pass over it (expr_jit.cu).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace ebi {

// One instruction: acc = a OP b (LOAD: acc = a; PUSH: push acc).
enum : uint8_t { I_LOAD = 0, I_PUSH = 1, I_ADD = 2, I_SUB = 3, I_MUL = 4, I_DIV = 5 };
enum : uint8_t { S_ACC = 0, S_POP = 1, S_COL = 2, S_LIT = 3 };
struct Instr {
    uint8_t op, a, b;
    uint8_t sa, sb;     // exact BUFF programs: left shifts aligning the operands' scales
    uint8_t pad[3];
    uint16_t ca, cb;    // column slot of an S_COL operand (a column index until a pass assigns slots)
    uint16_t pad2[2];
    double la, lb;      // literal of an S_LIT operand (exact programs: its integer numerator's bits)
};

// The fused exact pass (expr_fused.cuh) with the programs of a pass written
// out as straight-line code and compiled for this device at run time:
// aggregation a runs prog[first[a], first[a + 1]) (integer form: shifts,
// literal numerators) and has kind kind[a]; every chunk of the columns is at
// most 32 bits wide, and widths[j] is the common chunk width of column slot j
// (1..32: its chunks decode with constant plane counts).
// The kernel takes ebi_fx::Params and no dynamic shared memory.  Kernels are
// cached by their source.  Returns null, with the reason in *why, when
// run-time compilation is off (EBI_EXPR_JIT=0) or unavailable; *required is
// set when EBI_EXPR_JIT=require asks that a failure be an error.
// Whether exact passes may be compiled at run time here (NVRTC found, not
// switched off); a later compile can still fail.
bool fused_jit_enabled();

cudaKernel_t fused_jit_kernel(const std::vector<Instr>& prog, const uint32_t* first, const uint32_t* kind,
                              uint32_t n_aggs, uint32_t n_cols, const uint32_t* widths, std::string* why,
                              bool* required);

}  // namespace ebi
