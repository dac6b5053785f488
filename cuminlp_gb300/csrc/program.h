// program.h -- the fused evaluator's instruction set, shared by the host
// compiler (program.cpp) and the device interpreter (eval_core.cuh).
//
// A problem's expression DAG (model/dag.hpp:58-93 in the reference) is
// compiled once into a straight-line program over three kinds of storage:
//
//   VAR    the box's own variable intervals, staged per thread in shared
//          memory (the child box decoded from its parent in the kernel
//          prologue);
//   SLOT   a shared-memory value slot, allocated by liveness so that a
//          value occupies a slot only between its definition and last use;
//   ACC    one register-resident accumulator that carries the running sum
//          of a sum chain (sum_k c_k * x_i * x_j ...) without touching
//          shared memory.
//
// The reference evaluates every DAG node with its own kernel and a full
// HBM round trip per node (graph/builder.cuh:261-514); here a node's value
// lives in a register or in shared memory, and only the box goes in and
// the verdict comes out.  Every instruction performs exactly the rounding
// steps of the DAG nodes it stands for, in the same order, so the
// enclosures are bit-identical to node-by-node evaluation.
#pragma once

#include <cstdint>

namespace cmn {

enum OperandMode : uint8_t {
  kModeSlot = 0,
  kModeVar = 1,
  kModeAcc = 2,
  kModeConst = 3,
};

enum Opcode : uint8_t {
  // generic node: dst slot <- op(a, b)
  kOpGeneric = 0,
  // fused sum-chain term: acc <- acc (+|-) [c *] P,   P in {x_a*x_b,
  // sqr(x_a), x_a}; or acc <- [c *] P when kTermInit is set
  kOpTerm = 1,
  // slot <- acc
  kOpStoreAcc = 2,
  // acc <- operand a
  kOpLoadAcc = 3,
  // slot <- constant c (as a point interval / outward FP32 interval)
  kOpConstToSlot = 4,
  // feasibility of one constraint root: flag &= (lb <= rhs) [LE] or
  // (lb <= rhs <= ub) [EQ]; rhs in c
  kOpCheck = 5,
  // objective root: obj <- operand a
  kOpObjective = 6,
};

// node ops understood by kOpGeneric (values of cmn_op)
enum GenericOp : uint8_t {
  kGAdd = 2,
  kGSub = 3,
  kGMul = 4,
  kGDiv = 5,
  kGSqr = 6,
  kGNeg = 7,
  kGExp = 8,
  kGLog = 9,
  kGSqrt = 10,
  kGSin = 11,
  kGCos = 12,
  kGTanh = 13,
  kGPowN = 14,
  kGPow = 15,
  kGAbs = 16,
  kGMin = 17,
  kGMax = 18,
};

// kOpTerm flags (the sub-code of a term instruction)
enum TermFlags : uint8_t {
  kTermInit = 1,     // acc <- t   (start of a chain)
  kTermSub = 2,      // acc <- acc - t
  kTermHasC = 4,     // t = c * P
  kTermProd = 0,     // P = x_a * x_b      (bits 3-4)
  kTermSqr = 8,      // P = sqr(x_a)
  kTermVar = 16,     // P = x_a
  kTermPMask = 24,
};

// 16 bytes.  `head` packs the Opcode (bits 0-2) with its sub-code (bits
// 3-7: the GenericOp, the TermFlags, or the Cmp of a check).  For FP64
// programs `c` is the payload; for FP32 programs the same bytes hold the
// outward-rounded pair (clo, chi).
struct Instr {
  uint8_t head;
  uint8_t modes;  // bits 0-1 mode of a, bits 2-3 mode of b
  uint16_t dst;   // slot
  uint16_t a;     // var index / slot index
  uint16_t b;     // var index / slot index / PowN exponent (int16)
  union {
    double c;
    struct {
      float clo;
      float chi;
    } c32;
  };
};
static_assert(sizeof(Instr) == 16, "Instr layout");

inline constexpr uint8_t make_head(uint8_t code, uint8_t sub)
{
  return static_cast<uint8_t>(code | (sub << 3));
}

}  // namespace cmn
