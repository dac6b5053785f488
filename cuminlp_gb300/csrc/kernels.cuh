// kernels.cuh -- device data structures shared by the kernels and the host
// code that launches them.
#pragma once

#include <cmath>
#include <cstdint>

#include "program.h"

namespace cmn {

// One slot of one parent box: which variable it narrows and how
// (region/composition.hpp:50-56 SlotAssignment, flattened per slot).
struct SlotPlan {
  uint64_t width;   // fan-out of the slot
  uint64_t prefix;  // product of the previous slots' widths
  uint64_t dom;     // true domain size; parts >= dom are duplicates
  uint32_t vid;
  uint32_t kind;    // cmn_slot_kind
  // from the parent box: the width of one part (partition kinds) or the
  // ceiling of the lower bound (enumeration kinds), so that a child's
  // bounds cost one fused multiply-add instead of a division
  double step;
};

// SlotPlan::step of a slot over [plo, phi] (region/decode.hpp:44-71); the
// host and the device round the same IEEE operations the same way.
#ifdef __CUDACC__
__host__ __device__
#endif
inline double slot_step(uint32_t kind, double plo, double phi, uint64_t fan)
{
#ifdef __CUDA_ARCH__
  if (kind == 2 || kind == 3) return ceil(plo);
  return __ddiv_rn(__dsub_rn(phi, plo), (double)fan);
#else
  if (kind == 2 || kind == 3) return std::ceil(plo);
  return (phi - plo) / (double)fan;
#endif
}

struct ParentInfo {
  uint32_t count;   // slots in use
  uint32_t fathom;  // every live variable enumerated: exact points only
  uint64_t nreg;    // children the composition produces
};

// child verdict codes of the solver's evaluation
enum ChildState : uint8_t {
  kChildNone = 0,        // no child here (beyond nreg, or a fathomed parent)
  kChildDuplicate = 1,   // region::is_duplicate_child
  kChildInfeasible = 2,  // a constraint excludes the box
  kChildDominated = 3,   // obj lb above the incumbent
  kChildEligible = 4,    // survives (so far)
  kChildScreened = 5,    // FP32 screen left it open: certify in FP64
};

// Candidate of the incumbent reduction: smallest (value, parent, element).
struct Cand {
  double value;
  uint32_t k;
  uint32_t pad;
  uint64_t e;
};

__host__ __device__ inline bool cand_less(const Cand& a, const Cand& b)
{
  if (a.value < b.value) return true;
  if (b.value < a.value) return false;
  if (a.k != b.k) return a.k < b.k;
  return a.e < b.e;
}

// The lazy form's sample screen, per child slot: the smallest FP32 point
// value among its samples (+inf: none feasible in FP32, or not sampled) and
// that sample's index.
struct Best32 {
  float value;
  uint32_t i;
};

// The lazy form certifies a child in FP64 as soon as it is bounded when its
// FP32 bound lies within kCertifyBand * max(1, |incumbent|) below the
// incumbent: there the FP32 rounding error can hide a prune, further below
// FP64 would keep the child too.
constexpr double kCertifyBand = 1.0 / 1024.0;

#ifdef __CUDACC__
__host__ __device__
#endif
inline double certify_floor(double gub)
{
#ifdef __CUDA_ARCH__
  return __dsub_rn(gub, __dmul_rn(kCertifyBand, fmax(1.0, fabs(gub))));
#else
  return gub - kCertifyBand * std::fmax(1.0, std::fabs(gub));
#endif
}

// Children per chunk of the lazy form's sample verification: the point
// with the smallest FP32 value among the chunk's children is evaluated
// again in FP64 and is the chunk's incumbent candidate.
constexpr int kChunkLog2 = 5;

// Arguments of the child evaluation kernels.
struct EvalArgs {
  const Instr* prog;
  int prog_len;
  int n_vars;
  int n_slots;
  int log2C;             // children per parent = 2^log2C; -1: all children belong to parent 0
  const double* plo;     // parent planes: variable v of parent k at [v * pstride + k]
  const double* phi;
  const float* plo32;    // optional FP32 copies (rounded outward) read by the FP32 screen
  const float* phi32;
  uint64_t pstride;
  const ParentInfo* pinfo;  // null: every parent has no slots, one child
  const SlotPlan* slots;    // [k * max_slots + j]
  int max_slots;
  uint64_t n_children;            // used when n_children_dev is null
  const uint64_t* n_children_dev;
  const uint32_t* list;           // optional: evaluate only these children
  const uint64_t* list_count;
  const double* gub;              // incumbent at the start of the iteration
  const uint32_t* done;           // solver: nonzero once the search stopped
  const uint32_t* use_screen;     // FP32 screen: zero passes every child to the certify pass
  const double* parent_lb;        // lazy form: the parents' certified FP64 lower bounds
  // lazy form, incremental children (Program::inc_*): per (segment, parent)
  // the chain sums of the terms that touch no split variable, (lo, hi)
  // pairs at inc_common[2 * (s * pstride + k)]; per (segment, slot part,
  // parent) the chain sums of the terms of one split variable at one of
  // its parts, at inc_parts[2 * ((s * 2^log2C + u) * pstride + k)], where
  // u counts the parts of slot 0, then of slot 1, ...
  int inc_segments;
  const uint64_t* n_parents_dev;
  const int32_t* inc_seg;
  const int32_t* inc_off;
  const int32_t* inc_pcs;
  float* inc_common;
  float* inc_parts;
  // lane groups (null sched: one lane per box); see Program::sched
  const int32_t* sched;
  int g_max;
  uint64_t capacity;  // threads the launch keeps resident
  // outputs
  double* out_lb;
  double* out_ub;
  uint8_t* out_flag;  // role/raw: feasible; solver: ChildState
  uint32_t* error;    // solver: set when a staged program tile never arrived
  // byte offset in dynamic shared memory of the staged program tiles (FP64
  // passes with one lane per box); 0: the program is read from global memory
  size_t stage_at;
  // aggregate bounder: child c = r / agg_m folds into agg_keys[c] (min lb
  // key) and agg_keys[agg_k + c] (max ub key)
  unsigned long long* agg_keys;
  uint64_t agg_m;
  uint64_t agg_k;
};

struct SampleArgs {
  const Instr* prog;
  int prog_len;
  int n_vars;
  int n_slots;
  int log2C;
  const double* plo;
  const double* phi;
  uint64_t pstride;
  const ParentInfo* pinfo;
  const SlotPlan* slots;
  int max_slots;
  const int32_t* var_kinds;
  const double* root_lb;
  const double* root_ub;
  uint64_t n_children;
  const uint64_t* n_children_dev;
  uint64_t S;                // samples per child
  uint64_t salt;             // role: the salt; solver: salt of parent k is salt_base + k + 1
  const uint64_t* salt_base_dev;
  int exact;                 // role enumerator: exact points
  int sample_all;            // solver: sample every valid child, else only eligible ones
  const uint8_t* state;      // solver child states (null for roles)
  const double* gub;         // for the inadmissible-witness count
  const uint32_t* done;      // solver: nonzero once the search stopped
  Cand* block_best;          // [gridDim.x]
  unsigned long long* rejected;  // inadmissible feasible exact points below gub
  const int32_t* sched;      // lane groups, as EvalArgs
  int g_max;
  uint64_t capacity;
  int lg_min;                // points are shared by at least 2^lg_min lanes (sample_lg_min)
  // lazy form: the sample screen writes `cbest` (prog = the FP32 point
  // program); the sampler then evaluates only each chunk's best in FP64
  Best32* cbest;
};

}  // namespace cmn
