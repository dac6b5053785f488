// batch.hpp -- many independent instances of uneven sizes advanced together:
// each iteration is one captured graph in which the evaluator and the
// sampler are single launches over the children of every instance, and the
// per-instance steps (selection, incumbent, prune, pool rebuild, eviction)
// run as one thread block per instance in shared memory.
//
// Every instance follows the batched algorithm of the single-instance
// solver step for step (same selection order, salts, pool order, eviction
// and adaptive screen), so an instance's result does not depend on which
// other instances share the launches.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/cuminlp_gb300.h"
#include "kernels.cuh"

namespace cmn {

constexpr int kMiThreads = 1024;   // threads of a per-instance block
constexpr int kMiSortMax = 8192;   // largest pool a block sorts in shared memory

struct BatchCfg {
  int n_max;        // variables per instance, at most
  int slots_max;    // program slots per instance, at most
  int log2C;        // B: children per parent = 2^B
  int max_slots;    // = B
  int precision;
  int sample_all;
  int relative;
  uint64_t S;
  uint64_t e_max;         // parents per instance per iteration
  uint64_t cap;           // pool capacity per instance
  uint64_t P;             // pool stride: cap + e_max << B
  uint64_t K;             // instance slots
  uint64_t child_stride;  // child slots per instance: e_max << B
  int64_t max_cycle;
  int64_t enumerate_cap;
  int g_max;                 // lanes per child at most (1: one lane per child)
  uint64_t eval_capacity;    // threads the bound launches keep resident
  uint64_t sample_capacity;  // threads the sample launch keeps resident
  int seg_max;               // lazy form: sum-chain segments per instance program, at most
};

struct InstDesc {
  const Instr* prog64;
  const Instr* prog32;
  const int32_t* kinds;
  const double* root_lb;
  const double* root_ub;
  const int32_t* sched;  // lane schedules of the program (null: none)
  int32_t prog_len;
  int32_t n_vars;
  int32_t n_slots;
  int32_t active;
  int32_t g_max;        // lanes that may share one of its boxes
  int32_t pad_;
  uint64_t iter_limit;
  uint64_t batch_iter_limit;
  double tolerance;
  // lazy form: the FP32 point program, and the program's incremental
  // tables (Program::inc_*; inc_segments 0: the whole FP32 program bounds
  // each child)
  const Instr* prog32p;
  const int32_t* inc_seg;
  const int32_t* inc_off;
  const int32_t* inc_pcs;
  int32_t inc_segments;
  int32_t pad2_;
};

struct InstState {
  double gub;
  double glb;
  double dropped_lb_min;
  uint64_t pool_min_key;
  uint64_t pool_size;
  uint64_t n_parents;
  uint64_t salt_base;
  uint64_t expansions;
  uint64_t iterations;
  uint64_t remaining;
  uint64_t viable;
  uint64_t dropped_min_key;
  uint32_t done;
  uint32_t converged;
  uint32_t have_best;
  uint32_t use_screen;
  Cand best;
  cmn_counters counters;
};

struct BatchBufs {
  InstDesc* desc;
  InstState* st;
  double* lo;  // [K][n_max][P]
  double* hi;
  double* lb;  // [K][P]
  uint32_t* depth;
  double* plo;  // [K][n_max][e_max]
  double* phi;
  float* plo32;  // FP32 screen only: the same planes rounded outward
  float* phi32;
  uint32_t* pdepth;  // [K][e_max]
  ParentInfo* pinfo;
  SlotPlan* slots;  // [K][e_max][B]
  void* enum_scratch;  // [K][e_max][n_max]
  void* bis_scratch;
  uint64_t* heap_scratch;
  double* clb;  // [K][child_stride]
  uint8_t* cstate;
  double* cval;
  uint64_t* ce;
  uint32_t* list;  // certify list
  uint64_t* list_count;
  uint32_t* block_counts;
  uint32_t* block_offsets;
  uint64_t* child_base;  // [K + 2]: exclusive prefix of live children by `order` position, then the lane cap
  // [K]: the slots in the order the bound and sample launches walk their
  // children -- longest program first, so the launch's tail is short
  // programs (longest-processing-time-first balance)
  const uint32_t* order;
  double* best_point;  // [K][n_max]
  // lazy form
  double* plb;         // [K][e_max] the staged parents' certified FP64 lower bounds
  uint8_t* pfeas;      // [K][e_max] and their reference predicate
  float* inc_common;   // [K][seg_max][e_max] (lo, hi): chain sums without split variables
  float* inc_parts;    // [K][seg_max][2^B][e_max] (lo, hi): per slot part (incremental children)
  Best32* cbest;       // [K][child_stride] the FP32 screen's best sample per child
  // the verdict's warp runs: per `order` position the exclusive prefix of
  // its runs, then the total and the ticket the warps draw runs from
  uint64_t* vrun;      // [K + 2]
  uint8_t* vlg;        // [K] log2 of the lanes per parent of each position
};

// Puts `slot`'s root box in its pool and resets its state.
cudaError_t batch_init_slot(const BatchCfg& cfg, const BatchBufs& b, uint64_t slot, double gub0, cudaStream_t s);
// Blocks of the grid-stride launches of an iteration.  `eval` serves the
// evaluators, the verdict and the samplers (their lane groups size
// themselves to it); the lazy form's FP32 sum and screen passes use fewer
// registers and take as many blocks as stay resident on the GPU.
struct BatchGrids {
  int eval = 1;
  int inc_common = 1;
  int inc_parts = 1;
  int screen = 1;
};
BatchGrids batch_grids(const BatchCfg& cfg, int eval_grid);
// Enqueues one iteration over every active instance (capturable).
// `marks` (5 events or null) are recorded at the phase boundaries: start,
// after select + branch, after bound, after sample, after finish.
cudaError_t batch_iteration(const BatchCfg& cfg, const BatchBufs& b, const BatchGrids& grids, cudaStream_t s,
                            const cudaEvent_t* marks);
size_t batch_eval_smem(const BatchCfg& cfg, bool fp32);
size_t batch_sample_smem(const BatchCfg& cfg);
// resident blocks per SM of the bound (fp32: screen) and sample kernels
int batch_eval_occupancy(const BatchCfg& cfg, bool fp32);
int batch_sample_occupancy(const BatchCfg& cfg);
cudaError_t set_batch_kernel_attributes(int max_smem);

}  // namespace cmn
