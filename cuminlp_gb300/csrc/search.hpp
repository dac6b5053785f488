// search.hpp -- device-resident state of the batched branch-and-bound and
// the launchers of its kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/cuminlp_gb300.h"
#include "kernels.cuh"

namespace cmn {

constexpr int kRadixBits = 11;
constexpr int kRadixBins = 1 << kRadixBits;
constexpr int kScanBlock = 512;  // threads per block of the compaction kernels
constexpr int kScanItems = 8;    // items per thread
constexpr int kScanTile = kScanBlock * kScanItems;
constexpr int kHistUnroll = 8;   // entries per lane in flight in the radix histogram
constexpr int kPickThreads = kRadixBins / 2;  // two bins per thread

constexpr uint8_t kSelAlive = 0;
constexpr uint8_t kSelParent = 1;
constexpr uint8_t kSelEvicted = 2;
constexpr uint8_t kSelNextParent = 3;

// k-th smallest key search (radix select over lb keys). The threshold is
// the bucket `prefix` under `mask` (the digits fixed so far); entries below
// it are taken, and the first `k` entries inside it in position order.
// The search starts below the leading bits that the smallest and largest
// keys share, which every key of the set shares too.
struct RadixState {
  uint64_t prefix;
  uint64_t mask;
  uint64_t k;         // rank still to find inside the current prefix
  uint64_t less;      // entries with key below the prefix bucket so far
  uint32_t active;    // 0: take everything (k >= n)
  uint32_t settled;   // 1: the bucket is taken whole; no further digits
  uint32_t rank;      // 1: entries inside the bucket need position ranks
  uint32_t bits_left; // key bits below the mask
  uint32_t hist[kRadixBins];
};

// Everything the iteration kernels read and write, in device memory.
struct SolverDev {
  double gub;
  double glb;
  double dropped_lb_min;
  uint64_t pool_min_key;   // min lb key of the current pool
  uint64_t pool_max_key;   // max lb key of the current pool
  uint64_t child_min_key;  // min / max lb key of this iteration's kept children
  uint64_t child_max_key;
  uint64_t evict_lo_key;   // key range of the rebuilt pool (before eviction)
  uint64_t evict_hi_key;
  uint64_t pool_size;      // L
  uint64_t n_parents;      // E of this iteration
  uint64_t n_children;     // E << log2C
  uint64_t salt_base;      // expansions before this iteration
  uint64_t expansions;
  uint64_t iterations;
  uint64_t remaining;      // unselected pool entries kept
  uint64_t kept;           // children kept
  uint64_t new_size;       // remaining + kept: the rebuilt pool before eviction
  uint64_t extent;         // pool_size + kept: entries of the current buffer
  uint64_t survivors;      // entries moved to the other buffer
  uint64_t free_top;       // free box-store slots (height of the free stack)
  // the next iteration's parents, selected while this iteration rebuilds the
  // pool: how many were asked for and how many were marked and staged
  uint64_t pre_k;
  uint64_t pre_count;
  uint32_t pre_valid;      // the staged parents are the next iteration's
  uint32_t skip_select;    // this iteration's parents were staged already
  uint64_t certify_count;
  uint64_t evict;          // 1 when the rebuilt pool exceeds the cap
  uint64_t dropped_min_key;
  uint64_t iter_valid;     // children bounded this iteration (not duplicates)
  uint64_t iter_excluded;  // of those, excluded by the FP64 verdict
  uint32_t use_screen;     // FP32 screen on for this iteration
  uint32_t pad_;
  uint32_t parity;         // pool buffer holding the current pool
  uint32_t done;
  uint32_t converged;
  uint32_t have_best;
  uint32_t improved;
  uint32_t error;
  Cand best;
  cmn_counters counters;
};

// Static configuration baked into the captured iteration.
struct SolverCfg {
  int n_vars;
  int n_slots;
  int prog_len;
  int log2C;        // B
  int max_slots;    // = B
  int precision;
  int sample_all;
  int relative;
  uint64_t S;
  uint64_t e_max;   // parents per iteration
  uint64_t cap;     // pool capacity (entries kept after an iteration)
  uint64_t pstride; // pool plane stride (cap + e_max << B)
  uint64_t iter_limit;
  uint64_t batch_iter_limit;
  int64_t max_cycle;
  int64_t enumerate_cap;
  double tolerance;
  int g_max;                 // lanes per child at most (1: one lane per child)
  uint64_t eval_capacity;    // resident threads of the bound kernels
  uint64_t sample_capacity;  // resident threads of the sampler
  int screen_grid;           // lazy form: blocks of the FP32 sample screen
  int screen_lg_min;         // and its lanes per point column
  int sample_lg_min;         // sampler point columns: one per 2^sample_lg_min lanes
  int inc;                   // lazy form: children by the incremental chain sums
  int inc_segments;
};

struct SolverBufs {
  SolverDev* dev;
  RadixState* radix;  // two select targets
  // the pool in position order (two parities): lower bound and box slot
  double* lb[2];
  uint32_t* slot[2];
  // box store: boxes slot-major, [slot * n_vars + v], and depth [slot]. A box
  // keeps its slot from its append until it is expanded or evicted, so
  // rebuilding the pool moves 12 bytes per entry instead of the whole box;
  // slot-major keeps the one write of a box and its one read contiguous.
  double* lo;
  double* hi;
  uint32_t* depth;
  uint32_t* free_slots;  // stack of free store slots (free_top entries)
  // marks over the pool buffers (two parities): kSelAlive, kSelParent
  // (expanded this iteration: a hole), kSelEvicted (dropped by the cap),
  // kSelNextParent (stays, and is expanded next iteration)
  uint8_t* sel[2];
  // staging of this iteration's parents: planes [v * e_max + k]
  double* plo;
  double* phi;
  float* plo32;  // FP32 screen only: the same planes rounded outward
  float* phi32;
  uint32_t* pdepth;
  // lazy form: the FP64 verdict of each staged parent (its certified lower
  // bound, and whether the reference predicate keeps it)
  double* plb;
  uint8_t* pfeas;
  uint32_t* pslot;       // store slots of the next iteration's parents, in order
  ParentInfo* pinfo;
  SlotPlan* slots;
  // policy scratch [k * n_vars + i]
  void* enum_scratch;
  void* bis_scratch;
  uint64_t* heap_scratch;
  // children
  double* clb;
  uint8_t* cstate;
  Best32* cbest;         // lazy form: the FP32 sample screen's best per child
  // lazy form, incremental children: the program's tables and the common
  // chain sums [segment][parent] (lo, hi)
  const int32_t* inc_seg;
  const int32_t* inc_off;
  const int32_t* inc_pcs;
  float* inc_common;
  float* inc_parts;
  uint32_t* list;        // certify list
  // compaction scratch
  uint32_t* block_counts;
  uint32_t* block_offsets;
  uint32_t* block_counts2;   // the second select target's
  uint32_t* block_offsets2;
  Cand* block_best;
  int n_block_best;
  // problem
  const Instr* prog64;
  const Instr* prog32;
  const Instr* prog32p;  // FP32 point program (the lazy form's sample screen)
  const int32_t* sched;  // lane schedules of the program (null: none)
  const int32_t* kinds;
  const double* root_lb;
  const double* root_ub;
  double* best_point;
};

// Initialises the device state: the root box as the only pool entry.
cudaError_t solver_init(const SolverCfg& cfg, const SolverBufs& b, const double* root_lb_host,
                        const double* root_ub_host, double gub0, cudaStream_t s);
// The lazy form's second stream: the FP64 verdict of the staged parents
// runs on `stream` beside the branching and the FP32 child bounds, forked
// from and joined back to the iteration's stream by the two events.
struct SideStream {
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr;
  cudaEvent_t join = nullptr;
};

// Enqueues one batched iteration (all kernels) on `s`; capturable.
// `marks` (kPhaseMarks events or null) are recorded as event nodes: 0-4 at
// the phase boundaries (start, after branching, after bounding, after
// sampling, end); in the lazy form 5 and 6 around the FP64 verdict on the
// side stream and 7 after the FP32 child bounds.
// `with_select`: the iteration selects and stages its own parents (the first
// iteration); otherwise the previous iteration staged them, and the
// iteration flags a device error if it did not.
constexpr int kPhaseMarks = 8;
cudaError_t solver_iteration(const SolverCfg& cfg, const SolverBufs& b, int eval_grid, int sample_grid,
                             cudaStream_t s, const SideStream& side, const cudaEvent_t* marks, bool with_select);
// Fills min key / viable count of the current pool (after the run).
cudaError_t solver_pool_stats(const SolverCfg& cfg, const SolverBufs& b, uint64_t* viable_dev, cudaStream_t s);
// Copies pool entries [start, start + count) in position order: boxes as
// [i][v] (lo, hi) pairs and depths (either may be null).
cudaError_t solver_frontier_gather(const SolverCfg& cfg, const SolverBufs& b, uint64_t start, uint64_t count,
                                   double* boxes, uint32_t* depths, cudaStream_t s);


}  // namespace cmn
