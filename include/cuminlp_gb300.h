/*
 * cuminlp_gb300.h -- C ABI of the GB300-native interval branch-and-bound
 * hot path.
 *
 * Everything crosses this boundary as plain pointers, sizes and POD structs;
 * no exception, no C++ type and no torch type leaves the library.  Every
 * entry point returns a cmn_status; on failure cmn_last_error() holds a
 * human-readable message for the calling thread.
 *
 * Each declaration names the interface of the reference (CuMINLPSearch,
 * include/cuminlp/...) that it replaces, as file:line.
 *
 * Conventions
 *   - A box is n_vars (lb, ub) pairs of doubles, interleaved: the exact
 *     memory layout of `cu::interval<double>[n_vars]`
 *     (backend/backend.hpp:39-44, Region::box).
 *   - Pointers returned by a role call are views into storage the role
 *     owns, valid until the next call on that role
 *     (backend/backend.hpp:52-54, 66-67).
 *   - One handle is never used from two threads at once.
 *   - A problem lives on the device current when it is created.  Calls on
 *     a problem, role, solver or batch make that device current and leave
 *     it current (cmn_sample_noalloc alone restores the caller's); a thread
 *     that drives several GPUs sets its device again after such a call.
 */
#ifndef CUMINLP_GB300_H
#define CUMINLP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------
 * Status codes.  Mirror the reference's exception hierarchy
 * (errors.hpp:11-57: InvalidDAG, InvalidProblem, ShapeMismatch,
 * InvalidConfiguration, ResourceExhausted), CUDAError
 * (cuda_utils.cuh:22-35) and OverBudgetError (backend/backend.hpp:236-287).
 * ------------------------------------------------------------------- */
typedef enum cmn_status {
  CMN_OK = 0,
  CMN_INVALID_DAG = 1,
  CMN_INVALID_PROBLEM = 2,
  CMN_SHAPE_MISMATCH = 3,
  CMN_INVALID_CONFIGURATION = 4,
  CMN_OVER_BUDGET = 5,
  CMN_CUDA_ERROR = 6,
  CMN_TIMEOUT = 7,
  CMN_INTERNAL = 8
} cmn_status;

/* Operators, in the order of model::Op (model/dag.hpp:12-33). */
typedef enum cmn_op {
  CMN_OP_VAR = 0,
  CMN_OP_CONST = 1,
  CMN_OP_ADD = 2,
  CMN_OP_SUB = 3,
  CMN_OP_MUL = 4,
  CMN_OP_DIV = 5,
  CMN_OP_SQR = 6,
  CMN_OP_NEG = 7,
  CMN_OP_EXP = 8,
  CMN_OP_LOG = 9,
  CMN_OP_SQRT = 10,
  CMN_OP_SIN = 11,
  CMN_OP_COS = 12,
  CMN_OP_TANH = 13,
  CMN_OP_POWN = 14,
  CMN_OP_POW = 15,
  CMN_OP_ABS = 16,
  CMN_OP_MIN = 17,
  CMN_OP_MAX = 18
} cmn_op;

/* model::VarKind (model/problem.hpp:16-21). */
typedef enum cmn_var_kind {
  CMN_VAR_CONTINUOUS = 0,
  CMN_VAR_INTEGER = 1,
  CMN_VAR_BINARY = 2
} cmn_var_kind;

/* model::Cmp (model/problem.hpp:22-26). */
typedef enum cmn_cmp { CMN_CMP_LE = 0, CMN_CMP_EQ = 1 } cmn_cmp;

/* region::SlotKind (region/slot.hpp:12-18). */
typedef enum cmn_slot_kind {
  CMN_SLOT_CONTINUOUS = 0,
  CMN_SLOT_INTEGER_PARTITION = 1,
  CMN_SLOT_INTEGER_ENUMERATE = 2,
  CMN_SLOT_BINARY_ENUMERATE = 3
} cmn_slot_kind;

/* One model::DAGNode (model/dag.hpp:58-68), flattened.  `in0`/`in1` are
 * operand node ids (-1 when absent); `n_in` says how many are used.  The
 * payload union of the reference becomes three plain fields, of which the
 * one matching `op` is read: `constant` (Const), `var_index` (Var),
 * `int_exp` (PowN). */
typedef struct cmn_node {
  int32_t op;
  int32_t n_in;
  int64_t in0;
  int64_t in1;
  int64_t var_index;
  double constant;
  int32_t int_exp;
  int32_t reserved;
} cmn_node;

/* model::ConstraintRef (model/problem.hpp:34-40). */
typedef struct cmn_constraint {
  int64_t root;
  int32_t cmp;
  int32_t reserved;
  double rhs;
} cmn_constraint;

/* The flattened model::Problem<double> (model/problem.hpp:195-358). */
typedef struct cmn_problem_desc {
  const cmn_node* nodes;
  int64_t n_nodes;
  const double* var_lb;
  const double* var_ub;
  const int32_t* var_kinds;
  int64_t n_vars;
  int64_t objective_root;
  const cmn_constraint* constraints;
  int64_t n_constraints;
} cmn_problem_desc;

typedef struct cmn_problem cmn_problem; /* opaque, owns device copies */

/* What the library derived from a problem when it was created. */
typedef struct cmn_problem_info {
  int64_t n_vars;
  int64_t n_constraints;
  int64_t n_nodes;
  int64_t buffer_node_count;  /* backend/graph/cost.hpp:38-68 */
  int64_t program_length;     /* fused-evaluator instructions */
  int64_t program_slots;      /* shared-memory value slots per box */
  double flops_per_box;       /* algorithmic FP64 ops of one interval eval */
  double point_flops_per_box; /* algorithmic FP64 ops of one point eval */
  double bytes_per_box;       /* algorithmic HBM bytes of one box eval */
  int64_t program_segments;   /* independent sum chains (0: not split) */
  int64_t lanes_per_box_max;  /* lanes that may share one box (1: none) */
} cmn_problem_info;

/* Thread-local message describing the last failure on this thread. */
const char* cmn_last_error(void);

/* Library version string. */
const char* cmn_version(void);

/* Builds a problem from a flattened DAG and validates it exactly as
 * Problem::validate() does (model/problem.hpp:282-355), then uploads the
 * compiled evaluation program to the current CUDA device. */
cmn_status cmn_problem_create(const cmn_problem_desc* desc,
                              cmn_problem** out);
void cmn_problem_destroy(cmn_problem* problem);
cmn_status cmn_problem_get_info(const cmn_problem* problem,
                                cmn_problem_info* out);

/* backend::RegionCostModel (backend/cost_model.hpp:26-76) of the fused
 * backend: device bytes per sample / region and a fixed per-role part. */
typedef struct cmn_cost_model {
  uint64_t sampler_bytes_per_sample;
  uint64_t bound_bytes_per_region;
  uint64_t exact_bytes_per_region;
  uint64_t fixed_bytes;
} cmn_cost_model;
/* Replaces RegionBackendFactory::cost_model (backend/backend.hpp:200-201)
 * and graph::cost_model_for (backend/graph/cost.hpp:83-99). */
cmn_status cmn_cost_model_get(const cmn_problem* problem, cmn_cost_model* out);

/* Host-side policy and decode, for drivers that run on the host.
 *
 * Replaces BisectionBudgetCompositionPolicy::choose
 * (policy/bisection_budget.hpp:81-262) on one box (interleaved (lb, ub),
 * n_vars pairs): writes up to 64 slots (kinds, var_ids, widths, domain
 * sizes) and their count; `fathom` (may be NULL) is 1 when every live
 * variable is enumerated.  Ties resolve in the reference's heap order, as
 * the device policy does. */
cmn_status cmn_bisection_choose(const double* box, const int32_t* var_kinds,
                                int64_t n_vars, int32_t budget_bits,
                                uint64_t max_cycle_size, uint64_t enumerate_cap,
                                int32_t relative_width, uint8_t* slot_kinds,
                                uint64_t* var_ids, uint64_t* widths,
                                uint64_t* domain_sizes, int64_t* slot_count,
                                int32_t* fathom);
/* region::decode::slot_bounds (region/decode.hpp:44-71) in the FMA form the
 * device evaluates. */
void cmn_slot_bounds(int32_t kind, double plo, double phi, uint64_t part,
                     uint64_t fan_out, double* lo, double* hi);

/* ---------------------------------------------------------------------
 * Region roles: the plugin boundary of the reference
 * (backend/backend.hpp:81-219).  A role is built once per Composition
 * (its slot kinds) and launched per box with per-launch var_ids/widths.
 * ------------------------------------------------------------------- */
typedef enum cmn_role_kind {
  CMN_ROLE_BOUNDER = 0,    /* RegionBounder     backend/backend.hpp:93-101 */
  CMN_ROLE_SAMPLER = 1,    /* RegionSampler     backend/backend.hpp:81-90  */
  CMN_ROLE_ENUMERATOR = 2  /* RegionEnumerator  backend/backend.hpp:108-116 */
} cmn_role_kind;

typedef struct cmn_role cmn_role; /* opaque */

/* backend::OverBudget facts (backend/backend.hpp:236-260). */
typedef struct cmn_over_budget {
  uint64_t needed_bytes;
  uint64_t budget_bytes;
  uint64_t n_regions;
  uint64_t elements_per_region;
  uint64_t bytes_per_element;
} cmn_over_budget;

/* backend::CandidateResult (backend/backend.hpp:57-64).  `point` is all-NaN
 * when `found` is 0; `value` is +inf then. */
typedef struct cmn_candidate {
  int32_t found;
  int32_t reserved;
  double value;
  const double* point;
  int64_t index;
} cmn_candidate;

/* Replaces RegionBackendFactory::build_subdivision for one role
 * (backend/backend.hpp:215-219; graph/replay.cuh:264-521 GraphReplay::build).
 * `budget_bytes` 0 means "what the device has free".  On CMN_OVER_BUDGET
 * `facts` (if non-null) is filled and nothing is allocated; more than 2^32
 * regions is over budget too (needed_bytes UINT64_MAX), as a saturated
 * fan-out is in the reference (graph_replay_test.cu:442-461).  Building an
 * enumerator for a composition that is not fully enumerable returns
 * CMN_INVALID_CONFIGURATION. */
cmn_status cmn_role_build(const cmn_problem* problem, int32_t role,
                          const uint8_t* slot_kinds, int64_t slot_count,
                          uint64_t n_regions, uint64_t budget_bytes,
                          uint64_t sample_points, cmn_role** out,
                          cmn_over_budget* facts);
void cmn_role_destroy(cmn_role* role);
uint64_t cmn_role_n_regions(const cmn_role* role);
/* n_samples() / n_points() of the reference roles. */
uint64_t cmn_role_n_elements(const cmn_role* role);

/* RegionBounder::bound (backend/backend.hpp:99; graph/replay.cuh:823-828).
 * `feasible`/`obj_lb` receive pointers to n_regions entries each. */
cmn_status cmn_bound(cmn_role* role, const double* box,
                     const uint64_t* var_ids, const uint64_t* widths,
                     const uint8_t** feasible, const double** obj_lb,
                     uint64_t* n_regions);

/* RegionSampler::sample (backend/backend.hpp:87-88; graph/replay.cuh:830-836). */
cmn_status cmn_sample(cmn_role* role, const double* box,
                      const uint64_t* var_ids, const uint64_t* widths,
                      uint64_t salt, cmn_candidate* out);

/* RegionEnumerator::enumerate (backend/backend.hpp:114; replay.cuh:838-843). */
cmn_status cmn_enumerate(cmn_role* role, const double* box,
                         const uint64_t* var_ids, const uint64_t* widths,
                         cmn_candidate* out);

/* Allocation-free sampler.  No counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc -- processes whose device memory is
 * owned by a pool they do not control (a serving framework's caching
 * allocator, a fixed arena on a shared GPU) or code that must not grow its
 * device footprint after start-up.  It does what a sampler role built by
 * cmn_role_build(slot_kinds, n_regions, sample_points) then cmn_sample(box,
 * var_ids, widths, salt) does, with the same results, but allocates no
 * device memory: its scratch is one 512 KiB device array per GPU, held by
 * the library until the process exits.  Host inputs and outputs; `point`
 * receives n_vars doubles and out->point points at it.  Limits (beyond
 * them the call returns CMN_INVALID_CONFIGURATION): at most 8192 variables
 * (the array's share for the box and the witness), and the sampler's point
 * columns must fit in one block's shared memory -- 8 * (n_vars + program
 * slots) * 128 / G bytes, where G lanes share a point: up to 32 for a
 * program without shared slots (every generated QCQP; n_vars + slots up to
 * about 7,200 on GB300), 1 for a program with them (up to about 226).
 * Every call looks up the array's address on the problem's device with
 * cudaGetSymbolAddress; the first call on a device also loads the
 * library's device code there, so make it before any stream capture.  The
 * call makes the problem's device current and restores the caller's
 * current device before it returns.  All calls share the array and it
 * keeps the last call's contents; calls that overlap on the GPU (several
 * streams or threads at once) race on it and must be serialised by the
 * caller.  `stream` is a cudaStream_t or NULL; the call returns after the
 * results are on the host. */
cmn_status cmn_sample_noalloc(const cmn_problem* problem,
                              const uint8_t* slot_kinds, int64_t slot_count,
                              uint64_t n_regions, uint64_t sample_points,
                              const double* box, const uint64_t* var_ids,
                              const uint64_t* widths, uint64_t salt,
                              cmn_candidate* out, double* point,
                              void* stream);

/* ---------------------------------------------------------------------
 * Raw batched evaluation: the fused evaluator (a) over a frontier of boxes
 * stored SoA as lo/hi planes (plane v holds variable v of every box).
 * Replaces the per-node kernel chain of graph/kernels.cuh:177-419 for a
 * batch of already-materialised boxes.
 * ------------------------------------------------------------------- */
typedef enum cmn_precision {
  CMN_PRECISION_FP64 = 0,            /* plain FP64 directed rounding */
  CMN_PRECISION_FP32_SCREEN = 1,     /* FP32 outward screen, FP64 certify of
                                        every survivor (the plain FP64
                                        trajectory, bit for bit) */
  CMN_PRECISION_FP32_LAZY = 2        /* solver only: children bounded in
                                        FP32 only; a box's bound is certified
                                        in FP64 when it is selected for
                                        expansion (see cmn_solve_options) */
} cmn_precision;

/* `lo`/`hi` point at n_vars planes of `stride` doubles; outputs have
 * n_boxes entries.  `device_pointers` 1 means every array is device memory
 * and the call is asynchronous on `stream` (a cudaStream_t, or NULL for the
 * legacy default stream); 0 means host memory and the call blocks.
 * precision FP32_SCREEN evaluates in FP32 with outward-rounded inputs and
 * writes the (sound, wider) FP32 enclosure widened to double. */
cmn_status cmn_eval_boxes(const cmn_problem* problem, int32_t precision,
                          const double* lo, const double* hi,
                          uint64_t n_boxes, uint64_t stride,
                          double* obj_lb, double* obj_ub, uint8_t* feasible,
                          int32_t device_pointers, void* stream);

/* ---------------------------------------------------------------------
 * Device-resident batched branch-and-bound: the solver API
 * (search/driver.hpp:36-54 SolveOutcome, :97-134 SearchDriver constructor,
 * :137-537 solve()).  The frontier (box pool) lives in HBM; one iteration
 * selects the best parents, branches them (BisectionBudget policy,
 * policy/bisection_budget.hpp:81-262), bounds and samples every child,
 * prunes and compacts -- all as one captured CUDA graph.
 * ------------------------------------------------------------------- */

/* search::StopReason (search/budget.hpp:21-29), plus FrontierCap. */
typedef enum cmn_stop_reason {
  CMN_STOP_CONVERGED = 0,
  CMN_STOP_EXHAUSTED = 1,
  CMN_STOP_ITERATION_LIMIT = 2,
  CMN_STOP_HOST_MEMORY = 3,
  CMN_STOP_ALLOCATION_FAILURE = 4,
  CMN_STOP_DEVICE_MEMORY = 5,
  CMN_STOP_RUNNING = 6
} cmn_stop_reason;

typedef struct cmn_solve_options {
  uint64_t iter_limit;        /* max boxes expanded (SearchDriver iter_limit) */
  uint64_t batch_iter_limit;  /* max batched iterations, 0 = unlimited */
  double tolerance;           /* gap_closed tolerance, default 1e-6 */
  int32_t precision;          /* cmn_precision */
  int32_t bisection_budget;   /* B: each expanded box gets 2^B children */
  uint64_t frontier_cap;      /* pool capacity in boxes */
  uint64_t batch_parents;     /* max boxes expanded per iteration */
  uint64_t sample_points;     /* samples per child */
  int32_t sample_all;         /* 1: sample every child (reference order) */
  int32_t relative_width;     /* RelativeBisectionBudget heap key */
  uint64_t max_cycle_size;    /* slot cap (SearchCalibration) 0 = 64 */
  uint64_t enumerate_cap;     /* SearchCalibration::enumerate_cap */
  int32_t has_known_primal;   /* seeds GUB (known_primal_bound) */
  int32_t autotune;           /* 1: the evaluator's launch shape from
                                 cmn_autotune (run on first use) */
  double known_primal_bound;
  uint64_t time_limit_ms;     /* 0 = none */
} cmn_solve_options;

/* report::RunTelemetry (report/telemetry.hpp:23-87) plus the batched and
 * precision counters. */
typedef struct cmn_counters {
  uint64_t iterations;         /* batched iterations */
  uint64_t expansions;         /* boxes expanded (reference iterations) */
  uint64_t fathomed;
  uint64_t fathomed_points;
  uint64_t bounded;            /* child boxes evaluated */
  uint64_t sampled;
  uint64_t enqueued;
  uint64_t witness_rejected;
  uint64_t pruned_duplicate;
  uint64_t pruned_infeasible;
  uint64_t pruned_dominated;
  uint64_t dropped_viable;
  uint64_t dropped_dominated;
  uint64_t screened_fp32;      /* children evaluated by the FP32 screen */
  uint64_t certified_fp64;     /* boxes evaluated in FP64 (children, or
                                  the selected parents of the lazy form) */
  uint64_t peak_frontier;
  uint64_t certify_pruned;     /* lazy form: selected boxes whose FP64
                                  bound is infeasible or above the
                                  incumbent, so they are not expanded */
} cmn_counters;

typedef struct cmn_outcome {
  double lower_bound;
  double upper_bound;
  int32_t stop_reason;
  int32_t proven_optimal;
  int32_t infeasible;
  int32_t found_incumbent;
  uint64_t frontier_size;
  uint64_t viable;
  double dropped_lb_min;
  double elapsed_ms;
  cmn_counters counters;
} cmn_outcome;

/* aggregate::AggregateBound (aggregate/bound.hpp:40-59).  `hull_ub` is
 * not an incumbent: it bounds the objective over the child's unexcluded
 * part, at no known point. */
typedef struct cmn_aggregate_bound {
  double lb;       /* min objective lb over the child's feasible regions */
  double hull_ub;  /* max objective ub over them */
  int32_t feasible;
  int32_t reserved;
} cmn_aggregate_bound;

/* Replaces AggregateBounder::bound_children (aggregate/bound.hpp:84-105;
 * the AggregateBounderReplay launch and fold, backend/aggregate/
 * replay.cuh:320-361, 497-556, with mask_bounds_kernel,
 * backend/aggregate/kernels.cuh:32-47) for one region.  `role` is a bounder
 * of N regions; region r belongs to child r / (N / k), which is how the
 * reference lays out a partition's launch slots (refine slots first, branch
 * slots last: aggregate/partition.hpp).  The per-region verdicts are folded
 * on the device and only k results cross to the host.  Minimum and maximum
 * follow IEEE total order on equal magnitudes (-0 below +0).  A child whose
 * regions are all excluded is (+inf, +inf, feasible = 0).  `out` is a view
 * of k entries, valid until the next call on the role. */
cmn_status cmn_bound_children(cmn_role* role, const double* box,
                              const uint64_t* var_ids, const uint64_t* widths,
                              uint64_t k, const cmn_aggregate_bound** out);

/* Fills `opts` with the defaults (SearchDriver defaults where they exist:
 * driver.hpp:97-109). */
void cmn_solve_options_default(cmn_solve_options* opts);

typedef struct cmn_solver cmn_solver; /* opaque */

cmn_status cmn_solver_create(const cmn_problem* problem,
                             const cmn_solve_options* opts,
                             cmn_solver** out);
void cmn_solver_destroy(cmn_solver* solver);
/* Runs up to `max_iterations` batched iterations (0 = until a stop
 * condition).  Returns CMN_OK while running or stopped normally. */
cmn_status cmn_solver_step(cmn_solver* solver, uint64_t max_iterations);
/* Live queries: bounds, incumbent and gap (GUB - GLB). */
cmn_status cmn_query_bounds(const cmn_solver* solver, double* lower_bound,
                            double* upper_bound);
/* Copies the incumbent into `point` (n_vars doubles); returns 0 in
 * `found` when there is none. */
cmn_status cmn_query_incumbent(const cmn_solver* solver, double* point,
                               int32_t* found);
cmn_status cmn_query_gap(const cmn_solver* solver, double* gap);
/* Final (or current) outcome after finalise_bounds
 * (search/epilogue.hpp:89-127). */
cmn_status cmn_solver_outcome(cmn_solver* solver, cmn_outcome* out);
/* The CUDA stream the solver's iteration runs on (a cudaStream_t). */
void* cmn_solver_stream(cmn_solver* solver);
/* Copies the current frontier (pool order) to the host: up to `room`
 * boxes as interleaved (lb, ub) pairs, their lower bounds and depths.
 * `count` receives the frontier size.  The reference keeps this state in
 * IntervalPQueue + IntervalHistory (search/frontier.hpp:152-338,
 * search/history.hpp:20-137); any pointer may be NULL. */
cmn_status cmn_solver_frontier(cmn_solver* solver, double* boxes,
                               double* lower_bounds, uint32_t* depths,
                               uint64_t room, uint64_t* count);

/* Phase timings of the most recent iteration, from CUDA events recorded
 * inside the captured iteration: [0] select+branch, [1] bound (FP64
 * evaluation, or FP32 screen + FP64 certify; in the lazy form the FP32
 * child bounds, the wait for the parents' FP64 verdict that runs beside
 * them, and the fold), [2] sample + incumbent, [3] prune + pool rebuild,
 * [4] whole iteration; milliseconds. */
cmn_status cmn_solver_phase_ms(cmn_solver* solver, double* ms5);
/* Lazy form only: [0] the FP64 verdict of the staged parents, timed on
 * its own stream, [1] the FP32 child bounds, timed on the iteration's
 * stream from the end of branching; both run at once, so they overlap
 * phases [0] and [1] above.  Milliseconds, most recent iteration. */
cmn_status cmn_solver_lazy_ms(cmn_solver* solver, double* ms2);
/* Kernel nodes one captured iteration launches. */
uint64_t cmn_solver_kernels_per_iteration(const cmn_solver* solver);

/* Measures the device's FP64 (precision 0) or FP32 (precision 1) FMA
 * throughput with a dependent-chain-free FMA loop on every SM; writes
 * TFLOP/s (2 flops per FMA).  A roofline denominator, not part of the
 * search path. */
cmn_status cmn_measure_fma_peak(int32_t precision, double* tflops);

/* Self-test of the integer-pipe binary64 add / subtract / multiply with
 * directed rounding, and multiply rounded to nearest, against the device's
 * FP64 instructions, over `n`
 * operand pairs of one family (0: any bits, 1: close exponents, 2:
 * cancellation, 3: range edges, 4: runs of ones and zeros) from `seed`.
 * out3: [0] mismatches, [1] results the integer path produced, [2] results
 * checked.  Not part of the search path. */
cmn_status cmn_fp64_emu_check(uint64_t n, uint64_t seed, int32_t family, uint64_t* out3);
/* The same check with the integer path compiled for the host, against the
 * host FPU in each rounding mode; needs no GPU. */
cmn_status cmn_fp64_emu_check_host(uint64_t n, uint64_t seed, int32_t family, uint64_t* out3);

/* One integer-path operation on the host, for checks against exact
 * arithmetic: op 0/1 add rounded down/up, 2/3 subtract down/up, 4/5
 * multiply down/up, 6 multiply to nearest (ties to even).  *handled is 0,
 * and *out unwritten, when an operand or the result is not a normal number
 * or a sum cancels exactly (those take the FP64 instruction). */
cmn_status cmn_fp64_emu_op_host(int32_t op, double a, double b, double* out, int32_t* handled);

/* Timed autotuning of the fused evaluator's launch shape for one problem.
 * No counterpart in the reference (its graph backend launches one kernel
 * per DAG node with a fixed shape).  Candidates: blocks per SM from 1 to
 * the kernel's residency, and caps on the lanes that share one box (boxes
 * per warp = 32 / lanes) of 1, 2, 4 ... up to the program's useful
 * maximum; each is timed with CUDA events over `n_boxes` random boxes
 * inside the root box, best of three launches.  The fastest is recorded on
 * the problem (for `precision` 0, FP64, or 1, FP32) and used by every
 * solver created for it with cmn_solve_options.autotune = 1; results never
 * depend on the choice.  Synchronous; allocates its test boxes. */
typedef struct cmn_tune_result {
  int32_t blocks_per_sm;   /* chosen */
  int32_t lanes_cap;       /* chosen: most lanes per box */
  double ms_best;          /* its launch time */
  double ms_default;       /* the untuned shape's (full residency, program's lane maximum) */
  int32_t candidates;      /* shapes timed */
  int32_t reserved;
} cmn_tune_result;
cmn_status cmn_autotune(cmn_problem* problem, int32_t precision, uint64_t n_boxes, cmn_tune_result* out);

/* The compiled program of a problem (the fused evaluator's straight-line
 * code), for tools and tests: `precision` 0 gives the FP64 program, 1 the
 * FP32 screen program (constants as outward-rounded pairs).  Each
 * instruction is 16 bytes: u8 head (bits 0-2 the opcode, 3-7 its
 * sub-code), u8 operand modes, u16 dst, u16 a, u16 b, then an f64 payload
 * or, in the FP32 program, an (f32 lo, f32 hi) pair.  Writes at most
 * `capacity` instructions to `out` (16 * capacity bytes) and the program's
 * length to *length. */
cmn_status cmn_problem_program(const cmn_problem* problem, int32_t precision,
                               void* out, int64_t capacity, int64_t* length);
/* The same program, compiled on the host straight from a description:
 * needs no CUDA device and allocates no device memory, for tools and tests
 * that run where no GPU is present.  The description is validated as
 * cmn_problem_create validates it. */
cmn_status cmn_program_compile(const cmn_problem_desc* desc, int32_t precision,
                               void* out, int64_t capacity, int64_t* length);

/* One-call solve: create, run to a stop condition, report, destroy. */
cmn_status cmn_solve(const cmn_problem* problem,
                     const cmn_solve_options* opts, cmn_outcome* outcome,
                     double* best_point);

/* ------------------------------------------------------------------------
 * Multi-instance batch: many independent problems of uneven sizes advanced
 * together, one captured graph per iteration over every occupied slot.
 * No reference counterpart (the reference solves one problem per
 * SearchDriver, search/driver.hpp:137-537); every instance follows the
 * batched algorithm of cmn_solver step for step, so its outcome, incumbent
 * and counters are those cmn_solver gives it with the same options.
 *
 * The batch fixes the shared options when it is created: precision,
 * bisection_budget, batch_parents (parents per instance per iteration),
 * frontier_cap (pool per instance), sample_points, sample_all,
 * relative_width, max_cycle_size and enumerate_cap.  Per instance:
 * iter_limit, batch_iter_limit, tolerance and the known primal bound.
 * Limits: frontier_cap + batch_parents * 2^bisection_budget <= 8192.
 * ---------------------------------------------------------------------- */
typedef struct cmn_batch cmn_batch; /* opaque */

typedef struct {
  uint64_t slots;            /* instances resident at once */
  int32_t max_vars;          /* largest n_vars an instance may have */
  int32_t max_program_slots; /* largest program slot count; -1: as many as
                                fit (smaller tiles give more resident blocks) */
  int32_t device;            /* CUDA device of the batch and its problems */
  int32_t max_segments;      /* lazy form: largest number of sum-chain
                                segments (objective + constraint chains) of
                                an instance's program; 0: max_vars + 1 */
  cmn_solve_options shared;  /* the shared options listed above */
} cmn_batch_config;

cmn_status cmn_batch_create(const cmn_batch_config* config, cmn_batch** out);
void cmn_batch_destroy(cmn_batch* batch);
/* Puts `problem` into a free slot (written to `slot`) with its root box.
 * `opts` gives the per-instance options; its shared options must equal
 * the batch's.  CMN_OVER_BUDGET when no slot is free.  The problem must
 * outlive its slot. */
cmn_status cmn_batch_add(cmn_batch* batch, const cmn_problem* problem,
                         const cmn_solve_options* opts, uint64_t* slot);
/* Runs up to `max_iterations` iterations (0 = until every occupied slot
 * has stopped); `running` receives the occupied slots still searching. */
cmn_status cmn_batch_step(cmn_batch* batch, uint64_t max_iterations,
                          uint64_t* running);
/* The two halves of cmn_batch_step, for callers that overlap several
 * batches: enqueue `iterations` iterations without waiting, then wait for
 * them and refresh the per-slot state (`running` as in cmn_batch_step). */
cmn_status cmn_batch_launch(cmn_batch* batch, uint64_t iterations);
cmn_status cmn_batch_sync(cmn_batch* batch, uint64_t* running);
/* Non-blocking: 1 in `idle` when every launched iteration has finished. */
cmn_status cmn_batch_query(cmn_batch* batch, int32_t* idle);
/* Sum of the counters of every occupied slot (as of the device's current
 * state) and the number of occupied slots still searching. */
cmn_status cmn_batch_totals(cmn_batch* batch, cmn_counters* sum,
                            uint64_t* running);
/* Phase timings of the most recent batch iteration, as
 * cmn_solver_phase_ms reports them. */
cmn_status cmn_batch_phase_ms(cmn_batch* batch, double* ms5);
/* Device bytes one slot's box pool and work buffers take. */
uint64_t cmn_batch_slot_bytes(const cmn_batch* batch);
/* State of `slot` as of the last step: 1 in `done` once it stopped. */
cmn_status cmn_batch_poll(const cmn_batch* batch, uint64_t slot,
                          int32_t* done);
/* Outcome (finalise_bounds, search/epilogue.hpp:89-127) and incumbent of
 * `slot` (`best_point`: n_vars doubles, NaN when none; may be NULL). */
cmn_status cmn_batch_outcome(cmn_batch* batch, uint64_t slot,
                             cmn_outcome* out, double* best_point);
/* Copies `slot`'s frontier (pool order) as cmn_solver_frontier does. */
cmn_status cmn_batch_frontier(cmn_batch* batch, uint64_t slot, double* boxes,
                              double* lower_bounds, uint32_t* depths,
                              uint64_t room, uint64_t* count);
/* Frees `slot` for another problem. */
cmn_status cmn_batch_release(cmn_batch* batch, uint64_t slot);
/* The CUDA stream the batch runs on (a cudaStream_t). */
void* cmn_batch_stream(cmn_batch* batch);
/* Kernel nodes one captured batch iteration launches. */
uint64_t cmn_batch_kernels_per_iteration(const cmn_batch* batch);
/* Solves `count` problems with up to `config->slots` resident at once,
 * refilling slots as instances stop; opts[i] are problem i's options.
 * outcomes[i] and best_points + i * point_stride (n_vars of problem i;
 * NULL to skip) receive the results. */
cmn_status cmn_batch_solve(const cmn_batch_config* config,
                           const cmn_problem* const* problems,
                           const cmn_solve_options* opts, uint64_t count,
                           cmn_outcome* outcomes, double* best_points,
                           uint64_t point_stride);

/* ------------------------------------------------------------------------
 * Serving: a request loop with continuous batching.  No reference
 * counterpart.  A worker thread owns one cmn_batch per size class (each
 * on its own stream, so the classes' iterations overlap on the device);
 * between rounds of `iterations_per_round` iterations it admits queued
 * requests into free slots of the smallest class that holds them, while the
 * resident box pools stay within `pool_budget_bytes`, and retires the
 * requests that stopped.  A request's result does not depend on the other
 * requests or on its class: it is what cmn_batch (and cmn_solver) give
 * it alone with the same options.
 * ---------------------------------------------------------------------- */
typedef struct cmn_server cmn_server; /* opaque */

#define CMN_SERVER_MAX_CLASSES 8

typedef struct {
  cmn_solve_options shared;  /* as cmn_batch_config.shared */
  int32_t device;
  int32_t n_classes;                                /* 1..8 */
  int32_t class_max_vars[CMN_SERVER_MAX_CLASSES];   /* ascending */
  int32_t class_max_program_slots[CMN_SERVER_MAX_CLASSES];
  uint64_t class_slots[CMN_SERVER_MAX_CLASSES];
  uint64_t pool_budget_bytes;     /* cap on admitted slots' bytes; 0: none */
  uint64_t iterations_per_round;  /* iterations between admissions; 0: 4 */
} cmn_server_config;

typedef struct {
  uint64_t submitted, admitted, completed, queued, running;
  uint64_t converged;          /* completed requests that closed the gap */
  uint64_t boxes;              /* child boxes bounded for completed requests */
  uint64_t rounds;             /* admission rounds of the worker */
  uint64_t pool_bytes_in_use, pool_bytes_peak, pool_budget_bytes;
  double latency_p50_ms, latency_p99_ms, latency_mean_ms, latency_max_ms;
  double queue_p50_ms, queue_p99_ms;  /* submit -> admission */
  double wall_ms;              /* first submit -> last completion */
  double boxes_per_s;          /* boxes / wall_ms */
} cmn_server_stats;

cmn_status cmn_server_create(const cmn_server_config* config,
                             cmn_server** out);
/* Stops the worker (running requests are abandoned) and frees everything. */
void cmn_server_destroy(cmn_server* server);
/* Queues a solve of `problem` (which must outlive the request).  `opts`
 * shared options must equal the server's; CMN_INVALID_CONFIGURATION when
 * no class takes the problem.  A finished request's outcome and best point
 * (a few hundred bytes of host memory plus 8 per variable) stay readable until the
 * server is destroyed, so a long-running caller recreates the server from
 * time to time. */
cmn_status cmn_server_submit(cmn_server* server, const cmn_problem* problem,
                             const cmn_solve_options* opts,
                             uint64_t* request_id);
/* Non-blocking: `done` is 1 once the request finished; then `out` (its
 * elapsed_ms is submit -> completion) and `best_point` (may be NULL) are
 * filled. */
cmn_status cmn_server_poll(cmn_server* server, uint64_t request_id,
                           int32_t* done, cmn_outcome* out,
                           double* best_point);
/* Blocks until the request finished or `timeout_ms` passed (0: no limit;
 * CMN_TIMEOUT then). */
cmn_status cmn_server_wait(cmn_server* server, uint64_t request_id,
                           uint64_t timeout_ms, cmn_outcome* out,
                           double* best_point);
/* Latency percentiles and throughput over the completed requests. */
cmn_status cmn_server_stats_get(cmn_server* server, cmn_server_stats* out);

#ifdef __cplusplus
}
#endif

#endif /* CUMINLP_GB300_H */
