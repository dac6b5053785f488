/*
 * oracle.h -- CPU oracle for the interval branch-and-bound hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (CuMINLPSearch, include/cuminlp/...) used as the checker for
 * the CUDA path and as the timed CPU baseline.  Only tests/, the smoke
 * check and bench.py's CPU-baseline / reference arm may load it.  The
 * product library never links or calls it.
 *
 * Arithmetic: directed rounding is computed exactly with error-free
 * transformations (TwoSum, fma-based TwoProduct) around round-to-nearest
 * operations, so the results are the IEEE-754 correctly rounded
 * round-down / round-up values on any host, independent of the compiler's
 * handling of the floating-point environment.  Build with
 * -ffp-contract=off.
 */
#ifndef CUMINLP_ORACLE_H
#define CUMINLP_ORACLE_H

#include <stdint.h>

#include "../include/cuminlp_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_problem orc_problem;

/* Returns NULL (and an error string via orc_last_error) on a malformed
 * problem; validation follows Problem::validate() (model/problem.hpp:282). */
orc_problem* orc_problem_create(const cmn_problem_desc* desc);
void orc_problem_destroy(orc_problem* p);
const char* orc_last_error(void);
int64_t orc_buffer_node_count(const orc_problem* p);

/* ---- primitive directed-rounding operations (for exact-arithmetic pins) */
double orc_add_rd(double a, double b);
double orc_add_ru(double a, double b);
double orc_mul_rd(double a, double b);
double orc_mul_ru(double a, double b);
double orc_div_rd(double a, double b);
double orc_div_ru(double a, double b);
float orc_addf_rd(float a, float b);
float orc_addf_ru(float a, float b);
float orc_mulf_rd(float a, float b);
float orc_mulf_ru(float a, float b);
float orc_d2f_rd(double a);
float orc_d2f_ru(double a);

/* Interval op on [alo,ahi] (op) [blo,bhi]; `op` is a cmn_op. */
void orc_interval_op_f64(int op, double alo, double ahi, double blo,
                         double bhi, int int_exp, double* lo, double* hi);
void orc_interval_op_f32(int op, float alo, float ahi, float blo, float bhi,
                         int int_exp, float* lo, float* hi);

/* ---- evaluation -------------------------------------------------------- */
/* Every node enclosure on one box (box = n_vars interleaved lb,ub pairs).
 * Nodes no root reaches, and Const nodes, get NaN. */
int orc_eval_nodes_f64(const orc_problem* p, const double* box,
                       double* node_lo, double* node_hi);
/* FP32 screen enclosure of every node (outward-rounded inputs/constants). */
int orc_eval_nodes_f32(const orc_problem* p, const double* box,
                       float* node_lo, float* node_hi);
/* SoA batch: lo/hi are n_vars planes of `stride` entries. */
int orc_eval_boxes(const orc_problem* p, int precision, const double* lo,
                   const double* hi, int64_t n_boxes, int64_t stride,
                   double* obj_lb, double* obj_ub, uint8_t* feasible,
                   int threads);
/* Point evaluation: plain round-to-nearest, point feasibility predicates
 * (graph/kernels.cuh:283-320). */
int orc_eval_point(const orc_problem* p, const double* x, double* obj,
                   uint8_t* feasible);

/* ---- region decode and sampler primitives ------------------------------ */
void orc_slot_bounds(int kind, double plo, double phi, uint64_t part,
                     uint64_t fan_out, double* lo, double* hi);
uint64_t orc_sample_hash(uint64_t vid, uint64_t i, uint64_t region,
                         uint64_t salt);
double orc_sample_continuous(double lb, double ub, uint64_t vid, uint64_t i,
                             uint64_t region, uint64_t salt);
double orc_sample_discrete(double lb, double ub, uint64_t vid, uint64_t i,
                           uint64_t region, uint64_t salt);
float orc_sample_continuous_f32(float lb, float ub, uint64_t vid, uint64_t i,
                                uint64_t region, uint64_t salt);
float orc_sample_discrete_f32(float lb, float ub, uint64_t vid, uint64_t i,
                              uint64_t region, uint64_t salt);

/* ---- roles (reference semantics, graph/replay.cuh:823-844) ------------- */
/* The library's compiled FP32 program (cmn_problem_program, precision 1):
 * enables the lazy form's incremental child bounds, derived from it the way
 * the device evaluates them.  Returns 1 when the program has the sum-chain
 * shape they need, else 0 (the lazy form then bounds children node by
 * node). */
int orc_set_program32(orc_problem* p, const void* instrs, int64_t len);
/* The library's compiled FP64 program (cmn_problem_program precision 0):
 * the lazy form's verdict of each expanded box runs it with fused terms,
 * as the device does.  Required for the lazy form. */
int orc_set_program64(orc_problem* p, const void* instrs, int64_t len);
/* One box (n_vars (lo, hi) pairs) through that FP64 program with every
 * operation rounded on its own, as the device's plain form runs it: 1
 * feasible, 0 not, -1 an operator without an interval form, -2 no program
 * set; *lb, *ub the objective's enclosure.  Node-by-node evaluation gives
 * the same enclosures bit for bit (signs of zero aside) when the compiler
 * keeps every node's roundings in their order. */
int orc_program_eval64(const orc_problem* p, const double* box, double* lb, double* ub);
/* The same through the FP32 program (orc_set_program32): variables widened
 * outward, constants as outward pairs, every operation directed in FP32;
 * 1 when no constraint is proven violated (rhs compared in FP64), 0 when
 * one is, -1 / -2 as above.  Equals node-by-node FP32 evaluation. */
int orc_program_eval32(const orc_problem* p, const double* box, double* lb, double* ub);

/* The epilogue (search/epilogue.hpp:89-127, finalise_bounds) over a drop
 * record that folds each dropped lb against the gub it was dropped under
 * (search/budget.hpp:190-209, DropAccounting::fold): fills
 * out->proven_optimal, out->infeasible and out->lower_bound. */
int orc_finalise(double glb, double gub, double tol, int found, int converged, int pending_empty,
                 double frontier_min, uint64_t viable, const double* drop_lbs, const double* drop_gubs,
                 int64_t n_drops, cmn_outcome* out);

/* The lazy form's incremental FP32 bound of every region of one parent
 * box, after orc_set_program32. */
int orc_bound_inc32(const orc_problem* p, const double* box, const uint8_t* slot_kinds, const uint64_t* var_ids,
                    const uint64_t* widths, int64_t slot_count, uint64_t n_regions, uint8_t* feasible,
                    double* obj_lb, double* obj_ub);

int orc_bound(const orc_problem* p, const double* box,
              const uint8_t* slot_kinds, const uint64_t* var_ids,
              const uint64_t* widths, int64_t slot_count, uint64_t n_regions,
              uint8_t* feasible, double* obj_lb, int threads);
/* orc_bound with the host's directed-rounding hardware (the timed CPU
 * path; same results bit for bit). */
int orc_bound_hw(const orc_problem* p, const double* box,
                 const uint8_t* slot_kinds, const uint64_t* var_ids,
                 const uint64_t* widths, int64_t slot_count, uint64_t n_regions,
                 uint8_t* feasible, double* obj_lb, int threads);
/* AggregateBounder::bound_children for one region: k children of
 * n_regions / k contiguous regions each. */
int orc_aggregate_bound(const orc_problem* p, const double* box,
                        const uint8_t* slot_kinds, const uint64_t* var_ids,
                        const uint64_t* widths, int64_t slot_count,
                        uint64_t n_regions, uint64_t k, double* child_lb,
                        double* child_hull_ub, int32_t* child_feasible,
                        int threads);
int orc_sample(const orc_problem* p, const double* box,
               const uint8_t* slot_kinds, const uint64_t* var_ids,
               const uint64_t* widths, int64_t slot_count,
               uint64_t n_regions, uint64_t sample_points, uint64_t salt,
               int32_t* found, double* value, int64_t* index, double* point,
               int threads);
int orc_enumerate(const orc_problem* p, const double* box,
                  const uint8_t* slot_kinds, const uint64_t* var_ids,
                  const uint64_t* widths, int64_t slot_count,
                  uint64_t n_regions, int32_t* found, double* value,
                  int64_t* index, double* point, int threads);

/* ---- policies ----------------------------------------------------------- */
/* BisectionBudgetCompositionPolicy::choose (policy/bisection_budget.hpp:81).
 * Outputs have room for n_vars slots.  Returns the slot count. */
int64_t orc_bisection_choose(const double* box, const int32_t* var_kinds,
                             int64_t n_vars, int64_t B, int64_t max_cycle,
                             int64_t enumerate_cap, int relative,
                             uint8_t* kinds, uint64_t* var_ids,
                             uint64_t* widths, uint64_t* domain_sizes);

/* ---- search ------------------------------------------------------------- */
/* SearchDriver::solve (search/driver.hpp:137-537) restated: best-first,
 * one box per iteration, BisectionBudget policy, roles above. */
int orc_solve_reference(const orc_problem* p, const cmn_solve_options* opts,
                        cmn_outcome* out, double* best_point, int threads);
/* The batched device algorithm, restated on the CPU step for step so the
 * GPU solver can be checked bit for bit. */
int orc_solve_batched(const orc_problem* p, const cmn_solve_options* opts,
                      cmn_outcome* out, double* best_point, int threads);
/* Batched search that stops after `iterations` and dumps the pool:
 * pool_box (count x 2n), pool_lb, pool_depth; returns the pool size. */
int64_t orc_batched_frontier(const orc_problem* p,
                             const cmn_solve_options* opts,
                             uint64_t iterations, double* pool_box,
                             double* pool_lb, uint32_t* pool_depth,
                             int64_t pool_room, cmn_outcome* out,
                             double* best_point, int threads);

#ifdef __cplusplus
}
#endif

#endif
