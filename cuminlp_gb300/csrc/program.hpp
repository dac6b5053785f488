// program.hpp -- host-side problem model and the DAG -> program compiler.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/cuminlp_gb300.h"
#include "program.h"

namespace cmn {

// A validated, flattened model::Problem<double> (model/problem.hpp:195-358).
struct HostProblem {
  std::vector<cmn_node> nodes;
  std::vector<double> var_lb, var_ub;
  std::vector<int32_t> var_kinds;
  int64_t objective_root = -1;
  std::vector<cmn_constraint> constraints;
  std::vector<uint8_t> reach;  // reachable from a root
  int64_t buffer_node_count = 0;

  int64_t n_vars() const { return (int64_t)var_lb.size(); }
};

// Builds a HostProblem from the C description, applying the checks of
// Problem::validate() (model/problem.hpp:282-355) plus the structural
// checks the reference's GraphBuilder makes at build time
// (graph/builder.cuh:266-271, 466-470, 497-501).  Returns a cmn_status and
// fills `err` on failure.
cmn_status build_host_problem(const cmn_problem_desc* desc, HostProblem& out, std::string& err);

struct Program {
  std::vector<Instr> code64;  // FP64 interval / point program
  std::vector<Instr> code32;  // FP32 outward-rounded screen program
  std::vector<Instr> code32p; // FP32 point program (constants rounded to nearest)
  int n_slots = 0;
  bool interval_supported = true;  // every reachable op has an interval form
  std::string unsupported_op;
  double flops_per_box = 0;        // algorithmic FP64 ops, interval eval
  double point_flops_per_box = 0;  // algorithmic FP64 ops, point eval
  int64_t n_terms = 0;             // fused sum-chain terms
  // Lane schedules for boxes shared by a group of G = 2^l lanes (l = 1..5),
  // built only for programs without slots, whose segments (independent sum
  // chains) can run in any order.  Layout: sched[l] is the offset of level
  // l's block: G + 1 per-lane offsets into the pair list that follows, then
  // (pc0, pc1) pairs in lane order.  Lanes get segments by longest-first
  // greedy assignment (LPT); within a lane, and in level 0 (one lane, the
  // program's order), the segments that hold the objective come last, so a
  // point evaluation stops at a violated constraint before it.
  int n_segments = 0;
  int group_max = 1;               // largest G that still shortens a box's critical path
  std::vector<int32_t> sched;
  std::vector<int64_t> makespan;   // instructions on the busiest lane, per level
  // Incremental child evaluation (the lazy form's FP32 children), built for
  // a slot-free program whose segments are each one sum chain -- a LoadAcc
  // or an initialising TERM, then TERMs -- followed by the checks and the
  // objective that read it.  The chain terms that touch none of a parent's
  // split variables are summed once per parent; each child adds the terms
  // that touch its split variables.
  bool inc_ok = false;
  int inc_segments = 0;
  // per segment s: pcs [inc_seg[3s], inc_seg[3s+1]) accumulate,
  // [inc_seg[3s+1], inc_seg[3s+2]) are its checks / objective
  std::vector<int32_t> inc_seg;
  // the accumulating instructions of segment s that read variable v:
  // inc_pcs[inc_off[v * inc_segments + s] .. inc_off[v * inc_segments + s + 1])
  std::vector<int32_t> inc_off;
  std::vector<int32_t> inc_pcs;
};

// Compiles the reachable DAG into the fused straight-line program.
void compile_program(const HostProblem& p, Program& out);

// Outward conversion of an FP64 constant to an FP32 pair.
float d2f_rd(double x);
float d2f_ru(double x);
float d2f_rn(double x);

}  // namespace cmn
