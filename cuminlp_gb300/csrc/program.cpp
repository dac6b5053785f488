// program.cpp -- validation and the DAG -> fused program compiler.
#include "program.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

namespace cmn {

float d2f_rd(double x)
{
  if (std::isnan(x)) return (float)x;
  float f = (float)x;
  if (std::isinf(f) && !std::isinf(x)) return x > 0 ? FLT_MAX : -INFINITY;
  if ((double)f > x) f = std::nextafter(f, -INFINITY);
  return f;
}

float d2f_ru(double x)
{
  if (std::isnan(x)) return (float)x;
  float f = (float)x;
  if (std::isinf(f) && !std::isinf(x)) return x < 0 ? -FLT_MAX : INFINITY;
  if ((double)f < x) f = std::nextafter(f, INFINITY);
  return f;
}

// FP64 -> FP32 rounded to nearest, ties to even, whatever the host's
// current rounding mode
float d2f_rn(double x)
{
  const float lo = d2f_rd(x), hi = d2f_ru(x);
  if (lo == hi || std::isnan(x)) return lo;
  const double dl = x - (double)lo, dh = (double)hi - x;
  if (dl != dh) return dl < dh ? lo : hi;
  uint32_t bits;
  std::memcpy(&bits, &lo, 4);
  return (bits & 1u) ? hi : lo;
}

static bool is_unary(int op)
{
  return op == CMN_OP_SQR || op == CMN_OP_NEG || op == CMN_OP_EXP || op == CMN_OP_LOG || op == CMN_OP_SQRT ||
         op == CMN_OP_SIN || op == CMN_OP_COS || op == CMN_OP_TANH || op == CMN_OP_POWN || op == CMN_OP_ABS;
}

static bool interval_op(int op)
{
  switch (op) {
    case CMN_OP_ADD: case CMN_OP_SUB: case CMN_OP_MUL: case CMN_OP_DIV: case CMN_OP_SQR:
    case CMN_OP_NEG: case CMN_OP_SQRT: case CMN_OP_POWN: case CMN_OP_ABS: case CMN_OP_MIN:
    case CMN_OP_MAX: case CMN_OP_EXP: case CMN_OP_LOG: case CMN_OP_SIN: case CMN_OP_COS:
    case CMN_OP_TANH: case CMN_OP_POW:
      return true;
    default:
      return false;
  }
}

static const char* op_name(int op)
{
  static const char* names[] = {"Var", "Const", "Add", "Sub", "Mul", "Div", "Sqr", "Neg", "Exp", "Log",
                                "Sqrt", "Sin", "Cos", "Tanh", "PowN", "Pow", "Abs", "Min", "Max"};
  return (op >= 0 && op <= 18) ? names[op] : "?";
}

cmn_status build_host_problem(const cmn_problem_desc* d, HostProblem& p, std::string& err)
{
  if (d == nullptr || d->nodes == nullptr || d->n_nodes <= 0) {
    err = "empty DAG";
    return CMN_INVALID_DAG;
  }
  p.nodes.assign(d->nodes, d->nodes + d->n_nodes);
  if (d->n_vars > 0) {
    if (!d->var_lb || !d->var_ub || !d->var_kinds) {
      err = "missing variable bounds or kinds";
      return CMN_INVALID_PROBLEM;
    }
    p.var_lb.assign(d->var_lb, d->var_lb + d->n_vars);
    p.var_ub.assign(d->var_ub, d->var_ub + d->n_vars);
    p.var_kinds.assign(d->var_kinds, d->var_kinds + d->n_vars);
  }
  if (d->n_constraints > 0) {
    if (!d->constraints) {
      err = "missing constraints";
      return CMN_INVALID_PROBLEM;
    }
    p.constraints.assign(d->constraints, d->constraints + d->n_constraints);
  }
  p.objective_root = d->objective_root;
  const int64_t n = (int64_t)p.nodes.size();

  // graph bookkeeping (model/problem.hpp:286-307)
  int64_t var_nodes = 0;
  for (int64_t i = 0; i < n; ++i) {
    const cmn_node& nd = p.nodes[i];
    if (nd.op < 0 || nd.op > CMN_OP_MAX) {
      err = "node " + std::to_string(i) + " has an unknown op";
      return CMN_INVALID_DAG;
    }
    const int need = (nd.op == CMN_OP_VAR || nd.op == CMN_OP_CONST) ? 0 : (is_unary(nd.op) ? 1 : 2);
    if (nd.n_in != need) {
      err = "node " + std::to_string(i) + " (" + op_name(nd.op) + ") has " + std::to_string(nd.n_in) +
            " operands, expected " + std::to_string(need);
      return CMN_INVALID_DAG;
    }
    if ((need >= 1 && (nd.in0 < 0 || nd.in0 >= i)) || (need >= 2 && (nd.in1 < 0 || nd.in1 >= i))) {
      err = "DAG node operand id is not strictly less than the node's own id; topological-order invariant "
            "violated";
      return CMN_INVALID_DAG;
    }
    if (nd.op == CMN_OP_VAR) {
      if (nd.var_index != var_nodes) {
        err = "Var nodes must carry var_index 0, 1, ... in node order";
        return CMN_INVALID_DAG;
      }
      ++var_nodes;
    }
    if (nd.op == CMN_OP_POWN && (nd.int_exp < -32768 || nd.int_exp > 32767)) {
      err = "PowN exponent out of range";
      return CMN_INVALID_DAG;
    }
  }
  if (var_nodes != (int64_t)p.var_lb.size()) {
    err = "box_bounds/var_kinds are out of sync with the number of Op::Var nodes";
    return CMN_INVALID_DAG;
  }
  if (p.objective_root >= 0 && p.objective_root < n && p.nodes[p.objective_root].op == CMN_OP_CONST) {
    err = "objective root is a bare Const; set_objective was given a fixed() value rather than an expression to "
          "optimise";
    return CMN_INVALID_DAG;
  }
  for (const auto& c : p.constraints) {
    if (c.root < 0 || c.root >= n) {
      err = "constraint root out of range";
      return CMN_INVALID_DAG;
    }
    if (p.nodes[c.root].op == CMN_OP_CONST) {
      err = "constraint root is a bare Const; add_constraint was given a fixed() value rather than an expression";
      return CMN_INVALID_DAG;
    }
    if (c.cmp != CMN_CMP_LE && c.cmp != CMN_CMP_EQ) {
      err = "constraint comparison must be LE or EQ";
      return CMN_INVALID_PROBLEM;
    }
  }
  // problem-level checks (model/problem.hpp:324-354)
  if (p.var_lb.empty()) {
    err = "Problem has zero variables";
    return CMN_INVALID_PROBLEM;
  }
  if (p.objective_root < 0 || p.objective_root >= n) {
    err = "Problem's objective was never set (set_objective was never called)";
    return CMN_INVALID_PROBLEM;
  }
  for (size_t i = 0; i < p.var_lb.size(); ++i) {
    const double lb = p.var_lb[i], ub = p.var_ub[i];
    if (!(lb <= ub)) {
      err = "variable's lower bound exceeds its upper bound";
      return CMN_INVALID_PROBLEM;
    }
    const int k = p.var_kinds[i];
    if (k != CMN_VAR_CONTINUOUS && k != CMN_VAR_INTEGER && k != CMN_VAR_BINARY) {
      err = "unknown variable kind";
      return CMN_INVALID_PROBLEM;
    }
    if (k == CMN_VAR_INTEGER || k == CMN_VAR_BINARY) {
      if (std::floor(lb) < lb || std::floor(ub) < ub) {
        err = "Integer/Binary variable has non-integer-valued bounds";
        return CMN_INVALID_PROBLEM;
      }
    }
    if (k == CMN_VAR_BINARY && (lb < 0 || lb > 0 || ub < 1 || ub > 1)) {
      err = "Binary variable's bounds are not exactly [0,1]";
      return CMN_INVALID_PROBLEM;
    }
  }
  for (const auto& c : p.constraints) {
    if (!std::isfinite(c.rhs)) {
      err = "constraint rhs must be finite";
      return CMN_INVALID_PROBLEM;
    }
  }
  if (p.var_lb.size() > 60000) {
    err = "more than 60000 variables";
    return CMN_INVALID_PROBLEM;
  }

  // reachability (backend/graph/cost.hpp:38-68)
  p.reach.assign(n, 0);
  p.reach[p.objective_root] = 1;
  for (const auto& c : p.constraints) p.reach[c.root] = 1;
  p.buffer_node_count = 0;
  for (int64_t i = n - 1; i >= 0; --i) {
    if (!p.reach[i]) continue;
    const cmn_node& nd = p.nodes[i];
    if (nd.n_in >= 1) p.reach[nd.in0] = 1;
    if (nd.n_in >= 2) p.reach[nd.in1] = 1;
    if (nd.op != CMN_OP_CONST) ++p.buffer_node_count;
  }
  for (int64_t i = 0; i < n; ++i) {
    if (!p.reach[i]) continue;
    const cmn_node& nd = p.nodes[i];
    if ((is_unary(nd.op)) && p.nodes[nd.in0].op == CMN_OP_CONST) {
      err = std::string(op_name(nd.op)) + " applied directly to an Op::Const";
      return CMN_INVALID_DAG;
    }
  }
  return CMN_OK;
}

namespace {

enum State : uint8_t { kNone, kVarS, kConstS, kSlotS, kAccS, kDeferred, kAbsorbed };

struct TermForm {
  bool ok = false;
  uint8_t pkind = 0;  // kTermProd / kTermSqr / kTermVar
  bool has_c = false;
  double c = 0;
  uint16_t a = 0, b = 0;
  int64_t inner = -1;  // absorbed product node, if any
};

class Compiler {
 public:
  Compiler(const HostProblem& p, Program& out) : p_(p), out_(out) {}

  void run()
  {
    const int64_t n = (int64_t)p_.nodes.size();
    uses_.assign(n, 0);
    state_.assign(n, kNone);
    slot_of_.assign(n, -1);
    form_.assign(n, TermForm{});
    consumer_.assign(n, -1);
    for (int64_t i = 0; i < n; ++i) {
      if (!p_.reach[i]) continue;
      const cmn_node& nd = p_.nodes[i];
      if (nd.n_in >= 1) {
        ++uses_[nd.in0];
        consumer_[nd.in0] = i;
      }
      if (nd.n_in >= 2) {
        ++uses_[nd.in1];
        consumer_[nd.in1] = i;
      }
    }
    ++uses_[p_.objective_root];
    for (const auto& c : p_.constraints) ++uses_[c.root];
    // roots are consumed by their checks, never by a chain
    is_root_.assign(n, 0);
    is_root_[p_.objective_root] = 1;
    for (const auto& c : p_.constraints) is_root_[c.root] = 1;

    // algorithmic op counts (weights: add/sub 2, scalar*interval 2,
    // interval*interval 8, sqr 2, neg 0, feasibility 1 compare)
    for (int64_t i = 0; i < n; ++i) {
      if (!p_.reach[i]) continue;
      const cmn_node& nd = p_.nodes[i];
      switch (nd.op) {
        case CMN_OP_VAR: case CMN_OP_CONST: break;
        case CMN_OP_ADD: case CMN_OP_SUB: out_.flops_per_box += 2; out_.point_flops_per_box += 1; break;
        case CMN_OP_MUL: {
          const bool sc = p_.nodes[nd.in0].op == CMN_OP_CONST || p_.nodes[nd.in1].op == CMN_OP_CONST;
          out_.flops_per_box += sc ? 2 : 8;
          out_.point_flops_per_box += 1;
          break;
        }
        case CMN_OP_SQR: out_.flops_per_box += 2; out_.point_flops_per_box += 1; break;
        case CMN_OP_NEG: break;
        case CMN_OP_DIV: out_.flops_per_box += 8; out_.point_flops_per_box += 1; break;
        default: out_.flops_per_box += 2; out_.point_flops_per_box += 1; break;
      }
      if (!(nd.op == CMN_OP_VAR || nd.op == CMN_OP_CONST) && !interval_op(nd.op) && out_.interval_supported) {
        out_.interval_supported = false;
        out_.unsupported_op = op_name(nd.op);
      }
    }
    out_.flops_per_box += (double)p_.constraints.size();
    out_.point_flops_per_box += (double)p_.constraints.size();

    classify_terms();
    emit_all();
    out_.n_slots = max_slots_;
    build_schedule();
    build_incremental();
    out_.code32 = out_.code64;
    out_.code32p = out_.code64;
    for (size_t k = 0; k < out_.code64.size(); ++k) {
      Instr& s = out_.code32[k];
      Instr& q = out_.code32p[k];
      const Instr& d = out_.code64[k];
      const int code = d.head & 7;
      if (code == kOpCheck) continue;  // rhs stays FP64
      const bool has_const = code == kOpTerm || code == kOpConstToSlot ||
                             (code == kOpGeneric && ((d.modes & 3) == kModeConst || ((d.modes >> 2) & 3) == kModeConst)) ||
                             (code == kOpLoadAcc && (d.modes & 3) == kModeConst) ||
                             (code == kOpObjective && (d.modes & 3) == kModeConst);
      if (has_const) {
        const double c = d.c;
        s.c32.clo = d2f_rd(c);
        s.c32.chi = d2f_ru(c);
        q.c32.clo = d2f_rn(c);
        q.c32.chi = q.c32.clo;
      }
    }
  }

 private:
  // Splits a slot-free program at every accumulator reset (a chain's first
  // TERM, or LoadAcc) into independent segments, then assigns them to the
  // lanes of groups of 2..32 lanes, longest first, each to the lane with
  // the least work so far.
  void build_schedule()
  {
    const int len = (int)out_.code64.size();
    if (out_.n_slots != 0 || len == 0) return;
    std::vector<std::pair<int, int>> segs;
    int start = 0;
    for (int pc = 1; pc < len; ++pc) {
      const Instr& in = out_.code64[pc];
      const int code = in.head & 7, sub = in.head >> 3;
      if ((code == kOpTerm && (sub & kTermInit)) || code == kOpLoadAcc) {
        segs.push_back({start, pc});
        start = pc;
      }
    }
    segs.push_back({start, len});
    // a point stops at its first violated constraint: the segments that
    // hold the objective come last in every lane's list (level 0: one lane,
    // program order otherwise)
    auto holds_objective = [&](const std::pair<int, int>& sg) {
      for (int pc = sg.first; pc < sg.second; ++pc)
        if ((out_.code64[pc].head & 7) == kOpObjective) return true;
      return false;
    };
    const std::vector<std::pair<int, int>> in_order = segs;
    std::stable_sort(segs.begin(), segs.end(), [](const std::pair<int, int>& a, const std::pair<int, int>& b) {
      return (a.second - a.first) > (b.second - b.first);
    });
    const int ns = (int)segs.size();
    out_.n_segments = ns;
    out_.sched.assign(6, 0);
    out_.makespan.assign(6, 0);
    out_.makespan[0] = len;
    out_.sched[0] = (int32_t)out_.sched.size();
    out_.sched.push_back(0);
    out_.sched.push_back(ns);
    for (int pass = 0; pass < 2; ++pass)
      for (const auto& sg : in_order)
        if (holds_objective(sg) == (pass == 1)) {
          out_.sched.push_back(sg.first);
          out_.sched.push_back(sg.second);
        }
    for (int l = 1; l <= 5; ++l) {
      const int G = 1 << l;
      std::vector<std::vector<int>> lanes(G);
      std::vector<int64_t> load(G, 0);
      for (int j = 0; j < ns; ++j) {
        int best = 0;
        for (int q = 1; q < G; ++q)
          if (load[q] < load[best]) best = q;
        lanes[best].push_back(j);
        load[best] += segs[j].second - segs[j].first;
      }
      out_.makespan[l] = *std::max_element(load.begin(), load.end());
      out_.sched[l] = (int32_t)out_.sched.size();
      int32_t acc = 0;
      out_.sched.push_back(0);
      for (int q = 0; q < G; ++q) {
        acc += (int32_t)lanes[q].size();
        out_.sched.push_back(acc);
      }
      for (int q = 0; q < G; ++q)
        for (int pass = 0; pass < 2; ++pass)
          for (int j : lanes[q])
            if (holds_objective(segs[j]) == (pass == 1)) {
              out_.sched.push_back(segs[j].first);
              out_.sched.push_back(segs[j].second);
            }
    }
    // more lanes per box only while they cut the busiest lane's work by a
    // fifth or more
    out_.group_max = 1;
    for (int l = 1; l <= 5; ++l) {
      if (out_.makespan[l] * 5 > out_.makespan[l - 1] * 4) break;
      out_.group_max = 1 << l;
    }
  }

  // Segments of a slot-free program as sum chains plus their readers, and
  // per (variable, segment) the chain instructions that read the variable
  // (Program::inc_*).  Leaves inc_ok false for any other shape.
  void build_incremental()
  {
    const std::vector<Instr>& code = out_.code64;
    const int len = (int)code.size();
    const int n = (int)p_.n_vars();
    if (out_.n_slots != 0 || len == 0) return;
    auto accumulates = [](const Instr& in) {
      const int code = in.head & 7;
      return code == kOpTerm || code == kOpLoadAcc;
    };
    auto starts = [](const Instr& in) {
      const int code = in.head & 7, sub = in.head >> 3;
      return (code == kOpTerm && (sub & kTermInit)) || code == kOpLoadAcc;
    };
    std::vector<int32_t> seg;
    int pc = 0;
    while (pc < len) {
      const int b = pc;
      int t = pc;
      if (starts(code[pc])) {
        t = pc + 1;
        while (t < len && accumulates(code[t]) && !starts(code[t])) ++t;
      }
      int e = t;
      while (e < len && !accumulates(code[e])) {
        const int c = code[e].head & 7;
        if (c != kOpCheck && c != kOpObjective) return;  // slots or other forms
        ++e;
      }
      if (e == b) return;  // an accumulating instruction that does not start a chain
      seg.push_back(b);
      seg.push_back(t);
      seg.push_back(e);
      pc = e;
    }
    const int S = (int)seg.size() / 3;
    std::vector<std::vector<int32_t>> lists((size_t)n * S);
    for (int s = 0; s < S; ++s) {
      for (int q = seg[3 * s]; q < seg[3 * s + 1]; ++q) {
        const Instr& in = code[q];
        const int c = in.head & 7;
        int va = -1, vb = -1;
        if (c == kOpTerm) {
          va = in.a;
          vb = in.b;
        } else if ((in.modes & 3) == kModeVar) {  // LoadAcc of a variable
          va = vb = in.a;
        }
        if (va >= n || vb >= n) return;
        if (va >= 0) lists[(size_t)va * S + s].push_back(q);
        if (vb >= 0 && vb != va) lists[(size_t)vb * S + s].push_back(q);
      }
    }
    out_.inc_seg = seg;
    out_.inc_segments = S;
    out_.inc_off.assign((size_t)n * S + 1, 0);
    out_.inc_pcs.clear();
    for (size_t i = 0; i < lists.size(); ++i) {
      out_.inc_off[i] = (int32_t)out_.inc_pcs.size();
      out_.inc_pcs.insert(out_.inc_pcs.end(), lists[i].begin(), lists[i].end());
    }
    out_.inc_off[lists.size()] = (int32_t)out_.inc_pcs.size();
    out_.inc_ok = true;
  }

  bool is_var(int64_t id) const { return p_.nodes[id].op == CMN_OP_VAR; }
  bool is_const(int64_t id) const { return p_.nodes[id].op == CMN_OP_CONST; }

  // P-form of a node built only from variables: x*y, sqr(x), x.
  bool pform(int64_t id, uint8_t& pk, uint16_t& a, uint16_t& b) const
  {
    const cmn_node& nd = p_.nodes[id];
    if (nd.op == CMN_OP_VAR) {
      pk = kTermVar;
      a = b = (uint16_t)nd.var_index;
      return true;
    }
    if (nd.op == CMN_OP_MUL && is_var(nd.in0) && is_var(nd.in1)) {
      pk = kTermProd;
      a = (uint16_t)p_.nodes[nd.in0].var_index;
      b = (uint16_t)p_.nodes[nd.in1].var_index;
      return true;
    }
    if (nd.op == CMN_OP_SQR && is_var(nd.in0)) {
      pk = kTermSqr;
      a = b = (uint16_t)p_.nodes[nd.in0].var_index;
      return true;
    }
    return false;
  }

  // A node whose single consumer is an Add/Sub and whose value is c*P or P
  // is evaluated inside that consumer's term instruction (deferred); the
  // inner P of a c*P term is absorbed into it.
  void classify_terms()
  {
    const int64_t n = (int64_t)p_.nodes.size();
    for (int64_t i = 0; i < n; ++i) {
      if (!p_.reach[i] || is_var(i) || is_const(i)) continue;
      if (uses_[i] != 1 || is_root_[i]) continue;
      const int64_t cons = consumer_[i];
      if (cons < 0) continue;
      const int cop = p_.nodes[cons].op;
      if (cop != CMN_OP_ADD && cop != CMN_OP_SUB) continue;
      const cmn_node& nd = p_.nodes[i];
      TermForm f;
      uint8_t pk;
      uint16_t a, b;
      if (nd.op == CMN_OP_MUL && (is_const(nd.in0) != is_const(nd.in1))) {
        const int64_t c_id = is_const(nd.in0) ? nd.in0 : nd.in1;
        const int64_t x_id = is_const(nd.in0) ? nd.in1 : nd.in0;
        if (pform(x_id, pk, a, b) && (is_var(x_id) || (uses_[x_id] == 1 && !is_root_[x_id]))) {
          f.ok = true;
          f.pkind = pk;
          f.has_c = true;
          f.c = p_.nodes[c_id].constant;
          f.a = a;
          f.b = b;
          f.inner = is_var(x_id) ? -1 : x_id;
        }
      } else if (pform(i, pk, a, b)) {
        f.ok = true;
        f.pkind = pk;
        f.a = a;
        f.b = b;
      }
      if (f.ok) {
        form_[i] = f;
        state_[i] = kDeferred;
        if (f.inner >= 0) state_[f.inner] = kAbsorbed;
      }
    }
  }

  int alloc_slot()
  {
    int s;
    if (!free_slots_.empty()) {
      // lowest free slot keeps the working set compact
      auto it = std::min_element(free_slots_.begin(), free_slots_.end());
      s = *it;
      free_slots_.erase(it);
    } else {
      s = next_slot_++;
    }
    max_slots_ = std::max(max_slots_, s + 1);
    return s;
  }

  void consume(int64_t id)
  {
    if (--uses_[id] == 0) {
      if (state_[id] == kSlotS && slot_of_[id] >= 0) {
        free_slots_.push_back(slot_of_[id]);
        slot_of_[id] = -1;
      }
      if (state_[id] == kAccS && acc_holder_ == id) acc_holder_ = -1;
    }
  }

  void emit(const Instr& ins) { out_.code64.push_back(ins); }

  static Instr blank()
  {
    Instr ins;
    std::memset(&ins, 0, sizeof ins);
    return ins;
  }

  // Frees the accumulator: a live value held there moves to a slot.
  void spill_acc()
  {
    if (acc_holder_ < 0) return;
    const int64_t h = acc_holder_;
    acc_holder_ = -1;
    if (uses_[h] <= 0) return;
    const int s = alloc_slot();
    Instr ins = blank();
    ins.head = make_head(kOpStoreAcc, 0);
    ins.dst = (uint16_t)s;
    emit(ins);
    state_[h] = kSlotS;
    slot_of_[h] = s;
  }

  // Ensures `id` is readable as an operand (slot, var, const or acc).
  void materialise(int64_t id)
  {
    if (state_[id] == kDeferred || state_[id] == kAbsorbed) {
      const TermForm f = form_[id];
      if (state_[id] == kDeferred && f.ok) {
        // evaluate the term generically: P into a slot, then c*P
        if (f.inner >= 0) materialise(f.inner);
        const cmn_node& nd = p_.nodes[id];
        emit_generic(id, nd);
        return;
      }
      emit_generic(id, p_.nodes[id]);
    }
  }

  void operand(int64_t id, uint8_t& mode, uint16_t& idx, Instr& ins)
  {
    switch (state_[id]) {
      case kVarS:
        mode = kModeVar;
        idx = (uint16_t)p_.nodes[id].var_index;
        break;
      case kConstS:
        mode = kModeConst;
        idx = 0;
        ins.c = p_.nodes[id].constant;
        break;
      case kAccS:
        mode = kModeAcc;
        idx = 0;
        break;
      default:
        mode = kModeSlot;
        idx = (uint16_t)slot_of_[id];
        break;
    }
  }

  void emit_generic(int64_t id, const cmn_node& nd)
  {
    int64_t a_id = nd.in0;
    int64_t b_id = nd.n_in >= 2 ? nd.in1 : nd.in0;
    materialise(a_id);
    if (nd.n_in >= 2) materialise(b_id);
    if (nd.n_in >= 2 && state_[a_id] == kConstS && state_[b_id] == kConstS) {
      // both operands constant: stage one of them in a slot
      const int s = alloc_slot();
      Instr ld = blank();
      ld.head = make_head(kOpConstToSlot, 0);
      ld.dst = (uint16_t)s;
      ld.c = p_.nodes[a_id].constant;
      emit(ld);
      Instr ins = blank();
      ins.head = make_head(kOpGeneric, (uint8_t)nd.op);
      uint8_t mb;
      uint16_t ib;
      operand(b_id, mb, ib, ins);
      ins.modes = (uint8_t)(kModeSlot | (mb << 2));
      ins.a = (uint16_t)s;
      ins.b = ib;
      consume(a_id);
      consume(b_id);
      free_slots_.push_back(s);
      ins.dst = (uint16_t)alloc_slot();
      emit(ins);
      state_[id] = kSlotS;
      slot_of_[id] = ins.dst;
      return;
    }
    Instr ins = blank();
    ins.head = make_head(kOpGeneric, (uint8_t)nd.op);
    // unary ops read no second operand: point it at the accumulator so the
    // interpreter's uniform operand fetch never indexes a slot
    uint8_t ma, mb = kModeAcc;
    uint16_t ia, ib = 0;
    operand(a_id, ma, ia, ins);
    if (nd.n_in >= 2) operand(b_id, mb, ib, ins);
    ins.modes = (uint8_t)(ma | (mb << 2));
    ins.a = ia;
    ins.b = ib;
    if (nd.op == CMN_OP_POWN) ins.b = (uint16_t)(int16_t)nd.int_exp;
    consume(a_id);
    if (nd.n_in >= 2) consume(b_id);
    ins.dst = (uint16_t)alloc_slot();
    emit(ins);
    state_[id] = kSlotS;
    slot_of_[id] = ins.dst;
  }

  Instr term_instr(const TermForm& f, uint8_t flags)
  {
    Instr ins = blank();
    uint8_t sub = (uint8_t)(flags | f.pkind | (f.has_c ? kTermHasC : 0));
    ins.head = make_head(kOpTerm, sub);
    ins.a = f.a;
    ins.b = f.b;
    ins.c = f.has_c ? f.c : 0.0;
    ++out_.n_terms;
    return ins;
  }

  // Add/Sub whose operand `t` is a deferred term: fold it into the
  // accumulator.  Returns false when the shape does not fit.
  bool try_chain(int64_t id, const cmn_node& nd)
  {
    const bool is_sub = nd.op == CMN_OP_SUB;
    const int64_t L = nd.in0, R = nd.in1;
    const bool r_term = state_[R] == kDeferred && consumer_[R] == id;
    const bool l_term = state_[L] == kDeferred && consumer_[L] == id;
    if (L == R) return false;
    int64_t base = -1, term = -1;
    uint8_t flag = 0;
    if (r_term) {
      base = L;
      term = R;
      flag = is_sub ? kTermSub : 0;
    } else if (l_term && !is_sub) {
      base = R;
      term = L;
    } else {
      return false;
    }
    // bring `base` into the accumulator
    if (state_[base] == kDeferred && consumer_[base] == id) {
      // both operands are terms: acc = base_term, then acc (+|-)= term
      spill_acc();
      emit(term_instr(form_[base], kTermInit));
      state_[base] = kNone;
    } else if (state_[base] == kAccS && acc_holder_ == base && uses_[base] == 1) {
      // running sum already in the accumulator
    } else {
      materialise(base);
      if (state_[base] == kAccS && acc_holder_ == base) {
        // still needed elsewhere: keep a copy in a slot
        spill_acc();
      }
      spill_acc();
      Instr ld = blank();
      ld.head = make_head(kOpLoadAcc, 0);
      uint8_t m;
      uint16_t ix;
      operand(base, m, ix, ld);
      ld.modes = m;
      ld.a = ix;
      emit(ld);
      consume(base);
      emit(term_instr(form_[term], flag));
      state_[term] = kNone;
      state_[id] = kAccS;
      acc_holder_ = id;
      return true;
    }
    if (state_[base] == kAccS) consume(base);
    emit(term_instr(form_[term], flag));
    state_[term] = kNone;
    state_[id] = kAccS;
    acc_holder_ = id;
    return true;
  }

  void emit_roots(int64_t id)
  {
    if (id == p_.objective_root) {
      Instr ins = blank();
      ins.head = make_head(kOpObjective, 0);
      uint8_t m;
      uint16_t ix;
      operand(id, m, ix, ins);
      ins.modes = m;
      ins.a = ix;
      emit(ins);
      consume(id);
    }
    for (const auto& c : p_.constraints) {
      if (c.root != id) continue;
      Instr ins = blank();
      ins.head = make_head(kOpCheck, (uint8_t)c.cmp);
      uint8_t m;
      uint16_t ix;
      operand(id, m, ix, ins);
      ins.modes = m;
      ins.a = ix;
      ins.c = c.rhs;  // after operand(): a constant operand is impossible here
      emit(ins);
      consume(id);
    }
  }

  void emit_all()
  {
    const int64_t n = (int64_t)p_.nodes.size();
    for (int64_t i = 0; i < n; ++i) {
      if (!p_.reach[i]) continue;
      const cmn_node& nd = p_.nodes[i];
      if (nd.op == CMN_OP_VAR) {
        state_[i] = kVarS;
      } else if (nd.op == CMN_OP_CONST) {
        state_[i] = kConstS;
      } else if (state_[i] == kDeferred || state_[i] == kAbsorbed) {
        // evaluated by its consumer
      } else if ((nd.op == CMN_OP_ADD || nd.op == CMN_OP_SUB) && try_chain(i, nd)) {
        // folded into the accumulator
      } else {
        // a generic node may read the accumulator directly; but if it
        // writes its own result while the accumulator holds a different
        // live value, nothing is lost (generic results go to slots)
        emit_generic(i, nd);
      }
      if (is_root_[i]) emit_roots(i);
    }
  }

  const HostProblem& p_;
  Program& out_;
  std::vector<int> uses_;
  std::vector<uint8_t> state_;
  std::vector<int> slot_of_;
  std::vector<TermForm> form_;
  std::vector<int64_t> consumer_;
  std::vector<uint8_t> is_root_;
  std::vector<int> free_slots_;
  int next_slot_ = 0;
  int max_slots_ = 0;
  int64_t acc_holder_ = -1;
};

}  // namespace

void compile_program(const HostProblem& p, Program& out)
{
  out = Program{};
  Compiler c(p, out);
  c.run();
}

}  // namespace cmn
