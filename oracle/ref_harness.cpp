// ref_harness.cpp -- runs the reference's own host code on given inputs.
//
// TEST INFRASTRUCTURE ONLY.  Compiled (by oracle/build_ref.sh) straight
// from the reference sources where they lie, with the one-struct
// cuinterval shim in oracle/ref_shim; the binary lands in oracle/_ref/ and
// is used only to generate golden fixtures under tests/golden/.
//
// Region evaluation comes from the CPU oracle (liboracle), plugged in
// behind the reference's RegionBackendFactory interface
// (backend/backend.hpp:193-219), so the driver, policies, frontier heap,
// history and epilogue that run here are the reference's code.
//
// Commands (all numbers read and written as C99 hex floats / integers):
//   decode  <in> <out>   lines "kind plo phi part fan" -> "lo hi"
//   policy  <in> <out>   BisectionBudget / GreedyEnum choose() cases
//   driver  <in> <out>   SearchDriver::solve on a problem file
//   driverp <in> <out>   the same with any policy make_policy builds
//   aggdriver <in> <out> AggregateDriver::solve (WidestBranchPolicy) on a
//                        problem file, the oracle behind its roles
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "cuminlp/aggregate/driver.hpp"
#include "cuminlp/backend/backend.hpp"
#include "cuminlp/model/problem.hpp"
#include "cuminlp/policy/bisection_budget.hpp"
#include "cuminlp/policy/greedy_enum.hpp"
#include "cuminlp/policy/width_first.hpp"
#include "cuminlp/region/decode.hpp"
#include "cuminlp/search/driver.hpp"

extern "C" {
#include "oracle.h"
}
#include "ref_oracle_roles.hpp"

using namespace cuminlp;
using cmn_oracle_roles::OracleFactory;

static double rd(std::istream& in)
{
  std::string s;
  in >> s;
  return std::strtod(s.c_str(), nullptr);
}

static std::string hx(double x)
{
  char buf[64];
  std::snprintf(buf, sizeof buf, "%a", x);
  return buf;
}

// ---- problem file: the flattened DAG, rebuilt with ExprDAG::emit ------
struct Loaded {
  model::Problem<double> problem;
  std::vector<cmn_node> nodes;
  std::vector<double> lb, ub;
  std::vector<int32_t> kinds;
  std::vector<cmn_constraint> cons;
  orc_problem* orc = nullptr;
};

static void load_problem(std::istream& in, Loaded& L)
{
  size_t n_nodes;
  in >> n_nodes;
  for (size_t i = 0; i < n_nodes; ++i) {
    cmn_node nd{};
    in >> nd.op >> nd.n_in >> nd.in0 >> nd.in1 >> nd.var_index;
    nd.constant = rd(in);
    in >> nd.int_exp;
    L.nodes.push_back(nd);
    model::DAGNodePayload<double> p{};
    if (nd.op == CMN_OP_CONST) p.constant = nd.constant;
    if (nd.op == CMN_OP_VAR) p.var_index = (size_t)nd.var_index;
    if (nd.op == CMN_OP_POWN) p.int_exp = nd.int_exp;
    auto op = static_cast<model::Op>(nd.op);
    if (nd.n_in == 0) L.problem.graph.emit(op, {}, p);
    else if (nd.n_in == 1) L.problem.graph.emit(op, {(size_t)nd.in0}, p);
    else L.problem.graph.emit(op, {(size_t)nd.in0, (size_t)nd.in1}, p);
  }
  size_t n_vars;
  in >> n_vars;
  for (size_t v = 0; v < n_vars; ++v) {
    double lo = rd(in), hi = rd(in);
    int k;
    in >> k;
    L.lb.push_back(lo);
    L.ub.push_back(hi);
    L.kinds.push_back(k);
    L.problem.box_bounds.push_back({lo, hi});
    L.problem.var_kinds.push_back(static_cast<model::VarKind>(k));
  }
  in >> L.problem.objective_root;
  size_t m;
  in >> m;
  for (size_t c = 0; c < m; ++c) {
    cmn_constraint cc{};
    in >> cc.root >> cc.cmp;
    cc.rhs = rd(in);
    L.cons.push_back(cc);
    L.problem.constraints.push_back({(size_t)cc.root, static_cast<model::Cmp>(cc.cmp), cc.rhs});
  }
  L.problem.validate();
  cmn_problem_desc d{};
  d.nodes = L.nodes.data();
  d.n_nodes = (int64_t)L.nodes.size();
  d.var_lb = L.lb.data();
  d.var_ub = L.ub.data();
  d.var_kinds = L.kinds.data();
  d.n_vars = (int64_t)L.lb.size();
  d.objective_root = (int64_t)L.problem.objective_root;
  d.constraints = L.cons.data();
  d.n_constraints = (int64_t)L.cons.size();
  L.orc = orc_problem_create(&d);
  if (!L.orc) throw std::runtime_error(orc_last_error());
}

// ---- commands ----------------------------------------------------------
static int cmd_decode(std::istream& in, std::ostream& out)
{
  int kind;
  while (in >> kind) {
    double plo = rd(in), phi = rd(in);
    size_t part, fan;
    in >> part >> fan;
    cu::interval<double> parent{plo, phi}, child{};
    region::decode::slot_bounds<double>(static_cast<region::SlotKind>(kind), parent, part, fan, child);
    out << hx(child.lb) << ' ' << hx(child.ub) << '\n';
  }
  return 0;
}

// per case: "B <B> <max_cycle> <enum_cap> <relative> <n>" or
// "G <partition_num> <enumerate_cap> <max_cycle> <n>", then n kinds, then
// n (lb ub) pairs.  Output: "<count> (kind vid width dom)*"
static int cmd_policy(std::istream& in, std::ostream& out)
{
  std::string tag;
  while (in >> tag) {
    size_t B = 0, max_cycle = 0, enum_cap = 0, rel = 0, pn = 0, ecap = 0, n = 0;
    if (tag == "B") in >> B >> max_cycle >> enum_cap >> rel >> n;
    else in >> pn >> ecap >> max_cycle >> n;
    std::vector<model::VarKind> kinds(n);
    for (auto& k : kinds) {
      int x;
      in >> x;
      k = static_cast<model::VarKind>(x);
    }
    std::vector<cu::interval<double>> box(n);
    for (auto& b : box) {
      b.lb = rd(in);
      b.ub = rd(in);
    }
    config::SearchCalibration cal{};
    cal.max_cycle_size = max_cycle;
    cal.enumerate_cap = enum_cap;
    region::SlotAssignment a;
    if (tag == "B") {
      policy::BisectionBudgetCompositionPolicy<double> pol(B, cal, rel != 0);
      a = pol.choose(box, kinds);
    } else {
      policy::GreedyEnumCompositionPolicy<double> pol(region::FanOutSpec(pn, ecap), cal);
      a = pol.choose(box, kinds);
    }
    out << a.size();
    for (size_t j = 0; j < a.size(); ++j) {
      size_t dom = a.domain_sizes.empty() ? a.widths[j] : a.domain_sizes[j];
      out << ' ' << (int)a.composition[j] << ' ' << a.var_ids[j] << ' ' << a.widths[j] << ' ' << dom;
    }
    out << '\n';
  }
  return 0;
}

// "<iter_limit> <B> <samples> <tolerance>" then the problem
static int cmd_driver(std::istream& in, std::ostream& out)
{
  uint32_t iter_limit;
  size_t B, samples;
  in >> iter_limit >> B >> samples;
  double tol = rd(in);
  Loaded L;
  load_problem(in, L);
  auto pol = std::make_shared<policy::BisectionBudgetCompositionPolicy<double>>(B);
  auto fac = std::make_shared<OracleFactory>(L.orc);
  search::SearchDriver<double> drv(pol, fac, iter_limit, tol, samples);
  std::streambuf* prev = std::cout.rdbuf();
  std::ostringstream sink;
  std::cout.rdbuf(sink.rdbuf());
  auto o = drv.solve(L.problem);
  std::cout.rdbuf(prev);
  const auto& t = o.counters;
  out << hx(o.lower_bound) << ' ' << hx(o.upper_bound) << ' ' << search::to_string(o.stop_reason) << ' '
      << o.proven_optimal << ' ' << o.infeasible << '\n';
  out << t.iterations << ' ' << t.fathomed << ' ' << t.fathomed_points << ' ' << t.bounded << ' ' << t.sampled << ' '
      << t.enqueued << ' ' << t.witness_rejected << ' ' << t.pruned_duplicate << ' ' << t.pruned_infeasible << ' '
      << t.pruned_dominated << ' ' << t.pending << ' ' << t.viable << '\n';
  out << o.best_point.size();
  for (double x : o.best_point) out << ' ' << hx(x);
  out << '\n';
  orc_problem_destroy(L.orc);
  return 0;
}

// "<policy B|R|G|W> <iter_limit> <B> <partition_num> <enum_cap> <max_cycle>
// <samples> <tolerance>" then the problem: SearchDriver::solve with the
// policy make_policy (policy/greedy_enum.hpp:204-223) builds
static int cmd_driverp(std::istream& in, std::ostream& out)
{
  std::string pk;
  uint32_t iter_limit;
  size_t B, pn, ecap, max_cycle, samples;
  in >> pk >> iter_limit >> B >> pn >> ecap >> max_cycle >> samples;
  double tol = rd(in);
  Loaded L;
  load_problem(in, L);
  policy::PolicyKind kind = policy::PolicyKind::BisectionBudget;
  if (pk == "R") kind = policy::PolicyKind::RelativeBisectionBudget;
  else if (pk == "G") kind = policy::PolicyKind::GreedyEnumerate;
  else if (pk == "W") kind = policy::PolicyKind::WidthFirst;
  config::SearchCalibration cal{};
  cal.max_cycle_size = max_cycle;
  std::shared_ptr<const policy::CompositionPolicy<double>> pol =
      policy::make_policy<double>(kind, region::FanOutSpec(pn, ecap), B, cal);
  auto fac = std::make_shared<OracleFactory>(L.orc);
  search::SearchDriver<double> drv(pol, fac, iter_limit, tol, samples);
  std::streambuf* prev = std::cout.rdbuf();
  std::ostringstream sink;
  std::cout.rdbuf(sink.rdbuf());
  auto o = drv.solve(L.problem);
  std::cout.rdbuf(prev);
  const auto& t = o.counters;
  out << hx(o.lower_bound) << ' ' << hx(o.upper_bound) << ' ' << search::to_string(o.stop_reason) << ' '
      << o.proven_optimal << ' ' << o.infeasible << '\n';
  out << t.iterations << ' ' << t.fathomed << ' ' << t.fathomed_points << ' ' << t.bounded << ' ' << t.sampled << ' '
      << t.enqueued << ' ' << t.witness_rejected << ' ' << t.pruned_duplicate << ' ' << t.pruned_infeasible << ' '
      << t.pruned_dominated << ' ' << t.pending << ' ' << t.viable << '\n';
  out << o.best_point.size();
  for (double x : o.best_point) out << ' ' << hx(x);
  out << '\n';
  orc_problem_destroy(L.orc);
  return 0;
}

// ---- aggregate roles over the oracle ---------------------------------------
class OAggBounder : public aggregate::AggregateBounder<double> {
 public:
  OAggBounder(const orc_problem* p, std::size_t n, std::size_t k) : p_(p), n_(n), k_(k), out_(k) {}
  std::span<const aggregate::AggregateBound<double>> bound_children(
      std::span<const aggregate::AggregateRegion<double>> regions) override
  {
    const auto& launch = regions[0].partition.launch;
    std::vector<uint8_t> kinds;
    for (std::size_t j = 0; j < launch.size(); ++j) kinds.push_back(static_cast<uint8_t>(launch.composition[j]));
    std::vector<uint64_t> v(launch.var_ids.begin(), launch.var_ids.end()), w(launch.widths.begin(), launch.widths.end());
    std::vector<double> lb(k_), ub(k_);
    std::vector<int32_t> fe(k_);
    if (orc_aggregate_bound(p_, reinterpret_cast<const double*>(regions[0].box.data()), kinds.data(), v.data(),
                            w.data(), (int64_t)kinds.size(), n_, k_, lb.data(), ub.data(), fe.data(), 1))
      throw std::runtime_error(orc_last_error());
    for (std::size_t c = 0; c < k_; ++c) out_[c] = aggregate::AggregateBound<double>{lb[c], ub[c], fe[c] != 0};
    return out_;
  }
  std::size_t n_subregions() const override { return n_; }

 private:
  const orc_problem* p_;
  std::size_t n_, k_;
  std::vector<aggregate::AggregateBound<double>> out_;
};

class OAggSampler : public aggregate::AggregateSampler<double> {
 public:
  OAggSampler(const orc_problem* p, std::size_t n, std::size_t s) : p_(p), n_(n), s_(s) {}
  backend::CandidateResult<double> sample(std::span<const aggregate::AggregateRegion<double>> regions,
                                          std::uint64_t salt) override
  {
    const auto& launch = regions[0].partition.launch;
    std::vector<uint8_t> kinds;
    for (std::size_t j = 0; j < launch.size(); ++j) kinds.push_back(static_cast<uint8_t>(launch.composition[j]));
    std::vector<uint64_t> v(launch.var_ids.begin(), launch.var_ids.end()), w(launch.widths.begin(), launch.widths.end());
    point_.resize(regions[0].box.size());
    int32_t found;
    double value;
    int64_t index;
    if (orc_sample(p_, reinterpret_cast<const double*>(regions[0].box.data()), kinds.data(), v.data(), w.data(),
                   (int64_t)kinds.size(), n_, s_, salt, &found, &value, &index, point_.data(), 1))
      throw std::runtime_error(orc_last_error());
    return {found != 0, value, point_, index};
  }
  std::size_t n_samples() const override { return n_ * s_; }

 private:
  const orc_problem* p_;
  std::size_t n_, s_;
  std::vector<double> point_;
};

class OAggCache : public aggregate::AggregateRoleCache<double> {
 public:
  OAggCache(const orc_problem* p, std::size_t n, std::size_t ns, std::size_t k, std::size_t s)
      : bounder_(p, n, k), sampler_(p, ns, s) {}
  aggregate::AggregateBounder<double>& bounder(const region::Composition&) override { return bounder_; }
  aggregate::AggregateSampler<double>& sampler(const region::Composition&) override { return sampler_; }
  std::size_t graphs_built() const override { return 0; }
  std::size_t graphs_rebuilt() const override { return 0; }

 private:
  OAggBounder bounder_;
  OAggSampler sampler_;
};

// "<iter_limit> <k> <N> <Ns> <samples> <rule> <tolerance>" then the problem
static int cmd_aggdriver(std::istream& in, std::ostream& out)
{
  uint32_t iter_limit;
  size_t k, N, Ns, samples;
  std::string rule_name;
  in >> iter_limit >> k >> N >> Ns >> samples >> rule_name;
  double tol = rd(in);
  Loaded L;
  load_problem(in, L);
  auto rule = aggregate::parse_selection_rule(rule_name);
  if (!rule) throw std::runtime_error("unknown selection rule");
  auto pol = std::make_shared<aggregate::WidestBranchPolicy<double>>(k, N);
  auto spol = std::make_shared<aggregate::WidestBranchPolicy<double>>(k, Ns);
  auto cache = std::make_shared<OAggCache>(L.orc, N, Ns, k, samples);
  auto obs = std::make_shared<report::SearchObserver>();
  aggregate::AggregateDriver<double> drv(pol, spol, cache, *rule, iter_limit, tol, 0, obs);
  auto o = drv.solve(L.problem);
  const auto& t = o.counters;
  out << hx(o.lower_bound) << ' ' << hx(o.upper_bound) << ' ' << search::to_string(o.stop_reason) << ' '
      << o.proven_optimal << ' ' << o.infeasible << ' ' << o.selection_rule_engaged << '\n';
  out << t.iterations << ' ' << t.fathomed << ' ' << t.fathomed_points << ' ' << t.bounded << ' ' << t.sampled << ' '
      << t.enqueued << ' ' << t.witness_rejected << ' ' << t.pruned_duplicate << ' ' << t.pruned_infeasible << ' '
      << t.pruned_dominated << ' ' << t.pending << ' ' << t.viable << ' ' << t.history_freed << ' '
      << t.history_peak_live << '\n';
  out << o.best_point.size();
  for (double x : o.best_point) out << ' ' << hx(x);
  out << '\n';
  orc_problem_destroy(L.orc);
  return 0;
}

int main(int argc, char** argv)
{
  if (argc < 4) {
    std::cerr << "usage: ref_harness decode|policy|driver <in> <out>\n";
    return 2;
  }
  std::ifstream in(argv[2]);
  std::ofstream out(argv[3]);
  std::string cmd = argv[1];
  try {
    if (cmd == "decode") return cmd_decode(in, out);
    if (cmd == "policy") return cmd_policy(in, out);
    if (cmd == "driver") return cmd_driver(in, out);
    if (cmd == "driverp") return cmd_driverp(in, out);
    if (cmd == "aggdriver") return cmd_aggdriver(in, out);
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << '\n';
    return 1;
  }
  std::cerr << "unknown command\n";
  return 2;
}
