// ref_gpu.cu -- the reference's own host driver and CUDA graph backend,
// run on the GPU host beside this repository's library.
//
// TEST INFRASTRUCTURE ONLY.  Compiled against oracle/_ref/cuminlp_ref_gpu.cuh,
// the reference's headers as oracle/amalgamate.py writes them (its
// SearchDriver, policies, BackendCache and the whole CUDA graph backend of
// backend/graph/*), with the interval operators of oracle/ref_shim_gpu
// standing in for the un-vendored cuinterval library, and linked with
// libcuminlp_gb300.so through the reference-side adapter
// include/cuminlp_gb300/region_backend.hpp.
//
// Commands (numbers read and written as C99 hex floats / integers; the
// problem file is the flattened DAG of tests/golden/make_golden.py):
//
//   driver <backend> <in> <out>
//       SearchDriver::solve (search/driver.hpp:137-537) with the policy that
//       make_policy (policy/greedy_enum.hpp:204-223) builds, over
//       backend "gb300" (this library, through the adapter), "graph"
//       (the reference's GraphBackendFactory) or "oracle" (the CPU
//       oracle's roles on all host cores, oracle/ref_oracle_roles.hpp).  <in> starts with
//       "<policy B|R|G|W> <iter_limit> <B> <partition_num> <enum_cap>
//        <max_cycle> <samples> <tolerance>".  Writes bounds, stop reason,
//       claims, counters, best point, and the solve's wall time.
//
//   roles <in> <out>
//       Both backends' bounder and sampler built for the composition that
//       BisectionBudget(B) picks on the root box (2^B regions): bound() and
//       sample(salt) on the root region through each, outputs compared bit
//       for bit (feasible flags, lower bounds with +0 == -0, and the
//       candidate: found, value, index, point), and each call timed
//       (median wall time of <reps> calls; every call copies the box in and
//       the results out and synchronises, in both backends).  <in> starts
//       with "<B> <samples> <reps> <n_salts> <roles b|s|bs> <frac>": the
//       region is the root box, or for frac < 1 its part within frac of
//       its half-width around the origin (where the QCQPs' points are
//       feasible).
//
//   aggdriver <in> <out>
//       the reference's AggregateDriver over this library's aggregate roles
//       (include/cuminlp_gb300/aggregate_backend.hpp).
//
//   gams <model.gms> <out> <iter_limit> <B> <parents>
//       the reference's GAMS frontend, then the library's solver on the
//       lowered problem.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "cuminlp_ref_gpu.cuh"
#include "cuminlp_gb300/aggregate_backend.hpp"
#include "cuminlp_gb300/region_backend.hpp"

extern "C" {
#include "oracle.h"
}
#include "ref_oracle_roles.hpp"

using namespace cuminlp;

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

static double now_s()
{
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// the flattened DAG, rebuilt with ExprDAG::emit
static model::Problem<double> load_problem(std::istream& in)
{
  model::Problem<double> P;
  size_t n_nodes;
  in >> n_nodes;
  for (size_t i = 0; i < n_nodes; ++i) {
    int op, n_in;
    long long in0, in1, var_index, int_exp;
    in >> op >> n_in >> in0 >> in1 >> var_index;
    const double constant = rd(in);
    in >> int_exp;
    model::DAGNodePayload<double> p{};
    if (op == CMN_OP_CONST) p.constant = constant;
    if (op == CMN_OP_VAR) p.var_index = (size_t)var_index;
    if (op == CMN_OP_POWN) p.int_exp = (int)int_exp;
    const auto o = static_cast<model::Op>(op);
    if (n_in == 0) P.graph.emit(o, {}, p);
    else if (n_in == 1) P.graph.emit(o, {(size_t)in0}, p);
    else P.graph.emit(o, {(size_t)in0, (size_t)in1}, p);
  }
  size_t n_vars;
  in >> n_vars;
  for (size_t v = 0; v < n_vars; ++v) {
    const double lo = rd(in), hi = rd(in);
    int k;
    in >> k;
    P.box_bounds.push_back({lo, hi});
    P.var_kinds.push_back(static_cast<model::VarKind>(k));
  }
  in >> P.objective_root;
  size_t m;
  in >> m;
  for (size_t c = 0; c < m; ++c) {
    size_t root;
    int cmp;
    in >> root >> cmp;
    const double rhs = rd(in);
    P.constraints.push_back({root, static_cast<model::Cmp>(cmp), rhs});
  }
  P.validate();
  return P;
}

// The oracle's problem behind the "oracle" backend, alive until exit.
struct OracleProblem {
  orc_problem* p = nullptr;
  ~OracleProblem() { orc_problem_destroy(p); }
};

static std::shared_ptr<const backend::RegionBackendFactory<double>> make_backend(const std::string& name,
                                                                                 const model::Problem<double>& P)
{
  if (name == "gb300") return std::make_shared<cuminlp_gb300::GB300BackendFactory>();
  if (name == "graph") return std::make_shared<backend::graph::GraphBackendFactory<double>>();
  if (name == "oracle") {
    // the reference's region work on the host cores: the oracle's roles
    // with the host's directed-rounding hardware, one thread per core
    static OracleProblem held;
    if (held.p) orc_problem_destroy(held.p);
    cuminlp_gb300::detail::Flat f(P);
    held.p = orc_problem_create(&f.desc);
    if (!held.p) throw std::runtime_error(orc_last_error());
    const int threads = (int)std::max(1u, std::thread::hardware_concurrency());
    return std::make_shared<cmn_oracle_roles::OracleFactory>(held.p, threads, true);
  }
  throw std::runtime_error("unknown backend " + name);
}

static int cmd_driver(const std::string& backend_name, std::istream& in, std::ostream& out)
{
  std::string pk;
  uint32_t iter_limit;
  size_t B, pn, ecap, max_cycle, samples;
  in >> pk >> iter_limit >> B >> pn >> ecap >> max_cycle >> samples;
  const double tol = rd(in);
  model::Problem<double> P = load_problem(in);
  policy::PolicyKind kind = policy::PolicyKind::BisectionBudget;
  if (pk == "R") kind = policy::PolicyKind::RelativeBisectionBudget;
  else if (pk == "G") kind = policy::PolicyKind::GreedyEnumerate;
  else if (pk == "W") kind = policy::PolicyKind::WidthFirst;
  config::SearchCalibration cal{};
  cal.max_cycle_size = max_cycle;
  std::shared_ptr<const policy::CompositionPolicy<double>> pol =
      policy::make_policy<double>(kind, region::FanOutSpec(pn, ecap), B, cal);
  search::SearchDriver<double> drv(pol, make_backend(backend_name, P), iter_limit, tol, samples);
  std::streambuf* prev = std::cout.rdbuf();
  std::ostringstream sink;
  std::cout.rdbuf(sink.rdbuf());
  const double t0 = now_s();
  auto o = drv.solve(P);
  const double t1 = now_s();
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
  out << "seconds " << (t1 - t0) << '\n';
  return 0;
}

static bool same_bits(double a, double b)
{
  if (a == 0.0 && b == 0.0) return true;
  if (a != a && b != b) return true;
  uint64_t x, y;
  std::memcpy(&x, &a, 8);
  std::memcpy(&y, &b, 8);
  return x == y;
}

template <class F>
static double median_seconds(int reps, F&& f)
{
  std::vector<double> ts;
  for (int i = 0; i < reps; ++i) {
    const double t0 = now_s();
    f();
    ts.push_back(now_s() - t0);
  }
  std::sort(ts.begin(), ts.end());
  return ts[ts.size() / 2];
}

static int cmd_roles(std::istream& in, std::ostream& out)
{
  size_t B, samples, reps, n_salts;
  std::string which;
  in >> B >> samples >> reps >> n_salts >> which;
  const double frac = rd(in);
  model::Problem<double> P = load_problem(in);
  // the region: the root box, or for frac < 1 the part of it within
  // frac * (half its width) of the origin, integer bounds rounded inward
  std::vector<cu::interval<double>> box = P.box_bounds;
  if (frac < 1.0) {
    for (size_t v = 0; v < box.size(); ++v) {
      const double w = frac * 0.5 * (box[v].ub - box[v].lb);
      double lo = std::max(box[v].lb, -w), hi = std::min(box[v].ub, w);
      if (P.var_kinds[v] != model::VarKind::Continuous) {
        lo = std::ceil(lo);
        hi = std::max(std::floor(hi), lo);
      }
      box[v] = {lo, hi};
    }
  }
  policy::BisectionBudgetCompositionPolicy<double> pol(B);
  const region::SlotAssignment a = pol.choose(box, P.var_kinds);
  size_t n_regions = 1;
  for (size_t w : a.widths) n_regions *= w;
  const backend::Region<double> region{std::span<const cu::interval<double>>(box), a};
  backend::BuildBudget budget;
  budget.samples_per_region = samples;
  out << "n_regions " << n_regions << '\n' << "slots " << a.size() << '\n';
  const bool do_bound = which.find('b') != std::string::npos, do_sample = which.find('s') != std::string::npos;
  std::vector<std::string> names = {"gb300", "graph"};

  if (do_bound) {
    std::vector<std::vector<unsigned char>> fe(2);
    std::vector<std::vector<double>> lb(2);
    for (int b = 0; b < 2; ++b) {
      auto fac = make_backend(names[b], P);
      const double t0 = now_s();
      auto bundle = fac->build_subdivision(P, a.composition, n_regions, budget, backend::RoleRequest{false, true, false});
      out << "bound_build_seconds_" << names[b] << ' ' << (now_s() - t0) << '\n';
      auto r = bundle.bounder->bound(region);
      fe[b].assign(r.feasible.begin(), r.feasible.end());
      lb[b].assign(r.obj_lb.begin(), r.obj_lb.end());
      const double sec = median_seconds((int)reps, [&] { bundle.bounder->bound(region); });
      out << "bound_seconds_" << names[b] << ' ' << sec << '\n';
    }
    size_t bad_fe = 0, bad_lb = 0;
    for (size_t i = 0; i < n_regions; ++i) {
      bad_fe += fe[0][i] != fe[1][i];
      bad_lb += !same_bits(lb[0][i], lb[1][i]);
    }
    out << "bound_mismatch_feasible " << bad_fe << '\n' << "bound_mismatch_lb " << bad_lb << '\n';
    size_t n_feasible = 0;
    for (auto f : fe[1]) n_feasible += f != 0;
    out << "bound_feasible " << n_feasible << '\n';
  }
  if (do_sample) {
    size_t bad = 0;
    std::vector<std::vector<std::string>> rec(2);
    for (int b = 0; b < 2; ++b) {
      auto fac = make_backend(names[b], P);
      const double t0 = now_s();
      auto bundle = fac->build_subdivision(P, a.composition, n_regions, budget, backend::RoleRequest{true, false, false});
      out << "sample_build_seconds_" << names[b] << ' ' << (now_s() - t0) << '\n';
      for (size_t s = 1; s <= n_salts; ++s) {
        auto c = bundle.sampler->sample(region, s);
        std::ostringstream line;
        // the index is CUB's raw output in the reference when nothing is
        // found (and -1 here): compared only with a witness
        line << c.found << ' ' << hx(c.value);
        if (c.found) {
          line << ' ' << c.index;
          for (double x : c.point) line << ' ' << hx(x);
        }
        rec[b].push_back(line.str());
      }
      const double sec = median_seconds((int)reps, [&] { bundle.sampler->sample(region, 1); });
      out << "sample_seconds_" << names[b] << ' ' << sec << '\n';
    }
    size_t found = 0;
    for (size_t s = 0; s < n_salts; ++s) {
      bad += rec[0][s] != rec[1][s];
      found += rec[1][s][0] == '1';
      out << "sample_" << names[1] << ' ' << rec[1][s] << '\n';
    }
    out << "sample_found " << found << '\n';
    out << "sample_mismatch " << bad << '\n';
  }
  return 0;
}

static void print_outcome_lines(std::ostream& out, const search::SolveOutcome<double>& o)
{
  const auto& t = o.counters;
  out << hx(o.lower_bound) << ' ' << hx(o.upper_bound) << ' ' << search::to_string(o.stop_reason) << ' '
      << o.proven_optimal << ' ' << o.infeasible << '\n';
  out << t.iterations << ' ' << t.fathomed << ' ' << t.fathomed_points << ' ' << t.bounded << ' ' << t.sampled << ' '
      << t.enqueued << ' ' << t.witness_rejected << ' ' << t.pruned_duplicate << ' ' << t.pruned_infeasible << ' '
      << t.pruned_dominated << ' ' << t.pending << ' ' << t.viable << '\n';
}

// "<iter_limit> <k> <N> <Ns> <samples> <rule> <tolerance>" then the problem:
// the reference's AggregateDriver (aggregate/driver.hpp:137-420) with
// WidestBranchPolicy, over this library's roles through
// include/cuminlp_gb300/aggregate_backend.hpp
static int cmd_aggdriver(std::istream& in, std::ostream& out)
{
  uint32_t iter_limit;
  size_t k, N, Ns, samples;
  std::string rule_name;
  in >> iter_limit >> k >> N >> Ns >> samples >> rule_name;
  const double tol = rd(in);
  model::Problem<double> P = load_problem(in);
  auto rule = aggregate::parse_selection_rule(rule_name);
  if (!rule) throw std::runtime_error("unknown selection rule");
  auto pol = std::make_shared<aggregate::WidestBranchPolicy<double>>(k, N);
  auto spol = std::make_shared<aggregate::WidestBranchPolicy<double>>(k, Ns);
  auto cache = std::make_shared<cuminlp_gb300::AggregateRoleCache>(P, N, k, Ns, samples);
  auto obs = std::make_shared<report::SearchObserver>();
  aggregate::AggregateDriver<double> drv(pol, spol, cache, *rule, iter_limit, tol, 0, obs);
  const double t0 = now_s();
  auto o = drv.solve(P);
  const double t1 = now_s();
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
  out << "seconds " << (t1 - t0) << '\n';
  return 0;
}

// gams <model.gms> <out> <iter_limit> <B> <parents>: the reference's GAMS
// frontend (source/gams/frontend.cpp) lowers the model; the lowered Problem
// crosses the C ABI (include/cuminlp_gb300/region_backend.hpp's Flat) and
// the library's device-resident solver (cmn_solve) runs on it.  Writes the
// lowering in oracle/ref_gams.cpp's record format, then
//   solve <lb> <ub> <stop_reason> <proven_optimal> <infeasible> <iterations>
//         <expansions> <bounded> <seconds>
// or
//   solve_error <status> <message>
static int cmd_gams(const char* path, std::ostream& out, uint64_t iter_limit, int B, uint64_t parents)
{
  gams::ParsedModel<double> r;
  try {
    r = gams::parse_file<double>(path, {});
  } catch (const gams::ParseError& e) {
    out << "err " << (int)e.kind << ' ' << e.line << '\n';
    return 0;
  }
  const auto& p = r.problem;
  const auto& nodes = p.graph.nodes;
  out << "ok " << (r.sense == gams::Sense::Maximise ? "max" : "min") << ' ' << (r.objvar_kept ? 1 : 0) << ' '
      << nodes.size() << ' ' << p.box_bounds.size() << ' ' << p.constraints.size() << ' ' << r.warnings.size()
      << '\n';
  for (const auto& nd : nodes) {
    const long in0 = nd.in.size() > 0 ? (long)nd.in[0] : -1;
    const long in1 = nd.in.size() > 1 ? (long)nd.in[1] : -1;
    double c = 0.0;
    unsigned long vi = 0;
    int ie = 0;
    if (nd.op == model::Op::Const) c = nd.payload.constant;
    if (nd.op == model::Op::Var) vi = nd.payload.var_index;
    if (nd.op == model::Op::PowN) ie = nd.payload.int_exp;
    out << "node " << (int)nd.op << ' ' << nd.in.size() << ' ' << in0 << ' ' << in1 << ' ' << hx(c) << ' ' << vi
        << ' ' << ie << '\n';
  }
  for (std::size_t i = 0; i < p.box_bounds.size(); ++i)
    out << "var " << hx(p.box_bounds[i].lb) << ' ' << hx(p.box_bounds[i].ub) << ' ' << (int)p.var_kinds[i] << ' '
        << (i < r.var_names.size() ? r.var_names[i] : std::string("?")) << '\n';
  out << "obj " << (std::size_t)p.objective_root << '\n';
  for (std::size_t i = 0; i < p.constraints.size(); ++i)
    out << "con " << (std::size_t)p.constraints[i].root_id << ' ' << (int)p.constraints[i].cmp << ' '
        << hx(p.constraints[i].rhs) << ' '
        << (i < r.constraint_names.size() ? r.constraint_names[i] : std::string("?")) << '\n';
  cuminlp_gb300::detail::Flat f(p);
  cmn_problem* h = nullptr;
  cmn_status st = cmn_problem_create(&f.desc, &h);
  if (st != CMN_OK) {
    out << "solve_error " << (int)st << ' ' << cmn_last_error() << '\n';
    return 0;
  }
  cmn_solve_options o;
  cmn_solve_options_default(&o);
  o.iter_limit = iter_limit;
  o.bisection_budget = B;
  o.batch_parents = parents;
  o.frontier_cap = 1ull << 20;
  cmn_outcome oc{};
  const double t0 = now_s();
  st = cmn_solve(h, &o, &oc, nullptr);
  const double t1 = now_s();
  if (st != CMN_OK) {
    out << "solve_error " << (int)st << ' ' << cmn_last_error() << '\n';
  } else {
    out << "solve " << hx(oc.lower_bound) << ' ' << hx(oc.upper_bound) << ' ' << oc.stop_reason << ' '
        << oc.proven_optimal << ' ' << oc.infeasible << ' ' << oc.counters.iterations << ' '
        << oc.counters.expansions << ' ' << oc.counters.bounded << ' ' << (t1 - t0) << '\n';
  }
  cmn_problem_destroy(h);
  return 0;
}

int main(int argc, char** argv)
{
  if (argc < 4) {
    std::cerr << "usage: ref_gpu driver <gb300|graph> <in> <out> | roles|aggdriver <in> <out> | gams <gms> <out> <iters> <B> <parents>\n";
    return 2;
  }
  const std::string cmd = argv[1];
  try {
    if (cmd == "driver" && argc >= 5) {
      std::ifstream in(argv[3]);
      std::ofstream out(argv[4]);
      return cmd_driver(argv[2], in, out);
    }
    if (cmd == "roles") {
      std::ifstream in(argv[2]);
      std::ofstream out(argv[3]);
      return cmd_roles(in, out);
    }
    if (cmd == "aggdriver") {
      std::ifstream in(argv[2]);
      std::ofstream out(argv[3]);
      return cmd_aggdriver(in, out);
    }
    if (cmd == "gams" && argc >= 7) {
      std::ofstream out(argv[3]);
      return cmd_gams(argv[2], out, std::strtoull(argv[4], nullptr, 10), std::atoi(argv[5]),
                      std::strtoull(argv[6], nullptr, 10));
    }
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << '\n';
    return 1;
  }
  std::cerr << "unknown command\n";
  return 2;
}
