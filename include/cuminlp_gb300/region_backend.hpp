// region_backend.hpp -- the reference-side binding: a
// cuminlp::backend::RegionBackendFactory<double> (backend/backend.hpp:193-219)
// implemented over the cuminlp_gb300 C ABI, so the reference's own
// SearchDriver / BackendCache run unchanged on the GB300 kernels.
//
// Header-only.  Include it in a translation unit that also sees the
// reference's headers (cuminlp/backend/backend.hpp and friends) and link
// libcuminlp_gb300.so.  C ABI statuses become the reference's exceptions
// (errors.hpp, backend.hpp:275-287).
#pragma once

#include <cstdint>
#include <memory>
#include <span>
#include <string>
#include <vector>

#include "../cuminlp_gb300.h"
// The reference's headers: from its include directory, or already seen by
// this translation unit (a single-header build of the reference).
#if __has_include("cuminlp/backend/backend.hpp")
#include "cuminlp/backend/backend.hpp"
#include "cuminlp/errors.hpp"
#include "cuminlp/model/problem.hpp"
#endif

namespace cuminlp_gb300 {

namespace detail {

inline void throw_status(cmn_status st, const char* where)
{
  const std::string msg = std::string(where) + ": " + cmn_last_error();
  switch (st) {
    case CMN_OK: return;
    case CMN_INVALID_DAG: throw cuminlp::InvalidDAG(msg);
    case CMN_INVALID_PROBLEM: throw cuminlp::InvalidProblem(msg);
    case CMN_SHAPE_MISMATCH: throw cuminlp::ShapeMismatch(msg);
    case CMN_INVALID_CONFIGURATION: throw cuminlp::InvalidConfiguration(msg);
    case CMN_OVER_BUDGET: throw cuminlp::ResourceExhausted(msg);
    default: throw cuminlp::error(msg);
  }
}

// Flattens a reference Problem<double> into the C description.
struct Flat {
  std::vector<cmn_node> nodes;
  std::vector<double> lb, ub;
  std::vector<int32_t> kinds;
  std::vector<cmn_constraint> cons;
  cmn_problem_desc desc{};

  explicit Flat(const cuminlp::model::Problem<double>& p)
  {
    for (const auto& n : p.graph.nodes) {
      cmn_node c{};
      c.op = static_cast<int32_t>(n.op);
      c.n_in = static_cast<int32_t>(n.in.size());
      c.in0 = n.in.size() > 0 ? static_cast<int64_t>(n.in[0]) : -1;
      c.in1 = n.in.size() > 1 ? static_cast<int64_t>(n.in[1]) : -1;
      if (n.op == cuminlp::model::Op::Var) c.var_index = static_cast<int64_t>(n.payload.var_index);
      if (n.op == cuminlp::model::Op::Const) c.constant = n.payload.constant;
      if (n.op == cuminlp::model::Op::PowN) c.int_exp = n.payload.int_exp;
      nodes.push_back(c);
    }
    for (size_t v = 0; v < p.box_bounds.size(); ++v) {
      lb.push_back(p.box_bounds[v].lb);
      ub.push_back(p.box_bounds[v].ub);
      kinds.push_back(static_cast<int32_t>(p.var_kinds[v]));
    }
    for (const auto& c : p.constraints)
      cons.push_back(cmn_constraint{static_cast<int64_t>(c.root_id), static_cast<int32_t>(c.cmp), 0, c.rhs});
    desc.nodes = nodes.data();
    desc.n_nodes = static_cast<int64_t>(nodes.size());
    desc.var_lb = lb.data();
    desc.var_ub = ub.data();
    desc.var_kinds = kinds.data();
    desc.n_vars = static_cast<int64_t>(lb.size());
    desc.objective_root = static_cast<int64_t>(p.objective_root);
    desc.constraints = cons.data();
    desc.n_constraints = static_cast<int64_t>(cons.size());
  }
};

struct ProblemHandle {
  cmn_problem* h = nullptr;
  explicit ProblemHandle(const cuminlp::model::Problem<double>& p)
  {
    Flat f(p);
    throw_status(cmn_problem_create(&f.desc, &h), "cmn_problem_create");
  }
  ~ProblemHandle() { cmn_problem_destroy(h); }
  ProblemHandle(const ProblemHandle&) = delete;
  ProblemHandle& operator=(const ProblemHandle&) = delete;
};

struct RoleHandle {
  std::shared_ptr<ProblemHandle> problem;
  cmn_role* h = nullptr;
  std::size_t n_vars = 0;
  RoleHandle(std::shared_ptr<ProblemHandle> p, int32_t role, const cuminlp::region::Composition& comp,
             std::size_t n_regions, const cuminlp::backend::BuildBudget& budget, std::size_t n)
      : problem(std::move(p)), n_vars(n)
  {
    std::vector<uint8_t> kinds;
    for (auto k : comp) kinds.push_back(static_cast<uint8_t>(k));
    cmn_over_budget facts{};
    const cmn_status st = cmn_role_build(problem->h, role, kinds.data(), static_cast<int64_t>(kinds.size()),
                                         n_regions, budget.bytes, budget.samples_per_region, &h, &facts);
    if (st == CMN_OVER_BUDGET) {
      cuminlp::backend::OverBudget ob;
      ob.role = role == CMN_ROLE_BOUNDER ? "interval graph" : role == CMN_ROLE_SAMPLER ? "point graph" : "exact graph";
      ob.needed_bytes = facts.needed_bytes;
      ob.budget_bytes = facts.budget_bytes;
      ob.n_regions = facts.n_regions;
      ob.elements_per_region = facts.elements_per_region;
      ob.bytes_per_element = facts.bytes_per_element;
      ob.element_breakdown = "verdict bytes per region (fused evaluator)";
      ob.element_inventory = "regions";
      ob.composition = comp;
      throw cuminlp::backend::OverBudgetError(ob);
    }
    throw_status(st, "cmn_role_build");
  }
  ~RoleHandle() { cmn_role_destroy(h); }
};

inline const double* box_ptr(const cuminlp::backend::Region<double>& r)
{
  static_assert(sizeof(cu::interval<double>) == 2 * sizeof(double), "interval layout");
  return reinterpret_cast<const double*>(r.box.data());
}

inline std::vector<uint64_t> u64(const std::vector<std::size_t>& v) { return {v.begin(), v.end()}; }

}  // namespace detail

class Bounder final : public cuminlp::backend::RegionBounder<double> {
 public:
  explicit Bounder(std::unique_ptr<detail::RoleHandle> r) : r_(std::move(r)) {}
  cuminlp::backend::BoundResult<double> bound(const cuminlp::backend::Region<double>& region) override
  {
    const auto v = detail::u64(region.assignment.var_ids), w = detail::u64(region.assignment.widths);
    const uint8_t* fe = nullptr;
    const double* lb = nullptr;
    uint64_t n = 0;
    detail::throw_status(cmn_bound(r_->h, detail::box_ptr(region), v.data(), w.data(), &fe, &lb, &n), "cmn_bound");
    return {std::span<const unsigned char>(fe, n), std::span<const double>(lb, n), n};
  }
  std::size_t n_regions() const override { return cmn_role_n_regions(r_->h); }

 private:
  std::unique_ptr<detail::RoleHandle> r_;
};

class Sampler final : public cuminlp::backend::RegionSampler<double> {
 public:
  explicit Sampler(std::unique_ptr<detail::RoleHandle> r) : r_(std::move(r)) {}
  cuminlp::backend::CandidateResult<double> sample(const cuminlp::backend::Region<double>& region,
                                                   std::uint64_t salt) override
  {
    const auto v = detail::u64(region.assignment.var_ids), w = detail::u64(region.assignment.widths);
    cmn_candidate c{};
    detail::throw_status(cmn_sample(r_->h, detail::box_ptr(region), v.data(), w.data(), salt, &c), "cmn_sample");
    return {c.found != 0, c.value, std::span<const double>(c.point, r_->n_vars), c.index};
  }
  std::size_t n_samples() const override { return cmn_role_n_elements(r_->h); }

 private:
  std::unique_ptr<detail::RoleHandle> r_;
};

class Enumerator final : public cuminlp::backend::RegionEnumerator<double> {
 public:
  explicit Enumerator(std::unique_ptr<detail::RoleHandle> r) : r_(std::move(r)) {}
  cuminlp::backend::CandidateResult<double> enumerate(const cuminlp::backend::Region<double>& region) override
  {
    const auto v = detail::u64(region.assignment.var_ids), w = detail::u64(region.assignment.widths);
    cmn_candidate c{};
    detail::throw_status(cmn_enumerate(r_->h, detail::box_ptr(region), v.data(), w.data(), &c), "cmn_enumerate");
    return {c.found != 0, c.value, std::span<const double>(c.point, r_->n_vars), c.index};
  }
  std::size_t n_points() const override { return cmn_role_n_elements(r_->h); }

 private:
  std::unique_ptr<detail::RoleHandle> r_;
};

// The factory the reference's SearchDriver takes
// (search/driver.hpp:97-134).  One device copy of the problem is made per
// distinct Problem object and shared by every role built for it.
class GB300BackendFactory final : public cuminlp::backend::RegionBackendFactory<double> {
 public:
  cuminlp::backend::BackendCapabilities capabilities() const override { return {true, true}; }

  cuminlp::backend::RegionCostModel cost_model(const cuminlp::model::Problem<double>& p) const override
  {
    cmn_cost_model cm{};
    detail::throw_status(cmn_cost_model_get(handle(p)->h, &cm), "cmn_cost_model_get");
    cuminlp::backend::RegionCostModel out;
    out.sampler_bytes_per_sample = cm.sampler_bytes_per_sample;
    out.bound_bytes_per_region = cm.bound_bytes_per_region;
    out.exact_bytes_per_region = cm.exact_bytes_per_region;
    out.fixed_bytes = cm.fixed_bytes;
    return out;
  }

  cuminlp::backend::SubdivisionBundle<double> build_subdivision(const cuminlp::model::Problem<double>& p,
                                                                const cuminlp::region::Composition& comp,
                                                                std::size_t n_regions,
                                                                const cuminlp::backend::BuildBudget& budget,
                                                                cuminlp::backend::RoleRequest roles) const override
  {
    auto ph = handle(p);
    const std::size_t n = p.box_bounds.size();
    cuminlp::backend::SubdivisionBundle<double> b;
    if (roles.sampler)
      b.sampler = std::make_unique<Sampler>(
          std::make_unique<detail::RoleHandle>(ph, CMN_ROLE_SAMPLER, comp, n_regions, budget, n));
    if (roles.bounder)
      b.bounder = std::make_unique<Bounder>(
          std::make_unique<detail::RoleHandle>(ph, CMN_ROLE_BOUNDER, comp, n_regions, budget, n));
    if (roles.enumerator && cuminlp::region::is_fully_enumerable(comp))
      b.enumerator = std::make_unique<Enumerator>(
          std::make_unique<detail::RoleHandle>(ph, CMN_ROLE_ENUMERATOR, comp, n_regions, budget, n));
    return b;
  }

 private:
  std::shared_ptr<detail::ProblemHandle> handle(const cuminlp::model::Problem<double>& p) const
  {
    if (!problem_ || key_ != &p) {
      problem_ = std::make_shared<detail::ProblemHandle>(p);
      key_ = &p;
    }
    return problem_;
  }
  mutable std::shared_ptr<detail::ProblemHandle> problem_;
  mutable const cuminlp::model::Problem<double>* key_ = nullptr;
};

}  // namespace cuminlp_gb300
