// aggregate_backend.hpp -- the reference-side binding of the aggregate
// search: aggregate::AggregateBounder, AggregateSampler and
// AggregateRoleCache (aggregate/bound.hpp:84-127, aggregate/driver.hpp:79-91)
// implemented over the cuminlp_gb300 C ABI, so the reference's own
// AggregateDriver (aggregate/driver.hpp:137-420) runs unchanged on the GB300
// kernels.
//
// Header-only.  Include it after the reference's headers (or with its
// include directory on the path) and region_backend.hpp's dependencies, and
// link libcuminlp_gb300.so.  The bounder of N subregions folds them into k
// child bounds on the device (cmn_bound_children): only k results cross to
// the host per call.  Roles are built per launch composition, on first use,
// and kept for the life of the cache.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <span>
#include <vector>

#include "region_backend.hpp"
#if __has_include("cuminlp/aggregate/driver.hpp")
#include "cuminlp/aggregate/bound.hpp"
#include "cuminlp/aggregate/driver.hpp"
#endif

namespace cuminlp_gb300 {

namespace detail {

inline std::vector<uint8_t> kinds_of(const cuminlp::region::SlotAssignment& launch)
{
  std::vector<uint8_t> k;
  for (std::size_t j = 0; j < launch.size(); ++j) k.push_back(static_cast<uint8_t>(launch.composition[j]));
  return k;
}

}  // namespace detail

// AggregateBounder over one bounder role of N subregions: bound_children
// for the first (and, in the reference's driver, only) region of the span.
class AggregateBounder final : public cuminlp::aggregate::AggregateBounder<double> {
 public:
  AggregateBounder(std::unique_ptr<detail::RoleHandle> r, std::size_t k) : r_(std::move(r)), k_(k), out_(k) {}

  std::span<const cuminlp::aggregate::AggregateBound<double>> bound_children(
      std::span<const cuminlp::aggregate::AggregateRegion<double>> regions) override
  {
    const auto& region = regions[0];
    const auto& launch = region.partition.launch;
    const auto v = detail::u64(launch.var_ids), w = detail::u64(launch.widths);
    const cmn_aggregate_bound* res = nullptr;
    static_assert(sizeof(cu::interval<double>) == 2 * sizeof(double), "interval layout");
    detail::throw_status(cmn_bound_children(r_->h, reinterpret_cast<const double*>(region.box.data()), v.data(),
                                            w.data(), k_, &res),
                         "cmn_bound_children");
    for (std::size_t c = 0; c < k_; ++c)
      out_[c] = cuminlp::aggregate::AggregateBound<double>{res[c].lb, res[c].hull_ub, res[c].feasible != 0};
    return out_;
  }
  std::size_t n_subregions() const override { return cmn_role_n_regions(r_->h); }

 private:
  std::unique_ptr<detail::RoleHandle> r_;
  std::size_t k_;
  std::vector<cuminlp::aggregate::AggregateBound<double>> out_;
};

// AggregateSampler over one sampler role: the region's launch composition
// decoded and sampled as cmn_sample does for a plain region.
class AggregateSampler final : public cuminlp::aggregate::AggregateSampler<double> {
 public:
  explicit AggregateSampler(std::unique_ptr<detail::RoleHandle> r) : r_(std::move(r)) {}

  cuminlp::backend::CandidateResult<double> sample(
      std::span<const cuminlp::aggregate::AggregateRegion<double>> regions, std::uint64_t salt) override
  {
    const auto& region = regions[0];
    const auto& launch = region.partition.launch;
    const auto v = detail::u64(launch.var_ids), w = detail::u64(launch.widths);
    cmn_candidate c{};
    detail::throw_status(cmn_sample(r_->h, reinterpret_cast<const double*>(region.box.data()), v.data(), w.data(),
                                    salt, &c),
                         "cmn_sample");
    return {c.found != 0, c.value, std::span<const double>(c.point, r_->n_vars), c.index};
  }
  std::size_t n_samples() const override { return cmn_role_n_elements(r_->h); }

 private:
  std::unique_ptr<detail::RoleHandle> r_;
};

// AggregateRoleCache: one bounder (N subregions, k children) and one
// sampler (Ns subregions, S points each) per launch composition.
class AggregateRoleCache final : public cuminlp::aggregate::AggregateRoleCache<double> {
 public:
  AggregateRoleCache(const cuminlp::model::Problem<double>& p, std::size_t n, std::size_t k, std::size_t ns,
                     std::size_t samples, std::size_t budget_bytes = 0)
      : problem_(std::make_shared<detail::ProblemHandle>(p)), n_vars_(p.box_bounds.size()), n_(n), k_(k), ns_(ns),
        s_(samples), budget_(budget_bytes)
  {
  }

  cuminlp::aggregate::AggregateBounder<double>& bounder(const cuminlp::region::Composition& comp) override
  {
    auto& slot = bounders_[key(comp)];
    if (!slot) {
      slot = std::make_unique<AggregateBounder>(
          std::make_unique<detail::RoleHandle>(problem_, CMN_ROLE_BOUNDER, comp, n_, budget(1), n_vars_), k_);
      ++built_;
    }
    return *slot;
  }
  cuminlp::aggregate::AggregateSampler<double>& sampler(const cuminlp::region::Composition& comp) override
  {
    auto& slot = samplers_[key(comp)];
    if (!slot) {
      slot = std::make_unique<AggregateSampler>(
          std::make_unique<detail::RoleHandle>(problem_, CMN_ROLE_SAMPLER, comp, ns_, budget(s_), n_vars_));
      ++built_;
    }
    return *slot;
  }
  std::size_t graphs_built() const override { return built_; }
  std::size_t graphs_rebuilt() const override { return 0; }

 private:
  static std::vector<int> key(const cuminlp::region::Composition& comp)
  {
    std::vector<int> k;
    for (auto c : comp) k.push_back(static_cast<int>(c));
    return k;
  }
  cuminlp::backend::BuildBudget budget(std::size_t samples) const
  {
    cuminlp::backend::BuildBudget b;
    b.bytes = budget_;
    b.samples_per_region = samples;
    return b;
  }

  std::shared_ptr<detail::ProblemHandle> problem_;
  std::size_t n_vars_, n_, k_, ns_, s_, budget_;
  std::size_t built_ = 0;
  std::map<std::vector<int>, std::unique_ptr<AggregateBounder>> bounders_;
  std::map<std::vector<int>, std::unique_ptr<AggregateSampler>> samplers_;
};

}  // namespace cuminlp_gb300
