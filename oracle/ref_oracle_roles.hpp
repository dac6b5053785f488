// ref_oracle_roles.hpp -- the CPU oracle behind the reference's region
// role interface (backend/backend.hpp:81-219).
//
// TEST INFRASTRUCTURE ONLY.  Included by the reference harnesses
// (oracle/ref_harness.cpp, oracle/ref_gpu.cu) after the reference's own
// backend.hpp and oracle.h.  Each role forwards one call to liboracle:
// bound() to orc_bound (error-free directed rounding) or, with `hw`, to
// orc_bound_hw (the host's rounding modes, the same results bit for bit);
// sample() and enumerate() to orc_sample / orc_enumerate.  `threads` host
// threads share each call's regions.
#pragma once

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <utility>
#include <vector>

namespace cmn_oracle_roles
{
using namespace cuminlp;

struct OracleRoles {
  const orc_problem* p;
  std::vector<uint8_t> kinds;
  std::size_t n_regions;
  std::size_t samples;
  int threads;
  bool hw;
  std::vector<uint8_t> feas;
  std::vector<double> lb;
  std::vector<double> point;

  void args(const backend::Region<double>& r, std::vector<uint64_t>& vids, std::vector<uint64_t>& widths)
  {
    vids.assign(r.assignment.var_ids.begin(), r.assignment.var_ids.end());
    widths.assign(r.assignment.widths.begin(), r.assignment.widths.end());
  }
};

class OBounder : public backend::RegionBounder<double> {
 public:
  explicit OBounder(OracleRoles r) : r_(std::move(r)) {}
  backend::BoundResult<double> bound(const backend::Region<double>& region) override
  {
    std::vector<uint64_t> v, w;
    r_.args(region, v, w);
    r_.feas.resize(r_.n_regions);
    r_.lb.resize(r_.n_regions);
    const double* box = reinterpret_cast<const double*>(region.box.data());
    const int rc = r_.hw ? orc_bound_hw(r_.p, box, r_.kinds.data(), v.data(), w.data(), (int64_t)r_.kinds.size(),
                                        r_.n_regions, r_.feas.data(), r_.lb.data(), r_.threads)
                         : orc_bound(r_.p, box, r_.kinds.data(), v.data(), w.data(), (int64_t)r_.kinds.size(),
                                     r_.n_regions, r_.feas.data(), r_.lb.data(), r_.threads);
    if (rc) throw std::runtime_error(orc_last_error());
    return {r_.feas, r_.lb, r_.n_regions};
  }
  std::size_t n_regions() const override { return r_.n_regions; }

 private:
  OracleRoles r_;
};

class OSampler : public backend::RegionSampler<double> {
 public:
  explicit OSampler(OracleRoles r) : r_(std::move(r)) {}
  backend::CandidateResult<double> sample(const backend::Region<double>& region, std::uint64_t salt) override
  {
    std::vector<uint64_t> v, w;
    r_.args(region, v, w);
    r_.point.resize(region.box.size());
    int32_t found;
    double value;
    int64_t index;
    if (orc_sample(r_.p, reinterpret_cast<const double*>(region.box.data()), r_.kinds.data(), v.data(), w.data(),
                   (int64_t)r_.kinds.size(), r_.n_regions, r_.samples, salt, &found, &value, &index, r_.point.data(),
                   r_.threads))
      throw std::runtime_error(orc_last_error());
    return {found != 0, value, r_.point, index};
  }
  std::size_t n_samples() const override { return r_.n_regions * r_.samples; }

 private:
  OracleRoles r_;
};

class OEnumerator : public backend::RegionEnumerator<double> {
 public:
  explicit OEnumerator(OracleRoles r) : r_(std::move(r)) {}
  backend::CandidateResult<double> enumerate(const backend::Region<double>& region) override
  {
    std::vector<uint64_t> v, w;
    r_.args(region, v, w);
    r_.point.resize(region.box.size());
    int32_t found;
    double value;
    int64_t index;
    if (orc_enumerate(r_.p, reinterpret_cast<const double*>(region.box.data()), r_.kinds.data(), v.data(),
                      w.data(), (int64_t)r_.kinds.size(), r_.n_regions, &found, &value, &index, r_.point.data(),
                      r_.threads))
      throw std::runtime_error(orc_last_error());
    return {found != 0, value, r_.point, index};
  }
  std::size_t n_points() const override { return r_.n_regions; }

 private:
  OracleRoles r_;
};

class OracleFactory : public backend::RegionBackendFactory<double> {
 public:
  explicit OracleFactory(const orc_problem* p, int threads = 1, bool hw = false) : p_(p), threads_(threads), hw_(hw)
  {
  }
  backend::BackendCapabilities capabilities() const override { return {}; }
  backend::RegionCostModel cost_model(const model::Problem<double>&) const override
  {
    backend::RegionCostModel c;
    c.bound_bytes_per_region = 9;
    c.fixed_bytes = 1;
    return c;
  }
  backend::SubdivisionBundle<double> build_subdivision(const model::Problem<double>&,
                                                       const region::Composition& composition, std::size_t n_regions,
                                                       const backend::BuildBudget& budget,
                                                       backend::RoleRequest roles) const override
  {
    OracleRoles r{p_, {}, n_regions, budget.samples_per_region, threads_, hw_, {}, {}, {}};
    for (auto k : composition) r.kinds.push_back(static_cast<uint8_t>(k));
    backend::SubdivisionBundle<double> b;
    if (roles.sampler) b.sampler = std::make_unique<OSampler>(r);
    if (roles.bounder) b.bounder = std::make_unique<OBounder>(r);
    if (roles.enumerator && region::is_fully_enumerable(composition)) b.enumerator = std::make_unique<OEnumerator>(r);
    return b;
  }

 private:
  const orc_problem* p_;
  int threads_;
  bool hw_;
};
}  // namespace cmn_oracle_roles
