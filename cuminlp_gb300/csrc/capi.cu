// capi.cu -- the C ABI: problems, region roles, raw batched evaluation and
// the device-resident batched solver.  No exception leaves this file.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/cuminlp_gb300.h"
#include "handles.hpp"
#include "kernels.cuh"
#include "batch.hpp"
#include "launch.hpp"
#include "policy.cuh"
#include "program.hpp"
#include "search.hpp"

using namespace cmn;

namespace {

thread_local std::string g_err;

cmn_status fail(cmn_status st, const std::string& msg)
{
  g_err = msg;
  return st;
}

#define CK(call)                                                                                     \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess) return fail(CMN_CUDA_ERROR, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
cudaError_t dalloc(T** p, size_t n)
{
  *p = nullptr;
  if (n == 0) n = 1;
  return cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T));
}

void dfree(void* p)
{
  if (p) cudaFree(p);
}

int g_attr_device_mask = 0;
std::mutex g_attr_mu;

}  // namespace

// ----------------------------------------------------------------------
// device helpers declared in launch.hpp
// ----------------------------------------------------------------------
namespace cmn {

int sm_count()
{
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

int max_dynamic_smem()
{
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return n;
}

}  // namespace cmn

// kernel attribute setup lives with the kernels (eval_kernels.cu)
namespace cmn {
cudaError_t set_eval_kernel_attributes(int max_smem);
int eval_kernel_occupancy(int mode, bool fp32, size_t smem, int threads);
int sample_kernel_occupancy(size_t smem, int threads);
}  // namespace cmn

static cudaError_t ensure_attributes()
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_attr_mu);
  if (dev < 31 && (g_attr_device_mask & (1 << dev))) return cudaSuccess;
  e = set_eval_kernel_attributes(max_dynamic_smem());
  if (e == cudaSuccess) e = set_batch_kernel_attributes(max_dynamic_smem());
  if (e == cudaSuccess && dev < 31) g_attr_device_mask |= (1 << dev);
  return e;
}

// ----------------------------------------------------------------------
// problem
// ----------------------------------------------------------------------
cmn_problem::~cmn_problem()
{
  int cur = 0;
  if (cudaGetDevice(&cur) == cudaSuccess && cur != device) cudaSetDevice(device);
  dfree(d_prog64);
  dfree(d_prog32);
  dfree(d_prog32p);
  dfree(d_kinds);
  dfree(d_root_lb);
  dfree(d_root_ub);
  dfree(d_sched);
  dfree(d_inc_seg);
  dfree(d_inc_off);
  dfree(d_inc_pcs);
  if (cur != device) cudaSetDevice(cur);
}

namespace cmn {
cmn_status set_error(cmn_status st, const std::string& msg) { return fail(st, msg); }
cudaError_t ensure_kernel_attributes() { return ensure_attributes(); }
}  // namespace cmn

extern "C" const char* cmn_last_error(void) { return g_err.c_str(); }

extern "C" const char* cmn_version(void) { return "cuminlp-gb300 0.1 (sm_103a)"; }

extern "C" cmn_status cmn_problem_create(const cmn_problem_desc* desc, cmn_problem** out)
{
  if (out == nullptr) return fail(CMN_INVALID_CONFIGURATION, "null output pointer");
  *out = nullptr;
  try {
    cmn_problem* p = new cmn_problem();
    std::string err;
    cmn_status st = build_host_problem(desc, p->host, err);
    if (st != CMN_OK) {
      delete p;
      return fail(st, err);
    }
    compile_program(p->host, p->prog);
    if (cudaGetDevice(&p->device) != cudaSuccess) {
      delete p;
      return fail(CMN_CUDA_ERROR, "no CUDA device");
    }
    const size_t L = p->prog.code64.size();
    const int64_t n = p->host.n_vars();
    cudaError_t e = dalloc(&p->d_prog64, L);
    if (e == cudaSuccess) e = dalloc(&p->d_prog32, L);
    if (e == cudaSuccess) e = dalloc(&p->d_prog32p, L);
    if (e == cudaSuccess) e = dalloc(&p->d_kinds, (size_t)n);
    if (e == cudaSuccess) e = dalloc(&p->d_root_lb, (size_t)n);
    if (e == cudaSuccess) e = dalloc(&p->d_root_ub, (size_t)n);
    if (e == cudaSuccess && L) e = cudaMemcpy(p->d_prog64, p->prog.code64.data(), L * sizeof(Instr), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && L) e = cudaMemcpy(p->d_prog32, p->prog.code32.data(), L * sizeof(Instr), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && L)
      e = cudaMemcpy(p->d_prog32p, p->prog.code32p.data(), L * sizeof(Instr), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(p->d_kinds, p->host.var_kinds.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(p->d_root_lb, p->host.var_lb.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(p->d_root_ub, p->host.var_ub.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !p->prog.sched.empty()) {
      e = dalloc(&p->d_sched, p->prog.sched.size());
      if (e == cudaSuccess)
        e = cudaMemcpy(p->d_sched, p->prog.sched.data(), p->prog.sched.size() * sizeof(int32_t),
                       cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess && p->prog.inc_ok) {
      auto up = [&](int32_t** d, const std::vector<int32_t>& h) {
        if (e == cudaSuccess) e = dalloc(d, std::max<size_t>(1, h.size()));
        if (e == cudaSuccess && !h.empty())
          e = cudaMemcpy(*d, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
      };
      up(&p->d_inc_seg, p->prog.inc_seg);
      up(&p->d_inc_off, p->prog.inc_off);
      up(&p->d_inc_pcs, p->prog.inc_pcs);
    }
    if (e != cudaSuccess) {
      delete p;
      return fail(CMN_CUDA_ERROR, std::string("uploading the problem: ") + cudaGetErrorString(e));
    }
    *out = p;
    return CMN_OK;
  } catch (const std::bad_alloc&) {
    return fail(CMN_INTERNAL, "host allocation failed");
  } catch (const std::exception& ex) {
    return fail(CMN_INTERNAL, ex.what());
  }
}

extern "C" void cmn_problem_destroy(cmn_problem* p) { delete p; }

extern "C" cmn_status cmn_problem_get_info(const cmn_problem* p, cmn_problem_info* out)
{
  if (!p || !out) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  out->n_vars = p->host.n_vars();
  out->n_constraints = (int64_t)p->host.constraints.size();
  out->n_nodes = (int64_t)p->host.nodes.size();
  out->buffer_node_count = p->host.buffer_node_count;
  out->program_length = (int64_t)p->prog.code64.size();
  out->program_slots = p->prog.n_slots;
  out->flops_per_box = p->prog.flops_per_box;
  out->point_flops_per_box = p->prog.point_flops_per_box;
  out->bytes_per_box = 16.0 * (double)p->host.n_vars() + 17.0;
  out->program_segments = p->prog.n_segments;
  out->lanes_per_box_max = p->prog.group_max;
  return CMN_OK;
}

extern "C" cmn_status cmn_problem_program(const cmn_problem* p, int32_t precision, void* out, int64_t capacity,
                                          int64_t* length)
{
  if (!p || !length) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  if (precision != 0 && precision != 1) return fail(CMN_INVALID_CONFIGURATION, "precision must be 0 or 1");
  const std::vector<Instr>& code = precision == 0 ? p->prog.code64 : p->prog.code32;
  *length = (int64_t)code.size();
  if (out && capacity > 0)
    std::memcpy(out, code.data(), sizeof(Instr) * (size_t)std::min<int64_t>(capacity, (int64_t)code.size()));
  return CMN_OK;
}

extern "C" cmn_status cmn_program_compile(const cmn_problem_desc* desc, int32_t precision, void* out,
                                          int64_t capacity, int64_t* length)
{
  if (!desc || !length) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  if (precision != 0 && precision != 1) return fail(CMN_INVALID_CONFIGURATION, "precision must be 0 or 1");
  try {
    HostProblem host;
    std::string err;
    const cmn_status st = build_host_problem(desc, host, err);
    if (st != CMN_OK) return fail(st, err);
    Program prog;
    compile_program(host, prog);
    const std::vector<Instr>& code = precision == 0 ? prog.code64 : prog.code32;
    *length = (int64_t)code.size();
    if (out && capacity > 0)
      std::memcpy(out, code.data(), sizeof(Instr) * (size_t)std::min<int64_t>(capacity, (int64_t)code.size()));
    return CMN_OK;
  } catch (const std::bad_alloc&) {
    return fail(CMN_INTERNAL, "host allocation failed");
  } catch (const std::exception& ex) {
    return fail(CMN_INTERNAL, ex.what());
  }
}

static cmn_status check_interval(const cmn_problem* p)
{
  if (!p->prog.interval_supported)
    return fail(CMN_INVALID_CONFIGURATION,
                "op " + p->prog.unsupported_op + " has no interval implementation in this backend");
  return CMN_OK;
}

static cmn_status check_smem(const cmn_problem* p, bool fp32, int max_slots)
{
  const size_t need = eval_smem_bytes(p->prog.n_slots, max_slots, fp32, kEvalThreads);
  if ((int64_t)need > (int64_t)max_dynamic_smem())
    return fail(CMN_INVALID_CONFIGURATION, "the problem's program slots and split variables need " +
                                               std::to_string(need) +
                                               " B of shared memory per block; the device offers " +
                                               std::to_string(max_dynamic_smem()));
  return CMN_OK;
}

// per-role fixed device bytes: staging of one parent + reduction scratch
static uint64_t role_fixed_bytes(const cmn_problem* p)
{
  return (uint64_t)(16 * p->host.n_vars() + 64 * 48 + 4096 * sizeof(Cand) + 8 * p->host.n_vars());
}

// ----------------------------------------------------------------------
// host-side policy and decode, for drivers that run on the host
// ----------------------------------------------------------------------
extern "C" cmn_status cmn_bisection_choose(const double* box, const int32_t* var_kinds, int64_t n_vars,
                                           int32_t budget_bits, uint64_t max_cycle_size, uint64_t enumerate_cap,
                                           int32_t relative_width, uint8_t* slot_kinds, uint64_t* var_ids,
                                           uint64_t* widths, uint64_t* domain_sizes, int64_t* slot_count,
                                           int32_t* fathom)
{
  if (n_vars < 0 || (n_vars > 0 && (!box || !var_kinds)) || !slot_kinds || !var_ids || !widths || !domain_sizes ||
      !slot_count)
    return fail(CMN_INVALID_CONFIGURATION, "null argument");
  if (budget_bits < 1 || budget_bits > 62)
    return fail(CMN_INVALID_CONFIGURATION, "bisection budget must be within [1, 62]");
  if (max_cycle_size > 64) return fail(CMN_INVALID_CONFIGURATION, "max_cycle_size exceeds kMaxSlots (64)");
  try {
    std::vector<EnumCand> ec((size_t)std::max<int64_t>(n_vars, 1));
    std::vector<BisCand> bc((size_t)std::max<int64_t>(n_vars, 1));
    std::vector<uint64_t> heap((size_t)std::max<int64_t>(n_vars, 1));
    std::vector<SlotPlan> sp((size_t)budget_bits);
    const PolicyParams pp = {budget_bits, (int64_t)max_cycle_size, (int64_t)enumerate_cap, relative_width};
    // the interleaved box read as two planes of stride 2
    const ParentInfo pi = bisection_policy(box, box + 1, 2, (int)n_vars, var_kinds, pp, ec.data(), bc.data(),
                                           heap.data(), sp.data());
    for (uint32_t j = 0; j < pi.count; ++j) {
      slot_kinds[j] = (uint8_t)sp[j].kind;
      var_ids[j] = sp[j].vid;
      widths[j] = sp[j].width;
      domain_sizes[j] = sp[j].dom;
    }
    *slot_count = pi.count;
    if (fathom) *fathom = (int32_t)pi.fathom;
    return CMN_OK;
  } catch (const std::bad_alloc&) {
    return fail(CMN_INTERNAL, "host allocation failed");
  }
}

extern "C" void cmn_slot_bounds(int32_t kind, double plo, double phi, uint64_t part, uint64_t fan_out, double* lo,
                                double* hi)
{
  if (!lo || !hi) return;
  if (kind == CMN_SLOT_INTEGER_ENUMERATE || kind == CMN_SLOT_BINARY_ENUMERATE) {
    double value = std::ceil(plo) + (double)part;
    if (value > phi) value = phi;
    *lo = value;
    *hi = value;
    return;
  }
  // the device's FMA form (region/decode.hpp:44-71 as nvcc compiles it)
  const double width = (phi - plo) / (double)fan_out;
  *lo = std::fma(width, (double)part, plo);
  *hi = (part + 1 == fan_out) ? phi : std::fma(width, (double)(part + 1), plo);
}

extern "C" cmn_status cmn_cost_model_get(const cmn_problem* p, cmn_cost_model* out)
{
  if (!p || !out) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  // The fused evaluator keeps every intermediate on chip: per region only
  // the verdict (feasible byte + FP64 lower bound) reaches device memory,
  // and the sampler and enumerator keep nothing per element at all.
  out->sampler_bytes_per_sample = 0;
  out->bound_bytes_per_region = 9;
  out->exact_bytes_per_region = 0;
  out->fixed_bytes = role_fixed_bytes(p);
  return CMN_OK;
}

// ----------------------------------------------------------------------
// roles
// ----------------------------------------------------------------------
struct cmn_role {
  const cmn_problem* p = nullptr;
  int kind = 0;
  std::vector<uint8_t> slot_kinds;
  uint64_t n_regions = 0;
  uint64_t S = 1;
  cudaStream_t stream = nullptr;
  int grid = 1;
  int lg_min = 0;  // sampler: lanes per point column (sample_lg_min)
  // one device block: [box lo planes n][box hi planes n][slots][pinfo]
  unsigned char* d_stage = nullptr;
  unsigned char* h_stage = nullptr;
  size_t stage_bytes = 0;
  uint8_t* d_feas = nullptr;
  double* d_lb = nullptr;
  Cand* d_block_best = nullptr;
  double* d_point = nullptr;
  uint8_t* h_feas = nullptr;
  double* h_lb = nullptr;
  double* h_point = nullptr;
  Cand* h_cand = nullptr;
  // aggregate bounds: 2k fold keys on the device and host, k results
  unsigned long long* d_agg = nullptr;
  unsigned long long* h_agg = nullptr;
  cmn_aggregate_bound* h_agg_out = nullptr;
  uint64_t agg_cap = 0;

  ~cmn_role()
  {
    int cur = 0;
    if (p && cudaGetDevice(&cur) == cudaSuccess && cur != p->device) cudaSetDevice(p->device);
    if (stream) cudaStreamSynchronize(stream);
    dfree(d_agg);
    if (h_agg) cudaFreeHost(h_agg);
    if (h_agg_out) cudaFreeHost(h_agg_out);
    dfree(d_stage);
    dfree(d_feas);
    dfree(d_lb);
    dfree(d_block_best);
    dfree(d_point);
    if (h_stage) cudaFreeHost(h_stage);
    if (h_feas) cudaFreeHost(h_feas);
    if (h_lb) cudaFreeHost(h_lb);
    if (h_point) cudaFreeHost(h_point);
    if (h_cand) cudaFreeHost(h_cand);
    if (stream) cudaStreamDestroy(stream);
    if (p && cur != p->device) cudaSetDevice(cur);
  }
};

static bool is_enum_kind(uint8_t k) { return k == CMN_SLOT_INTEGER_ENUMERATE || k == CMN_SLOT_BINARY_ENUMERATE; }

extern "C" cmn_status cmn_role_build(const cmn_problem* p, int32_t role, const uint8_t* slot_kinds,
                                     int64_t slot_count, uint64_t n_regions, uint64_t budget_bytes,
                                     uint64_t sample_points, cmn_role** out, cmn_over_budget* facts)
{
  if (!p || !out) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  *out = nullptr;
  if (role < CMN_ROLE_BOUNDER || role > CMN_ROLE_ENUMERATOR) return fail(CMN_INVALID_CONFIGURATION, "unknown role");
  if (sample_points < 1)
    return fail(CMN_INVALID_CONFIGURATION,
                "sample_points must be at least 1; a point graph that samples nothing can never produce an incumbent");
  if (slot_count < 0 || slot_count > 64) return fail(CMN_SHAPE_MISMATCH, "slot_count must be within [0, 64]");
  if (slot_count > 0 && !slot_kinds) return fail(CMN_SHAPE_MISMATCH, "missing slot kinds");
  for (int64_t j = 0; j < slot_count; ++j)
    if (slot_kinds[j] > CMN_SLOT_BINARY_ENUMERATE) return fail(CMN_INVALID_CONFIGURATION, "unknown slot kind");
  if (n_regions < 1) return fail(CMN_INVALID_CONFIGURATION, "n_regions must be at least 1");
  if (role == CMN_ROLE_ENUMERATOR) {
    for (int64_t j = 0; j < slot_count; ++j)
      if (!is_enum_kind(slot_kinds[j]))
        return fail(CMN_INVALID_CONFIGURATION, "an enumerator needs a fully enumerable composition");
  }
  cmn_status st = check_interval(p);
  if (st != CMN_OK && role == CMN_ROLE_BOUNDER) return st;
  st = check_smem(p, false, (int)slot_count);
  if (st != CMN_OK) return st;
  try {
    if (cudaSetDevice(p->device) != cudaSuccess) return fail(CMN_CUDA_ERROR, "cudaSetDevice failed");
    CK(ensure_attributes());
    cmn_cost_model cm;
    cmn_cost_model_get(p, &cm);
    const uint64_t S = role == CMN_ROLE_SAMPLER ? sample_points : 1;
    uint64_t per = role == CMN_ROLE_BOUNDER ? cm.bound_bytes_per_region
                   : role == CMN_ROLE_SAMPLER ? cm.sampler_bytes_per_sample * S
                                              : cm.exact_bytes_per_region;
    // saturating, as the reference's estimate is: a fan-out that saturates
    // is over any budget rather than wrapped to an affordable size
    const uint64_t needed = per != 0 && n_regions > (UINT64_MAX - cm.fixed_bytes) / per
                                ? UINT64_MAX
                                : n_regions * per + cm.fixed_bytes;
    uint64_t budget = budget_bytes;
    if (budget == 0) {
      size_t fr = 0, tot = 0;
      CK(cudaMemGetInfo(&fr, &tot));
      budget = fr;
    }
    // Beyond 2^32 regions a role cannot index its launch; like a saturated
    // fan-out in the reference (graph_replay_test.cu:442-461) it is reported
    // as over budget, before anything is allocated, so a driver's cache can
    // evict, retry and finally stop the run as out of device memory.
    const bool too_many = n_regions > (1ULL << 32);
    if (needed > budget || too_many) {
      if (facts) {
        facts->needed_bytes = too_many ? UINT64_MAX : needed;
        facts->budget_bytes = budget;
        facts->n_regions = n_regions;
        facts->elements_per_region = S;
        facts->bytes_per_element = per;
      }
      const char* names[] = {"interval graph", "point graph", "exact graph"};
      if (too_many)
        return fail(CMN_OVER_BUDGET, std::string(names[role]) + " of " + std::to_string(n_regions) +
                                         " regions: a role indexes at most 2^32 regions per launch.");
      return fail(CMN_OVER_BUDGET, std::string(names[role]) + " needs " + std::to_string(needed) +
                                       " B of device memory, but only " + std::to_string(budget) + " B is available.");
    }
    const int lg_min = sample_lg_min((int)p->host.n_vars(), p->prog.n_slots, p->d_sched != nullptr, kEvalThreads);
    if (role != CMN_ROLE_BOUNDER &&
        sample_smem_bytes((int)p->host.n_vars(), p->prog.n_slots, kEvalThreads, lg_min) > (size_t)max_dynamic_smem())
      return fail(CMN_INVALID_CONFIGURATION,
                  "the sampler's per-thread point columns do not fit in shared memory (a program with shared slots "
                  "keeps one column of n_vars + slots doubles per thread)");
    cmn_role* r = new cmn_role();
    r->p = p;
    r->kind = role;
    r->lg_min = lg_min;
    r->slot_kinds.assign(slot_kinds, slot_kinds + slot_count);
    r->n_regions = n_regions;
    r->S = S;
    const int64_t n = p->host.n_vars();
    r->stage_bytes = (size_t)(16 * n) + 64 * sizeof(SlotPlan) + sizeof(ParentInfo);
    cudaError_t e = cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = dalloc(&r->d_stage, r->stage_bytes);
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&r->h_stage), r->stage_bytes);
    const int threads = kEvalThreads;
    const uint64_t blocks_needed = (n_regions * (uint64_t)p->prog.group_max + threads - 1) / threads;
    const int occ = std::max(
        1, eval_kernel_occupancy(0, false, eval_smem_bytes(p->prog.n_slots, (int)slot_count, false, threads), threads));
    r->grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(blocks_needed, (uint64_t)sm_count() * occ));
    if (role == CMN_ROLE_BOUNDER) {
      if (e == cudaSuccess) e = dalloc(&r->d_feas, n_regions);
      if (e == cudaSuccess) e = dalloc(&r->d_lb, n_regions);
      if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&r->h_feas), n_regions);
      if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&r->h_lb), n_regions * sizeof(double));
    } else {
      if (e == cudaSuccess) e = dalloc(&r->d_block_best, (size_t)r->grid + 1);
      if (e == cudaSuccess) e = dalloc(&r->d_point, (size_t)n);
      if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&r->h_point), n * sizeof(double));
      if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&r->h_cand), sizeof(Cand));
    }
    if (e != cudaSuccess) {
      delete r;
      return fail(CMN_CUDA_ERROR, std::string("role allocation: ") + cudaGetErrorString(e));
    }
    *out = r;
    return CMN_OK;
  } catch (const std::bad_alloc&) {
    return fail(CMN_INTERNAL, "host allocation failed");
  }
}

extern "C" void cmn_role_destroy(cmn_role* r) { delete r; }

extern "C" uint64_t cmn_role_n_regions(const cmn_role* r) { return r ? r->n_regions : 0; }

extern "C" uint64_t cmn_role_n_elements(const cmn_role* r) { return r ? r->n_regions * r->S : 0; }

// Stages the parent box and the per-launch slot data (var_ids, widths)
// with one host-to-device copy (graph/replay.cuh:610-771 set_domain).
static cmn_status stage_region(cmn_role* r, const double* box, const uint64_t* var_ids, const uint64_t* widths)
{
  const cmn_problem* p = r->p;
  const int64_t n = p->host.n_vars();
  const int64_t sc = (int64_t)r->slot_kinds.size();
  if (!box) return fail(CMN_SHAPE_MISMATCH, "null box");
  if (sc > 0 && (!var_ids || !widths)) return fail(CMN_SHAPE_MISMATCH, "null var_ids/widths");
  double* lo = reinterpret_cast<double*>(r->h_stage);
  double* hi = lo + n;
  SlotPlan* sp = reinterpret_cast<SlotPlan*>(hi + n);
  ParentInfo* pi = reinterpret_cast<ParentInfo*>(sp + 64);
  for (int64_t v = 0; v < n; ++v) {
    lo[v] = box[2 * v];
    hi[v] = box[2 * v + 1];
  }
  uint64_t running = 1;
  for (int64_t j = 0; j < sc; ++j) {
    if (var_ids[j] >= (uint64_t)n) return fail(CMN_SHAPE_MISMATCH, "var_id out of range");
    if (widths[j] < 1) return fail(CMN_SHAPE_MISMATCH, "slot width must be at least 1");
    sp[j].width = widths[j];
    sp[j].prefix = running;
    sp[j].dom = widths[j];
    sp[j].vid = (uint32_t)var_ids[j];
    sp[j].kind = r->slot_kinds[j];
    sp[j].step = slot_step(sp[j].kind, lo[var_ids[j]], hi[var_ids[j]], widths[j]);
    if (running > UINT64_MAX / widths[j]) running = UINT64_MAX;
    else running *= widths[j];
  }
  if (running != r->n_regions)
    return fail(CMN_SHAPE_MISMATCH, "the product of widths (" + std::to_string(running) +
                                        ") does not equal this role's n_regions (" + std::to_string(r->n_regions) + ")");
  pi->count = (uint32_t)sc;
  pi->fathom = 0;
  pi->nreg = r->n_regions;
  CK(cudaMemcpyAsync(r->d_stage, r->h_stage, r->stage_bytes, cudaMemcpyHostToDevice, r->stream));
  return CMN_OK;
}

static void role_ptrs(const cmn_role* r, const double*& plo, const double*& phi, const SlotPlan*& sp,
                      const ParentInfo*& pi)
{
  const int64_t n = r->p->host.n_vars();
  plo = reinterpret_cast<const double*>(r->d_stage);
  phi = plo + n;
  sp = reinterpret_cast<const SlotPlan*>(phi + n);
  pi = reinterpret_cast<const ParentInfo*>(sp + 64);
}

extern "C" cmn_status cmn_bound(cmn_role* r, const double* box, const uint64_t* var_ids, const uint64_t* widths,
                                const uint8_t** feasible, const double** obj_lb, uint64_t* n_regions)
{
  if (!r) return fail(CMN_INVALID_CONFIGURATION, "bound() called on a null role");
  if (r->kind != CMN_ROLE_BOUNDER) return fail(CMN_INVALID_CONFIGURATION, "bound() called on a role that is not a bounder");
  CK(cudaSetDevice(r->p->device));
  cmn_status st = stage_region(r, box, var_ids, widths);
  if (st != CMN_OK) return st;
  EvalArgs a = {};
  const double *plo, *phi;
  const SlotPlan* sp;
  const ParentInfo* pi;
  role_ptrs(r, plo, phi, sp, pi);
  a.prog = r->p->d_prog64;
  a.prog_len = (int)r->p->prog.code64.size();
  a.n_vars = (int)r->p->host.n_vars();
  a.n_slots = r->p->prog.n_slots;
  a.log2C = -1;
  a.plo = plo;
  a.phi = phi;
  a.pstride = 1;
  a.pinfo = pi;
  a.slots = sp;
  a.max_slots = (int)r->slot_kinds.size();  // one parent: the stride of the slot table is unused
  a.n_children = r->n_regions;
  a.out_lb = r->d_lb;
  a.out_flag = r->d_feas;
  a.sched = r->p->d_sched;
  a.g_max = r->p->prog.group_max;
  a.capacity = (uint64_t)r->grid * kEvalThreads;
  CK(launch_eval(a, 0, false, r->grid, kEvalThreads, r->stream));
  CK(cudaMemcpyAsync(r->h_feas, r->d_feas, r->n_regions, cudaMemcpyDeviceToHost, r->stream));
  CK(cudaMemcpyAsync(r->h_lb, r->d_lb, r->n_regions * sizeof(double), cudaMemcpyDeviceToHost, r->stream));
  CK(cudaStreamSynchronize(r->stream));
  if (feasible) *feasible = r->h_feas;
  if (obj_lb) *obj_lb = r->h_lb;
  if (n_regions) *n_regions = r->n_regions;
  return CMN_OK;
}

// total order of doubles used by the aggregate fold (NaN above +inf)
static uint64_t host_key(double x)
{
  uint64_t u;
  std::memcpy(&u, &x, 8);
  if (x != x) return ~0ULL;
  return (u >> 63) ? ~u : (u | 0x8000000000000000ULL);
}

static double host_unkey(uint64_t k)
{
  const uint64_t u = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
  double x;
  std::memcpy(&x, &u, 8);
  return x;
}

extern "C" cmn_status cmn_bound_children(cmn_role* r, const double* box, const uint64_t* var_ids,
                                          const uint64_t* widths, uint64_t k, const cmn_aggregate_bound** out)
{
  if (!r || !out) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  if (r->kind != CMN_ROLE_BOUNDER)
    return fail(CMN_INVALID_CONFIGURATION, "aggregate bounds need a role built as a bounder");
  if (k == 0 || r->n_regions % k != 0)
    return fail(CMN_SHAPE_MISMATCH, "k (" + std::to_string(k) + ") must divide the role's n_regions (" +
                                        std::to_string(r->n_regions) + ")");
  CK(cudaSetDevice(r->p->device));
  cmn_status st = stage_region(r, box, var_ids, widths);
  if (st != CMN_OK) return st;
  if (k > r->agg_cap) {
    dfree(r->d_agg);
    if (r->h_agg) cudaFreeHost(r->h_agg);
    if (r->h_agg_out) cudaFreeHost(r->h_agg_out);
    r->d_agg = nullptr;
    r->h_agg = nullptr;
    r->h_agg_out = nullptr;
    r->agg_cap = 0;
    CK(dalloc(&r->d_agg, 2 * k));
    CK(cudaMallocHost(reinterpret_cast<void**>(&r->h_agg), 2 * k * sizeof(unsigned long long)));
    CK(cudaMallocHost(reinterpret_cast<void**>(&r->h_agg_out), k * sizeof(cmn_aggregate_bound)));
    r->agg_cap = k;
  }
  // identities: every region excluded leaves (+inf, -inf)
  for (uint64_t c = 0; c < k; ++c) {
    r->h_agg[c] = host_key(INFINITY);
    r->h_agg[k + c] = host_key(-INFINITY);
  }
  CK(cudaMemcpyAsync(r->d_agg, r->h_agg, 2 * k * sizeof(unsigned long long), cudaMemcpyHostToDevice, r->stream));
  EvalArgs a = {};
  const double *plo, *phi;
  const SlotPlan* sp;
  const ParentInfo* pi;
  role_ptrs(r, plo, phi, sp, pi);
  a.prog = r->p->d_prog64;
  a.prog_len = (int)r->p->prog.code64.size();
  a.n_vars = (int)r->p->host.n_vars();
  a.n_slots = r->p->prog.n_slots;
  a.log2C = -1;
  a.plo = plo;
  a.phi = phi;
  a.pstride = 1;
  a.pinfo = pi;
  a.slots = sp;
  a.max_slots = (int)r->slot_kinds.size();
  a.n_children = r->n_regions;
  a.sched = r->p->d_sched;
  a.g_max = r->p->prog.group_max;
  a.capacity = (uint64_t)r->grid * kEvalThreads;
  a.agg_keys = r->d_agg;
  a.agg_m = r->n_regions / k;
  a.agg_k = k;
  CK(launch_eval(a, 4, false, r->grid, kEvalThreads, r->stream));
  CK(cudaMemcpyAsync(r->h_agg, r->d_agg, 2 * k * sizeof(unsigned long long), cudaMemcpyDeviceToHost, r->stream));
  CK(cudaStreamSynchronize(r->stream));
  for (uint64_t c = 0; c < k; ++c) {
    const double lb = host_unkey(r->h_agg[c]);
    const double ub = host_unkey(r->h_agg[k + c]);
    // replay.cuh:343-361: a child whose Max is still -inf had every region
    // excluded; it is normalised to (+inf, +inf, infeasible)
    const bool feasible = ub > -INFINITY;
    cmn_aggregate_bound& o = r->h_agg_out[c];
    o.lb = feasible ? lb : INFINITY;
    o.hull_ub = feasible ? ub : INFINITY;
    o.feasible = feasible ? 1 : 0;
    o.reserved = 0;
  }
  *out = r->h_agg_out;
  return CMN_OK;
}

static cmn_status candidate_role(cmn_role* r, const double* box, const uint64_t* var_ids, const uint64_t* widths,
                                 uint64_t salt, int exact, cmn_candidate* out)
{
  CK(cudaSetDevice(r->p->device));
  cmn_status st = stage_region(r, box, var_ids, widths);
  if (st != CMN_OK) return st;
  const double *plo, *phi;
  const SlotPlan* sp;
  const ParentInfo* pi;
  role_ptrs(r, plo, phi, sp, pi);
  SampleArgs a = {};
  a.prog = r->p->d_prog64;
  a.prog_len = (int)r->p->prog.code64.size();
  a.n_vars = (int)r->p->host.n_vars();
  a.n_slots = r->p->prog.n_slots;
  a.log2C = -1;
  a.plo = plo;
  a.phi = phi;
  a.pstride = 1;
  a.pinfo = pi;
  a.slots = sp;
  a.max_slots = 64;
  a.var_kinds = r->p->d_kinds;
  a.root_lb = r->p->d_root_lb;
  a.root_ub = r->p->d_root_ub;
  a.n_children = r->n_regions;
  a.S = r->S;
  a.salt = salt;
  a.exact = exact;
  a.block_best = r->d_block_best;
  a.sched = r->p->d_sched;
  a.g_max = r->p->prog.group_max;
  a.capacity = (uint64_t)r->grid * kEvalThreads;
  a.lg_min = r->lg_min;
  CK(launch_sample(a, r->grid, kEvalThreads, r->stream));
  Cand* best = r->d_block_best + r->grid;
  CK(launch_reduce_cand(r->d_block_best, r->grid, best, r->stream));
  CK(launch_witness(best, plo, phi, 1, pi, sp, 64, r->p->d_kinds, a.n_vars, r->S, salt, nullptr, exact, nullptr,
                    r->d_point, r->stream));
  CK(cudaMemcpyAsync(r->h_cand, best, sizeof(Cand), cudaMemcpyDeviceToHost, r->stream));
  CK(cudaMemcpyAsync(r->h_point, r->d_point, a.n_vars * sizeof(double), cudaMemcpyDeviceToHost, r->stream));
  CK(cudaStreamSynchronize(r->stream));
  const Cand c = *r->h_cand;
  out->found = c.value < DBL_MAX ? 1 : 0;
  out->reserved = 0;
  out->value = c.value;
  out->point = r->h_point;
  out->index = out->found ? (int64_t)c.e : -1;
  return CMN_OK;
}

extern "C" cmn_status cmn_sample(cmn_role* r, const double* box, const uint64_t* var_ids, const uint64_t* widths,
                                 uint64_t salt, cmn_candidate* out)
{
  if (!r || !out) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  if (r->kind != CMN_ROLE_SAMPLER) return fail(CMN_INVALID_CONFIGURATION, "sample() called on a role that is not a sampler");
  return candidate_role(r, box, var_ids, widths, salt, 0, out);
}

extern "C" cmn_status cmn_enumerate(cmn_role* r, const double* box, const uint64_t* var_ids, const uint64_t* widths,
                                    cmn_candidate* out)
{
  if (!r || !out) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  if (r->kind != CMN_ROLE_ENUMERATOR)
    return fail(CMN_INVALID_CONFIGURATION, "enumerate() called on a role that is not an enumerator");
  return candidate_role(r, box, var_ids, widths, 0, 1, out);
}

// ----------------------------------------------------------------------
// raw batched evaluation
// ----------------------------------------------------------------------
extern "C" cmn_status cmn_eval_boxes(const cmn_problem* p, int32_t precision, const double* lo, const double* hi,
                                     uint64_t n_boxes, uint64_t stride, double* obj_lb, double* obj_ub,
                                     uint8_t* feasible, int32_t device_pointers, void* stream)
{
  if (!p) return fail(CMN_INVALID_CONFIGURATION, "null problem");
  if (precision != CMN_PRECISION_FP64 && precision != CMN_PRECISION_FP32_SCREEN)
    return fail(CMN_INVALID_CONFIGURATION, "unknown precision");
  if (n_boxes == 0) return CMN_OK;
  if (!lo || !hi || !obj_lb || !feasible) return fail(CMN_SHAPE_MISMATCH, "null array");
  if (stride < n_boxes) return fail(CMN_SHAPE_MISMATCH, "stride below n_boxes");
  cmn_status st = check_interval(p);
  if (st != CMN_OK) return st;
  const bool fp32 = precision == CMN_PRECISION_FP32_SCREEN;
  st = check_smem(p, fp32, 0);
  if (st != CMN_OK) return st;
  CK(cudaSetDevice(p->device));
  CK(ensure_attributes());
  const int64_t n = p->host.n_vars();
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const double *dlo = lo, *dhi = hi;
  double *dlb = obj_lb, *dub = obj_ub;
  uint8_t* dfe = feasible;
  double* tmp = nullptr;
  uint8_t* tmpf = nullptr;
  uint64_t ps = stride;
  if (!device_pointers) {
    ps = n_boxes;
    const size_t planes = (size_t)n * n_boxes;
    CK(dalloc(&tmp, 2 * planes + 2 * n_boxes));
    CK(dalloc(&tmpf, n_boxes));
    for (int64_t v = 0; v < n; ++v) {
      CK(cudaMemcpyAsync(tmp + v * n_boxes, lo + v * stride, n_boxes * sizeof(double), cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(tmp + planes + v * n_boxes, hi + v * stride, n_boxes * sizeof(double), cudaMemcpyHostToDevice,
                         s));
    }
    dlo = tmp;
    dhi = tmp + planes;
    dlb = tmp + 2 * planes;
    dub = tmp + 2 * planes + n_boxes;
    dfe = tmpf;
  }
  EvalArgs a = {};
  a.prog = fp32 ? p->d_prog32 : p->d_prog64;
  a.prog_len = (int)p->prog.code64.size();
  a.n_vars = (int)n;
  a.n_slots = p->prog.n_slots;
  a.log2C = 0;
  a.plo = dlo;
  a.phi = dhi;
  a.pstride = ps;
  a.pinfo = nullptr;
  a.n_children = n_boxes;
  a.out_lb = dlb;
  a.out_ub = dub;
  a.out_flag = dfe;
  const int threads = kEvalThreads;
  const int occ =
      std::max(1, eval_kernel_occupancy(0, fp32, eval_smem_bytes(p->prog.n_slots, 0, fp32, threads), threads));
  const uint64_t need = (n_boxes * (uint64_t)p->prog.group_max + threads - 1) / threads;
  const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)sm_count() * occ));
  a.sched = p->d_sched;
  a.g_max = p->prog.group_max;
  a.capacity = (uint64_t)sm_count() * occ * threads;
  cudaError_t e = launch_eval(a, 0, fp32, grid, threads, s);
  if (e != cudaSuccess) {
    dfree(tmp);
    dfree(tmpf);
    return fail(CMN_CUDA_ERROR, std::string("eval launch: ") + cudaGetErrorString(e));
  }
  if (!device_pointers) {
    CK(cudaMemcpyAsync(obj_lb, dlb, n_boxes * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (obj_ub) CK(cudaMemcpyAsync(obj_ub, dub, n_boxes * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(feasible, dfe, n_boxes, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    dfree(tmp);
    dfree(tmpf);
  }
  return CMN_OK;
}

// ----------------------------------------------------------------------
// solver
// ----------------------------------------------------------------------
extern "C" cmn_status cmn_autotune(cmn_problem* p, int32_t precision, uint64_t n_boxes, cmn_tune_result* out)
{
  if (!p || !out) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  if (precision != 0 && precision != 1) return fail(CMN_INVALID_CONFIGURATION, "precision must be 0 or 1");
  if (n_boxes < 1) return fail(CMN_INVALID_CONFIGURATION, "n_boxes must be at least 1");
  cmn_status st = check_interval(p);
  if (st != CMN_OK) return st;
  const bool fp32 = precision == 1;
  st = check_smem(p, fp32, 0);
  if (st != CMN_OK) return st;
  CK(cudaSetDevice(p->device));
  CK(ensure_attributes());
  const int64_t n = p->host.n_vars();
  // random boxes inside the root box (a fixed seed), as planes
  std::vector<double> lo((size_t)n * n_boxes), hi((size_t)n * n_boxes);
  uint64_t x = 0x9e3779b97f4a7c15ULL;
  auto uni = [&]() {
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int64_t v = 0; v < n; ++v) {
    const double a = p->host.var_lb[v], b = p->host.var_ub[v];
    const double span = std::isfinite(b - a) ? b - a : 2.0;
    const double base = std::isfinite(a) ? a : -1.0;
    for (uint64_t i = 0; i < n_boxes; ++i) {
      const double c = base + span * uni(), w = span * 0.05 * uni();
      double l = std::max(base, c - w), h = std::min(base + span, c + w);
      if (p->host.var_kinds[v] != CMN_VAR_CONTINUOUS) {
        l = std::ceil(l);
        h = std::max(std::floor(h), l);
      }
      lo[(size_t)v * n_boxes + i] = l;
      hi[(size_t)v * n_boxes + i] = h;
    }
  }
  double* d = nullptr;
  uint8_t* f = nullptr;
  const size_t planes = (size_t)n * n_boxes;
  CK(dalloc(&d, 2 * planes + n_boxes));
  cudaError_t e = dalloc(&f, n_boxes);
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d, lo.data(), planes * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d + planes, hi.data(), planes * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  EvalArgs a = {};
  a.prog = fp32 ? p->d_prog32 : p->d_prog64;
  a.prog_len = (int)p->prog.code64.size();
  a.n_vars = (int)n;
  a.n_slots = p->prog.n_slots;
  a.log2C = 0;
  a.plo = d;
  a.phi = d + planes;
  a.pstride = n_boxes;
  a.n_children = n_boxes;
  a.out_lb = d + 2 * planes;
  a.out_flag = f;
  a.sched = p->d_sched;
  const int threads = kEvalThreads;
  const int occ =
      std::max(1, eval_kernel_occupancy(0, fp32, eval_smem_bytes(p->prog.n_slots, 0, fp32, threads), threads));
  const int lanes_max = p->d_sched ? p->prog.group_max : 1;
  auto time_shape = [&](int bps, int lanes, double& ms) {
    const uint64_t need = (n_boxes * (uint64_t)lanes + threads - 1) / threads;
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)sm_count() * bps));
    a.g_max = lanes;
    a.capacity = (uint64_t)grid * threads;
    ms = 1e30;
    for (int r = 0; r < 4 && e == cudaSuccess; ++r) {  // the first launch warms up
      e = cudaEventRecord(e0, s);
      if (e == cudaSuccess) e = launch_eval(a, 0, fp32, grid, threads, s);
      if (e == cudaSuccess) e = cudaEventRecord(e1, s);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float t = 0;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
      if (r > 0 && t < ms) ms = t;
    }
  };
  out->candidates = 0;
  out->ms_best = 1e30;
  time_shape(occ, lanes_max, out->ms_default);
  for (int bps = 1; bps <= occ && e == cudaSuccess; ++bps) {
    for (int lanes = 1; lanes <= lanes_max && e == cudaSuccess; lanes <<= 1) {
      double ms;
      time_shape(bps, lanes, ms);
      ++out->candidates;
      if (ms < out->ms_best) {
        out->ms_best = ms;
        out->blocks_per_sm = bps;
        out->lanes_cap = lanes;
      }
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  dfree(d);
  dfree(f);
  if (e != cudaSuccess) return fail(CMN_CUDA_ERROR, std::string("autotune: ") + cudaGetErrorString(e));
  out->reserved = 0;
  p->tuned_bps[precision] = out->blocks_per_sm;
  p->tuned_lanes[precision] = out->lanes_cap;
  return CMN_OK;
}

extern "C" void cmn_solve_options_default(cmn_solve_options* o)
{
  if (!o) return;
  std::memset(o, 0, sizeof *o);
  o->iter_limit = 1000000;
  o->batch_iter_limit = 0;
  o->tolerance = 1e-6;
  o->precision = CMN_PRECISION_FP64;
  o->bisection_budget = 4;
  o->frontier_cap = 1ull << 20;
  o->batch_parents = 1ull << 16;
  o->sample_points = 1;
  o->sample_all = 0;
  o->relative_width = 0;
  o->max_cycle_size = 0;
  o->enumerate_cap = 0;
  o->has_known_primal = 0;
  o->known_primal_bound = 0;
  o->time_limit_ms = 0;
}

struct cmn_solver {
  const cmn_problem* p = nullptr;
  cmn_solve_options opts{};
  SolverCfg cfg{};
  SolverBufs b{};
  cudaStream_t stream = nullptr;
  // the first iteration selects its parents; every later one finds them
  // staged by its predecessor and runs the graph without the select
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph_steady = nullptr;
  cudaGraphExec_t exec_steady = nullptr;
  SolverDev* h_dev = nullptr;  // pinned mirror
  uint64_t* d_viable = nullptr;
  uint64_t* h_viable = nullptr;
  std::vector<void*> allocs;
  int eval_grid = 1, sample_grid = 1;
  double elapsed_ms = 0;
  uint64_t launched = 0;
  uint64_t kernels_per_iter = 0;
  cudaEvent_t marks[kPhaseMarks] = {};
  SideStream side;

  ~cmn_solver()
  {
    int cur = 0;
    if (p && cudaGetDevice(&cur) == cudaSuccess && cur != p->device) cudaSetDevice(p->device);
    if (stream) cudaStreamSynchronize(stream);
    if (side.stream) cudaStreamSynchronize(side.stream);
    for (cudaEvent_t ev : marks)
      if (ev) cudaEventDestroy(ev);
    if (side.fork) cudaEventDestroy(side.fork);
    if (side.join) cudaEventDestroy(side.join);
    if (side.stream) cudaStreamDestroy(side.stream);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (exec_steady) cudaGraphExecDestroy(exec_steady);
    if (graph_steady) cudaGraphDestroy(graph_steady);
    for (void* a : allocs) cudaFree(a);
    if (h_dev) cudaFreeHost(h_dev);
    if (h_viable) cudaFreeHost(h_viable);
    if (stream) cudaStreamDestroy(stream);
    if (p && cur != p->device) cudaSetDevice(cur);
  }

  template <typename T>
  cudaError_t alloc(T** ptr, size_t n)
  {
    cudaError_t e = dalloc(ptr, n);
    if (e == cudaSuccess) allocs.push_back(*ptr);
    return e;
  }
};

extern "C" cmn_status cmn_solver_create(const cmn_problem* p, const cmn_solve_options* opts, cmn_solver** out)
{
  if (!p || !opts || !out) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  *out = nullptr;
  const cmn_solve_options& o = *opts;
  if (o.bisection_budget < 1 || o.bisection_budget > 20)
    return fail(CMN_INVALID_CONFIGURATION, "bisection_budget must be within [1, 20] for the batched solver");
  if (o.sample_points < 1) return fail(CMN_INVALID_CONFIGURATION, "sample_points must be at least 1");
  if (o.batch_parents < 1) return fail(CMN_INVALID_CONFIGURATION, "batch_parents must be at least 1");
  if (o.frontier_cap < 1) return fail(CMN_INVALID_CONFIGURATION, "frontier_cap must be at least 1");
  if (o.max_cycle_size > 64)
    return fail(CMN_INVALID_CONFIGURATION, "max_cycle_size (" + std::to_string(o.max_cycle_size) +
                                               ") exceeds kMaxSlots (64)");
  if (o.precision != CMN_PRECISION_FP64 && o.precision != CMN_PRECISION_FP32_SCREEN &&
      o.precision != CMN_PRECISION_FP32_LAZY)
    return fail(CMN_INVALID_CONFIGURATION, "unknown precision");
  const uint64_t C = 1ull << o.bisection_budget;
  if (o.batch_parents > ((1ull << 31) >> o.bisection_budget))  // shifted this way round, nothing wraps
    return fail(CMN_INVALID_CONFIGURATION, "batch_parents * 2^bisection_budget above 2^31 children per iteration");
  if (o.frontier_cap > (1ull << 31)) return fail(CMN_INVALID_CONFIGURATION, "frontier_cap above 2^31");
  cmn_status st = check_interval(p);
  if (st != CMN_OK) return st;
  st = check_smem(p, o.precision != CMN_PRECISION_FP64, o.bisection_budget);
  if (st != CMN_OK) return st;
  if (o.precision == CMN_PRECISION_FP32_LAZY) {  // the parents' FP64 pass
    st = check_smem(p, false, 0);
    if (st != CMN_OK) return st;
  }
  const int lg_min = sample_lg_min((int)p->host.n_vars(), p->prog.n_slots, p->d_sched != nullptr, kEvalThreads);
  if (sample_smem_bytes((int)p->host.n_vars(), p->prog.n_slots, kEvalThreads, lg_min) > (size_t)max_dynamic_smem())
    return fail(CMN_INVALID_CONFIGURATION,
                "the sampler's per-thread point columns do not fit in shared memory (a program with shared slots "
                "keeps one column of n_vars + slots doubles per thread)");
  const int lg_screen =
      sample_screen_lg_min((int)p->host.n_vars(), p->prog.n_slots, p->d_sched != nullptr, kEvalThreads);
  if (o.precision == CMN_PRECISION_FP32_LAZY &&
      sample_screen_smem_bytes((int)p->host.n_vars(), p->prog.n_slots, kEvalThreads, lg_screen) >
          (size_t)max_dynamic_smem())
    return fail(CMN_INVALID_CONFIGURATION, "the lazy form's FP32 sample screen keeps one column of n_vars + slots "
                                           "floats per thread for a program with shared slots; this problem's "
                                           "does not fit in shared memory");
  try {
    CK(cudaSetDevice(p->device));
    CK(ensure_attributes());
    cmn_solver* s = new cmn_solver();
    s->p = p;
    s->opts = o;
    SolverCfg& cfg = s->cfg;
    const int n = (int)p->host.n_vars();
    cfg.n_vars = n;
    cfg.n_slots = p->prog.n_slots;
    cfg.prog_len = (int)p->prog.code64.size();
    cfg.log2C = o.bisection_budget;
    cfg.max_slots = o.bisection_budget;
    cfg.precision = o.precision;
    cfg.sample_all = o.sample_all;
    cfg.relative = o.relative_width;
    cfg.S = o.sample_points;
    cfg.e_max = o.batch_parents;
    cfg.cap = o.frontier_cap;
    cfg.pstride = o.frontier_cap + (o.batch_parents << o.bisection_budget);
    cfg.iter_limit = o.iter_limit;
    cfg.batch_iter_limit = o.batch_iter_limit;
    cfg.max_cycle = (int64_t)o.max_cycle_size;
    cfg.enumerate_cap = (int64_t)o.enumerate_cap;
    cfg.tolerance = o.tolerance;
    const uint64_t maxc = cfg.e_max * C;
    const int threads = kEvalThreads;
    const bool fp32 = o.precision != CMN_PRECISION_FP64;
    const bool lazy = o.precision == CMN_PRECISION_FP32_LAZY;
    const int occ_e = std::max(1, eval_kernel_occupancy(lazy ? 5 : fp32 ? 2 : 1, fp32,
                                                        eval_smem_bytes(p->prog.n_slots, cfg.max_slots, fp32, threads), threads));
    cfg.sample_lg_min = lg_min;
    const int occ_s =
        std::max(1, sample_kernel_occupancy(sample_smem_bytes(n, p->prog.n_slots, threads, lg_min), threads));
    const int tp = fp32 ? 1 : 0;
    if (o.autotune && p->tuned_bps[tp] == 0) {
      cmn_tune_result tr{};
      cmn_status ts =
          cmn_autotune(const_cast<cmn_problem*>(p), tp, std::min<uint64_t>(maxc, 1ull << 18), &tr);
      if (ts != CMN_OK) {
        delete s;
        return ts;
      }
    }
    const bool tuned = o.autotune && p->tuned_bps[tp] > 0;
    const uint64_t need = (maxc * (uint64_t)p->prog.group_max + threads - 1) / threads;
    s->eval_grid = (int)std::max<uint64_t>(
        1, std::min<uint64_t>(need, (uint64_t)sm_count() * (tuned ? std::min(p->tuned_bps[tp], occ_e) : occ_e)));
    s->sample_grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)sm_count() * occ_s));
    if (lazy) {
      cfg.screen_lg_min = lg_screen;
      const int occ_q = std::max(
          1, sample_screen_occupancy(sample_screen_smem_bytes(n, p->prog.n_slots, threads, lg_screen), threads));
      cfg.screen_grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((maxc + threads - 1) / threads,
                                                                      (uint64_t)sm_count() * occ_q));
    }
    cfg.g_max = p->d_sched ? (tuned ? std::min(p->tuned_lanes[tp], p->prog.group_max) : p->prog.group_max) : 1;
    cfg.eval_capacity = (uint64_t)s->eval_grid * threads;
    cfg.sample_capacity = (uint64_t)s->sample_grid * threads;

    SolverBufs& b = s->b;
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    auto A = [&](auto** ptr, size_t count) {
      if (e == cudaSuccess) e = s->alloc(ptr, count);
    };
    A(&b.dev, 1);
    A(&b.radix, 2);
    for (int q = 0; q < 2; ++q) {
      A(&b.lb[q], cfg.pstride);
      A(&b.slot[q], cfg.pstride);
    }
    A(&b.lo, (size_t)n * cfg.pstride);
    A(&b.hi, (size_t)n * cfg.pstride);
    A(&b.depth, cfg.pstride);
    A(&b.free_slots, cfg.pstride);
    A(&b.sel[0], cfg.pstride);
    A(&b.sel[1], cfg.pstride);
    A(&b.plo, (size_t)n * cfg.e_max);
    A(&b.phi, (size_t)n * cfg.e_max);
    if (fp32) {
      A(&b.plo32, (size_t)n * cfg.e_max);
      A(&b.phi32, (size_t)n * cfg.e_max);
    }
    A(&b.pdepth, cfg.e_max);
    if (lazy) {
      A(&b.plb, cfg.e_max);
      A(&b.pfeas, cfg.e_max);
    }
    cfg.inc = lazy && p->d_inc_seg != nullptr ? 1 : 0;
    if (cfg.inc) {
      cfg.inc_segments = p->prog.inc_segments;
      b.inc_seg = p->d_inc_seg;
      b.inc_off = p->d_inc_off;
      b.inc_pcs = p->d_inc_pcs;
      A(&b.inc_common, 2 * (size_t)cfg.inc_segments * cfg.e_max);
      A(&b.inc_parts, 2 * (size_t)cfg.inc_segments * ((size_t)1 << cfg.log2C) * cfg.e_max);
    }
    A(&b.pslot, cfg.e_max);
    A(&b.pinfo, cfg.e_max);
    A(&b.slots, cfg.e_max * (size_t)cfg.max_slots);
    unsigned char* es = nullptr;
    unsigned char* bs = nullptr;
    A(&es, cfg.e_max * (size_t)n * sizeof(EnumCand));
    A(&bs, cfg.e_max * (size_t)n * sizeof(BisCand));
    b.enum_scratch = es;
    b.bis_scratch = bs;
    A(&b.heap_scratch, cfg.e_max * (size_t)n);
    A(&b.clb, maxc);
    A(&b.cstate, maxc);
    if (lazy) A(&b.cbest, maxc);
    A(&b.list, maxc);
    const size_t nblk = (std::max<uint64_t>(cfg.pstride, maxc) + kScanTile - 1) / kScanTile + 1;
    A(&b.block_counts, nblk);
    A(&b.block_offsets, nblk);
    A(&b.block_counts2, nblk);
    A(&b.block_offsets2, nblk);
    b.n_block_best = s->sample_grid + 1;
    A(&b.block_best, (size_t)b.n_block_best);
    A(&b.best_point, (size_t)n);
    A(&s->d_viable, 1);
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&s->h_dev), sizeof(SolverDev));
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&s->h_viable), sizeof(uint64_t));
    if (e != cudaSuccess) {
      delete s;
      if (e == cudaErrorMemoryAllocation)
        return fail(CMN_OVER_BUDGET, "the solver's pools do not fit in device memory (frontier_cap / batch_parents)");
      return fail(CMN_CUDA_ERROR, std::string("solver allocation: ") + cudaGetErrorString(e));
    }
    b.prog64 = p->d_prog64;
    b.prog32 = p->d_prog32;
    b.prog32p = p->d_prog32p;
    b.sched = p->d_sched;
    b.kinds = p->d_kinds;
    b.root_lb = p->d_root_lb;
    b.root_ub = p->d_root_ub;
    const double gub0 = o.has_known_primal ? o.known_primal_bound : DBL_MAX;
    e = solver_init(cfg, b, p->d_root_lb, p->d_root_ub, gub0, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.best_point, 0xff, (size_t)n * sizeof(double), s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    for (int i = 0; i < kPhaseMarks && e == cudaSuccess; ++i) e = cudaEventCreate(&s->marks[i]);
    // the side stream carries the lazy form's FP64 verdict, the longest of
    // the work it runs beside: its blocks go first
    int prio_low = 0, prio_high = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s->side.stream, cudaStreamNonBlocking, prio_high);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->side.fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->side.join, cudaEventDisableTiming);
    // capture one iteration, with and without the parent select
    for (int steady = 0; steady < 2 && e == cudaSuccess; ++steady) {
      cudaGraph_t* g = steady ? &s->graph_steady : &s->graph;
      e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        cudaError_t e2 =
            solver_iteration(cfg, b, s->eval_grid, s->sample_grid, s->stream, s->side, s->marks, steady == 0);
        e = cudaStreamEndCapture(s->stream, g);
        if (e2 != cudaSuccess) e = e2;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(steady ? &s->exec_steady : &s->exec, *g, 0);
    }
    if (e == cudaSuccess) {  // kernels of a steady iteration
      size_t nn = 0;
      e = cudaGraphGetNodes(s->graph_steady, nullptr, &nn);
      std::vector<cudaGraphNode_t> nodes(nn);
      if (e == cudaSuccess && nn) e = cudaGraphGetNodes(s->graph_steady, nodes.data(), &nn);
      for (size_t i = 0; i < nn && e == cudaSuccess; ++i) {
        cudaGraphNodeType t;
        e = cudaGraphNodeGetType(nodes[i], &t);
        if (t == cudaGraphNodeTypeKernel) ++s->kernels_per_iter;
      }
    }
    if (e != cudaSuccess) {
      delete s;
      return fail(CMN_CUDA_ERROR, std::string("solver setup: ") + cudaGetErrorString(e));
    }
    *out = s;
    return CMN_OK;
  } catch (const std::bad_alloc&) {
    return fail(CMN_INTERNAL, "host allocation failed");
  }
}

extern "C" void cmn_solver_destroy(cmn_solver* s) { delete s; }

extern "C" void* cmn_solver_stream(cmn_solver* s) { return s ? reinterpret_cast<void*>(s->stream) : nullptr; }

static cmn_status pull_state(cmn_solver* s)
{
  CK(cudaMemcpyAsync(s->h_dev, s->b.dev, sizeof(SolverDev), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return CMN_OK;
}

extern "C" cmn_status cmn_solver_step(cmn_solver* s, uint64_t max_iterations)
{
  if (!s) return fail(CMN_INVALID_CONFIGURATION, "null solver");
  CK(cudaSetDevice(s->p->device));
  const auto t0 = std::chrono::steady_clock::now();
  cmn_status st = pull_state(s);
  if (st != CMN_OK) return st;
  uint64_t done_iters = 0;
  uint64_t burst = 1;
  while (!s->h_dev->done && (max_iterations == 0 || done_iters < max_iterations)) {
    uint64_t k = burst;
    if (max_iterations) k = std::min<uint64_t>(k, max_iterations - done_iters);
    for (uint64_t i = 0; i < k; ++i) CK(cudaGraphLaunch(s->launched + i == 0 ? s->exec : s->exec_steady, s->stream));
    done_iters += k;
    s->launched += k;
    st = pull_state(s);
    if (st != CMN_OK) return st;
    if (s->h_dev->error) return fail(CMN_INTERNAL, "device-side error flag set");
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (s->opts.time_limit_ms && s->elapsed_ms + ms >= (double)s->opts.time_limit_ms) break;
    if (ms < 50.0 && burst < 64) burst *= 2;
  }
  s->elapsed_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return CMN_OK;
}

extern "C" cmn_status cmn_query_bounds(const cmn_solver* s, double* lower_bound, double* upper_bound)
{
  if (!s) return fail(CMN_INVALID_CONFIGURATION, "null solver");
  cmn_status st = pull_state(const_cast<cmn_solver*>(s));
  if (st != CMN_OK) return st;
  if (lower_bound) *lower_bound = s->h_dev->glb;
  if (upper_bound) *upper_bound = s->h_dev->gub;
  return CMN_OK;
}

extern "C" cmn_status cmn_query_gap(const cmn_solver* s, double* gap)
{
  double lb, ub;
  cmn_status st = cmn_query_bounds(s, &lb, &ub);
  if (st != CMN_OK) return st;
  if (gap) *gap = ub - lb;
  return CMN_OK;
}

extern "C" cmn_status cmn_query_incumbent(const cmn_solver* s, double* point, int32_t* found)
{
  if (!s) return fail(CMN_INVALID_CONFIGURATION, "null solver");
  cmn_solver* m = const_cast<cmn_solver*>(s);
  cmn_status st = pull_state(m);
  if (st != CMN_OK) return st;
  const bool f = s->h_dev->have_best && s->h_dev->gub < DBL_MAX;
  if (found) *found = f ? 1 : 0;
  if (point) {
    CK(cudaMemcpyAsync(point, s->b.best_point, s->p->host.n_vars() * sizeof(double), cudaMemcpyDeviceToHost,
                       m->stream));
    CK(cudaStreamSynchronize(m->stream));
    if (!f)
      for (int64_t v = 0; v < s->p->host.n_vars(); ++v) point[v] = NAN;
  }
  return CMN_OK;
}

extern "C" cmn_status cmn_solver_frontier(cmn_solver* s, double* boxes, double* lower_bounds, uint32_t* depths,
                                          uint64_t room, uint64_t* count)
{
  if (!s) return fail(CMN_INVALID_CONFIGURATION, "null solver");
  CK(cudaSetDevice(s->p->device));
  cmn_status st = pull_state(s);
  if (st != CMN_OK) return st;
  const uint64_t L = s->h_dev->pool_size;
  if (count) *count = L;
  const uint64_t m = std::min(L, room);
  if (m == 0) return CMN_OK;
  const uint32_t q = s->h_dev->parity;
  const int64_t n = s->p->host.n_vars();
  if (lower_bounds) CK(cudaMemcpyAsync(lower_bounds, s->b.lb[q], m * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  if (boxes || depths) {
    // unpack the boxes from the store in chunks of about 64 MB
    const uint64_t per = (uint64_t)(2 * n) * sizeof(double) + sizeof(uint32_t);
    const uint64_t chunk = std::max<uint64_t>(1, std::min<uint64_t>(m, (64ULL << 20) / per));
    double* d_boxes = nullptr;
    uint32_t* d_depths = nullptr;
    CK(cudaMalloc(&d_boxes, chunk * 2 * (uint64_t)n * sizeof(double) + 16));
    cudaError_t e = cudaMalloc(&d_depths, chunk * sizeof(uint32_t));
    for (uint64_t start = 0; e == cudaSuccess && start < m; start += chunk) {
      const uint64_t c = std::min(chunk, m - start);
      e = solver_frontier_gather(s->cfg, s->b, start, c, boxes ? d_boxes : nullptr, depths ? d_depths : nullptr,
                                 s->stream);
      if (e == cudaSuccess && boxes)
        e = cudaMemcpyAsync(boxes + start * 2 * n, d_boxes, c * 2 * n * sizeof(double), cudaMemcpyDeviceToHost,
                            s->stream);
      if (e == cudaSuccess && depths)
        e = cudaMemcpyAsync(depths + start, d_depths, c * sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    }
    cudaFree(d_depths);
    cudaFree(d_boxes);
    CK(e);
  }
  CK(cudaStreamSynchronize(s->stream));
  return CMN_OK;
}

static bool gap_closed_host(double gub, double bound, double tol)
{
  return gub - bound <= tol * std::max(1.0, std::fabs(gub));
}

extern "C" cmn_status cmn_solver_outcome(cmn_solver* s, cmn_outcome* out)
{
  if (!s || !out) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  CK(cudaSetDevice(s->p->device));
  CK(solver_pool_stats(s->cfg, s->b, s->d_viable, s->stream));
  CK(cudaMemcpyAsync(s->h_viable, s->d_viable, sizeof(uint64_t), cudaMemcpyDeviceToHost, s->stream));
  cmn_status st = pull_state(s);
  if (st != CMN_OK) return st;
  const SolverDev& d = *s->h_dev;
  const double tol = s->opts.tolerance;
  const bool pending_empty = d.pool_size == 0;
  const double frontier_min = pending_empty ? DBL_MAX : [&] {
    const uint64_t k = d.pool_min_key;
    const uint64_t u = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
    double x;
    std::memcpy(&x, &u, 8);
    return x;
  }();
  const bool found = d.gub < DBL_MAX;
  const uint64_t viable = *s->h_viable;
  std::memset(out, 0, sizeof *out);
  // finalise_bounds (search/epilogue.hpp:89-127)
  const double dropped_min = d.dropped_lb_min;
  const bool lost_nothing = d.counters.dropped_viable == 0;
  out->proven_optimal =
      found && (d.converged || pending_empty || viable == 0) && gap_closed_host(d.gub, dropped_min, tol);
  if (out->proven_optimal) {
    out->lower_bound = d.gub;
  } else if (pending_empty && lost_nothing) {
    out->infeasible = 1;
    out->lower_bound = d.glb;
  } else {
    double g = std::min(pending_empty ? DBL_MAX : frontier_min, dropped_min);
    if (found) g = std::min(g, d.gub);
    out->lower_bound = g;
  }
  out->upper_bound = d.gub;
  if (!d.done) {
    out->stop_reason = CMN_STOP_RUNNING;
  } else if (d.converged) {
    out->stop_reason = CMN_STOP_CONVERGED;
  } else {
    out->stop_reason = pending_empty ? CMN_STOP_EXHAUSTED
                       : gap_closed_host(d.gub, d.glb, tol) ? CMN_STOP_CONVERGED
                                                            : CMN_STOP_ITERATION_LIMIT;
  }
  out->found_incumbent = found ? 1 : 0;
  out->frontier_size = d.pool_size;
  out->viable = viable;
  out->dropped_lb_min = dropped_min;
  out->elapsed_ms = s->elapsed_ms;
  out->counters = d.counters;
  out->counters.iterations = d.iterations;
  out->counters.expansions = d.expansions;
  return CMN_OK;
}

extern "C" cmn_status cmn_solver_phase_ms(cmn_solver* s, double* ms5)
{
  if (!s || !ms5) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  CK(cudaEventSynchronize(s->marks[4]));
  float t = 0;
  for (int i = 0; i < 4; ++i) {
    CK(cudaEventElapsedTime(&t, s->marks[i], s->marks[i + 1]));
    ms5[i] = t;
  }
  CK(cudaEventElapsedTime(&t, s->marks[0], s->marks[4]));
  ms5[4] = t;
  return CMN_OK;
}

extern "C" cmn_status cmn_solver_lazy_ms(cmn_solver* s, double* ms2)
{
  if (!s || !ms2) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  if (s->cfg.precision != CMN_PRECISION_FP32_LAZY)
    return fail(CMN_INVALID_CONFIGURATION, "the solver does not run the lazy form");
  CK(cudaEventSynchronize(s->marks[4]));
  float t = 0;
  CK(cudaEventElapsedTime(&t, s->marks[5], s->marks[6]));
  ms2[0] = t;
  CK(cudaEventElapsedTime(&t, s->marks[1], s->marks[7]));
  ms2[1] = t;
  return CMN_OK;
}

extern "C" uint64_t cmn_solver_kernels_per_iteration(const cmn_solver* s) { return s ? s->kernels_per_iter : 0; }

namespace cmn {
cudaError_t launch_fma_peak(int precision, int grid, int threads, int iters, void* sink, cudaStream_t s);
}

extern "C" cmn_status cmn_measure_fma_peak(int32_t precision, double* tflops)
{
  if (!tflops) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  const int threads = 256, iters = 4096;
  const int grid = sm_count() * 8;
  void* sink = nullptr;
  CK(cudaMalloc(&sink, (size_t)grid * threads * sizeof(double)));
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  CK(launch_fma_peak(precision, grid, threads, iters, sink, nullptr));  // warm-up
  CK(cudaEventRecord(a, nullptr));
  const int reps = 5;
  for (int r = 0; r < reps; ++r) CK(launch_fma_peak(precision, grid, threads, iters, sink, nullptr));
  CK(cudaEventRecord(b, nullptr));
  CK(cudaEventSynchronize(b));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(sink);
  // 8 independent FMA chains per thread per iteration, 2 flops each
  const double flops = 2.0 * 8.0 * iters * (double)grid * threads * reps;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return CMN_OK;
}

extern "C" cmn_status cmn_solve(const cmn_problem* p, const cmn_solve_options* opts, cmn_outcome* outcome,
                                double* best_point)
{
  cmn_solver* s = nullptr;
  cmn_status st = cmn_solver_create(p, opts, &s);
  if (st != CMN_OK) return st;
  st = cmn_solver_step(s, 0);
  if (st == CMN_OK && outcome) st = cmn_solver_outcome(s, outcome);
  if (st == CMN_OK && best_point) {
    int32_t found = 0;
    st = cmn_query_incumbent(s, best_point, &found);
  }
  cmn_solver_destroy(s);
  return st;
}
