// batch.cu -- the C ABI of the multi-instance batch (cmn_batch_*): slot
// management, one captured iteration graph over every slot, host mirrors
// of the per-instance state.  No exception leaves this file.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/cuminlp_gb300.h"
#include "batch.hpp"
#include "handles.hpp"
#include "launch.hpp"
#include "policy.cuh"

using namespace cmn;

namespace {

cmn_status fail(cmn_status st, const std::string& msg) { return set_error(st, msg); }

#define BCK(call)                                                                                    \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess) return fail(CMN_CUDA_ERROR, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

using Clock = std::chrono::steady_clock;

bool gap_closed_host(double gub, double bound, double tol)
{
  return gub - bound <= tol * std::max(1.0, std::fabs(gub));
}

double key_to_lb(uint64_t k)
{
  const uint64_t u = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
  double x;
  std::memcpy(&x, &u, 8);
  return x;
}

// the options every instance of a batch shares
bool same_shared(const cmn_solve_options& a, const cmn_solve_options& b)
{
  return a.precision == b.precision && a.bisection_budget == b.bisection_budget &&
         a.batch_parents == b.batch_parents && a.frontier_cap == b.frontier_cap &&
         a.sample_points == b.sample_points && a.sample_all == b.sample_all &&
         a.relative_width == b.relative_width && a.max_cycle_size == b.max_cycle_size &&
         a.enumerate_cap == b.enumerate_cap;
}

}  // namespace

struct cmn_batch {
  cmn_batch_config conf{};
  BatchCfg cfg{};
  BatchBufs b{};
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  InstState* h_st = nullptr;  // pinned mirror, valid after pull()
  std::vector<InstDesc> h_desc;
  std::vector<uint32_t> h_order;  // BatchBufs::order on the host

  // Slots by descending program length (free slots, length 0, last; ties by
  // slot), uploaded as the launches' walk order.  The order changes only
  // which thread evaluates which child, never a result.
  cudaError_t upload_order()
  {
    h_order.resize(cfg.K);
    for (uint64_t i = 0; i < cfg.K; ++i) h_order[i] = (uint32_t)i;
    std::stable_sort(h_order.begin(), h_order.end(),
                     [&](uint32_t a, uint32_t x) { return h_desc[a].prog_len > h_desc[x].prog_len; });
    // pageable source: the copy is staged before the call returns
    return cudaMemcpyAsync(const_cast<uint32_t*>(b.order), h_order.data(), sizeof(uint32_t) * cfg.K,
                           cudaMemcpyHostToDevice, stream);
  }
  std::vector<const cmn_problem*> prob;
  std::vector<cmn_solve_options> opts;
  std::vector<uint8_t> busy;
  std::vector<Clock::time_point> t_add;
  std::vector<double> elapsed_ms;  // add -> first step that saw it stopped
  std::vector<void*> allocs;
  uint64_t alloc_bytes = 0;
  bool fresh = false;  // h_st matches the device: nothing enqueued since pull()
  int eval_grid = 1;
  BatchGrids grids;
  uint64_t kernels_per_iter = 0;
  cudaEvent_t marks[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};

  ~cmn_batch()
  {
    int cur = 0;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != device) cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    for (cudaEvent_t ev : marks)
      if (ev) cudaEventDestroy(ev);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (void* a : allocs) cudaFree(a);
    if (h_st) cudaFreeHost(h_st);
    if (stream) cudaStreamDestroy(stream);
    if (cur != device) cudaSetDevice(cur);
  }

  template <typename T>
  cudaError_t alloc(T** ptr, size_t n)
  {
    *ptr = nullptr;
    const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(ptr), bytes);
    if (e == cudaSuccess) {
      allocs.push_back(*ptr);
      alloc_bytes += bytes;
    }
    return e;
  }

  cmn_status pull()
  {
    BCK(cudaMemcpyAsync(h_st, b.st, sizeof(InstState) * cfg.K, cudaMemcpyDeviceToHost, stream));
    BCK(cudaStreamSynchronize(stream));
    const Clock::time_point now = Clock::now();
    for (uint64_t i = 0; i < cfg.K; ++i)
      if (busy[i] && h_st[i].done && elapsed_ms[i] < 0)
        elapsed_ms[i] = std::chrono::duration<double, std::milli>(now - t_add[i]).count();
    fresh = true;
    return CMN_OK;
  }

  uint64_t running() const
  {
    uint64_t r = 0;
    for (uint64_t i = 0; i < cfg.K; ++i)
      if (busy[i] && !h_st[i].done) ++r;
    return r;
  }
};

extern "C" cmn_status cmn_batch_create(const cmn_batch_config* config, cmn_batch** out)
{
  if (!config || !out) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  *out = nullptr;
  const cmn_batch_config& cf = *config;
  const cmn_solve_options& o = cf.shared;
  if (cf.slots < 1) return fail(CMN_INVALID_CONFIGURATION, "slots must be at least 1");
  if (cf.max_vars < 1) return fail(CMN_INVALID_CONFIGURATION, "max_vars must be at least 1");
  if (cf.max_program_slots < -1) return fail(CMN_INVALID_CONFIGURATION, "max_program_slots must be >= -1");
  if (o.bisection_budget < 1 || o.bisection_budget > 12)
    return fail(CMN_INVALID_CONFIGURATION, "bisection_budget must be within [1, 12] for a batch");
  if (o.sample_points < 1) return fail(CMN_INVALID_CONFIGURATION, "sample_points must be at least 1");
  if (o.batch_parents < 1 || o.frontier_cap < 1)
    return fail(CMN_INVALID_CONFIGURATION, "batch_parents and frontier_cap must be at least 1");
  if (o.max_cycle_size > 64) return fail(CMN_INVALID_CONFIGURATION, "max_cycle_size exceeds kMaxSlots (64)");
  if (o.precision != CMN_PRECISION_FP64 && o.precision != CMN_PRECISION_FP32_SCREEN &&
      o.precision != CMN_PRECISION_FP32_LAZY)
    return fail(CMN_INVALID_CONFIGURATION, "unknown precision");
  if (cf.max_segments < 0) return fail(CMN_INVALID_CONFIGURATION, "max_segments must not be negative");
  if (o.batch_parents > (uint64_t)kMiSortMax || o.frontier_cap > (uint64_t)kMiSortMax ||
      o.frontier_cap + (o.batch_parents << o.bisection_budget) > (uint64_t)kMiSortMax)
    return fail(CMN_INVALID_CONFIGURATION, "frontier_cap + batch_parents * 2^bisection_budget must be <= " +
                                               std::to_string(kMiSortMax) + " for a batch");
  const uint64_t child_stride = o.batch_parents << o.bisection_budget;
  if (cf.slots > (1ull << 31) / child_stride)
    return fail(CMN_INVALID_CONFIGURATION, "slots * batch_parents * 2^bisection_budget above 2^31");
  try {
    BCK(cudaSetDevice(cf.device));
    BCK(ensure_kernel_attributes());
    const int max_smem = max_dynamic_smem();
    const bool fp32 = o.precision == CMN_PRECISION_FP32_SCREEN;
    const bool lazy = o.precision == CMN_PRECISION_FP32_LAZY;
    const int64_t n_max = cf.max_vars;
    // program slots that fit beside the split variables in the FP64 bound
    // tile (the certify pass of the FP32 form is FP64 too) and beside
    // n_max variables in the sample tile
    const int64_t fit_eval = ((int64_t)max_smem / kEvalThreads - 20 * (int64_t)o.bisection_budget) / 16;
    const int64_t fit_smp = (int64_t)max_smem / (8 * kEvalThreads) - n_max;
    const int64_t fit = std::min(fit_eval, fit_smp);
    if (fit < 0) return fail(CMN_INVALID_CONFIGURATION, "max_vars too large for the evaluator's shared-memory tile");
    int64_t slots_max = cf.max_program_slots < 0 ? fit : cf.max_program_slots;
    if (slots_max > fit)
      return fail(CMN_INVALID_CONFIGURATION, "max_program_slots (" + std::to_string(slots_max) +
                                                 ") does not fit beside max_vars in shared memory (at most " +
                                                 std::to_string(fit) + ")");
    cmn_batch* s = new cmn_batch();
    s->conf = cf;
    s->device = cf.device;
    BatchCfg& c = s->cfg;
    c.n_max = (int)n_max;
    c.slots_max = (int)slots_max;
    c.log2C = o.bisection_budget;
    c.max_slots = o.bisection_budget;
    c.precision = o.precision;
    c.sample_all = o.sample_all;
    c.relative = o.relative_width;
    c.S = o.sample_points;
    c.e_max = o.batch_parents;
    c.cap = o.frontier_cap;
    c.P = o.frontier_cap + child_stride;
    c.K = cf.slots;
    c.child_stride = child_stride;
    c.max_cycle = (int64_t)o.max_cycle_size;
    c.enumerate_cap = (int64_t)o.enumerate_cap;
    c.seg_max = lazy ? (cf.max_segments > 0 ? cf.max_segments : (int)n_max + 1) : 0;
    const uint64_t K = c.K, nm = (uint64_t)n_max, G = K * child_stride;

    BatchBufs& b = s->b;
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    auto A = [&](auto** ptr, size_t count) {
      if (e == cudaSuccess) e = s->alloc(ptr, count);
    };
    A(&b.desc, K);
    A(&b.st, K);
    A(&b.lo, K * nm * c.P);
    A(&b.hi, K * nm * c.P);
    A(&b.lb, K * c.P);
    A(&b.depth, K * c.P);
    A(&b.plo, K * nm * c.e_max);
    A(&b.phi, K * nm * c.e_max);
    if (fp32 || lazy) {
      A(&b.plo32, K * nm * c.e_max);
      A(&b.phi32, K * nm * c.e_max);
    }
    if (lazy) {
      A(&b.plb, K * c.e_max);
      A(&b.pfeas, K * c.e_max);
      A(&b.inc_common, 2 * K * (uint64_t)c.seg_max * c.e_max);
      A(&b.inc_parts, 2 * K * (uint64_t)c.seg_max * child_stride);
      A(&b.cbest, G);
      A(&b.vrun, K + 2);
      A(&b.vlg, K);
    }
    A(&b.pdepth, K * c.e_max);
    A(&b.pinfo, K * c.e_max);
    A(&b.slots, K * c.e_max * (uint64_t)c.max_slots);
    EnumCand* ec = nullptr;
    BisCand* bc = nullptr;
    A(&ec, K * c.e_max * nm);
    A(&bc, K * c.e_max * nm);
    b.enum_scratch = ec;
    b.bis_scratch = bc;
    A(&b.heap_scratch, K * c.e_max * nm);
    A(&b.clb, G);
    A(&b.cstate, G);
    A(&b.cval, G);
    A(&b.ce, G);
    A(&b.list, G);
    A(&b.list_count, 1);
    A(&b.block_counts, (G + 511) / 512);
    A(&b.block_offsets, (G + 511) / 512);
    A(&b.child_base, K + 2);
    uint32_t* order = nullptr;
    A(&order, K);
    b.order = order;
    A(&b.best_point, K * nm);
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&s->h_st), sizeof(InstState) * K);
    if (e != cudaSuccess) {
      delete s;
      if (e == cudaErrorMemoryAllocation)
        return fail(CMN_OVER_BUDGET, "the batch's pools do not fit in device memory (slots / max_vars / frontier_cap)");
      return fail(CMN_CUDA_ERROR, std::string("batch allocation: ") + cudaGetErrorString(e));
    }
    s->h_desc.assign(K, InstDesc{});
    s->prob.assign(K, nullptr);
    s->opts.assign(K, o);
    s->busy.assign(K, 0);
    s->t_add.assign(K, Clock::now());
    s->elapsed_ms.assign(K, -1.0);
    std::memset(s->h_st, 0, sizeof(InstState) * K);
    for (uint64_t i = 0; i < K; ++i) s->h_st[i].done = 1;
    e = cudaMemsetAsync(b.desc, 0, sizeof(InstDesc) * K, s->stream);
    if (e == cudaSuccess) e = s->upload_order();
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.st, s->h_st, sizeof(InstState) * K, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    const int occ = std::max(1, std::min(batch_eval_occupancy(c, fp32), batch_sample_occupancy(c)));
    const uint64_t need = (G * 32 + kEvalThreads - 1) / kEvalThreads;  // room for 32 lanes per child
    s->eval_grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)sm_count() * occ));
    c.g_max = 32;
    c.eval_capacity = (uint64_t)s->eval_grid * kEvalThreads;
    c.sample_capacity = c.eval_capacity;
    s->grids = batch_grids(c, s->eval_grid);
    for (int i = 0; i < 5 && e == cudaSuccess; ++i) e = cudaEventCreate(&s->marks[i]);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      cudaError_t e2 = batch_iteration(c, b, s->grids, s->stream, s->marks);
      e = cudaStreamEndCapture(s->stream, &s->graph);
      if (e2 != cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) {
      size_t nn = 0;
      e = cudaGraphGetNodes(s->graph, nullptr, &nn);
      std::vector<cudaGraphNode_t> nodes(nn);
      if (e == cudaSuccess && nn) e = cudaGraphGetNodes(s->graph, nodes.data(), &nn);
      for (size_t i = 0; i < nn && e == cudaSuccess; ++i) {
        cudaGraphNodeType t;
        e = cudaGraphNodeGetType(nodes[i], &t);
        if (t == cudaGraphNodeTypeKernel) ++s->kernels_per_iter;
      }
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&s->exec, s->graph, 0);
    if (e != cudaSuccess) {
      delete s;
      return fail(CMN_CUDA_ERROR, std::string("batch setup: ") + cudaGetErrorString(e));
    }
    *out = s;
    return CMN_OK;
  } catch (const std::bad_alloc&) {
    return fail(CMN_INTERNAL, "host allocation failed");
  }
}

extern "C" void cmn_batch_destroy(cmn_batch* s) { delete s; }

extern "C" cmn_status cmn_batch_add(cmn_batch* s, const cmn_problem* p, const cmn_solve_options* opts,
                                    uint64_t* slot)
{
  if (!s || !p || !opts || !slot) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  if (!same_shared(*opts, s->conf.shared))
    return fail(CMN_INVALID_CONFIGURATION, "the instance's shared options differ from the batch's");
  if (p->device != s->device) return fail(CMN_INVALID_CONFIGURATION, "problem and batch are on different devices");
  if (!p->prog.interval_supported)
    return fail(CMN_INVALID_CONFIGURATION, "no interval implementation for op " + p->prog.unsupported_op);
  const int64_t n = p->host.n_vars();
  if (n > s->cfg.n_max)
    return fail(CMN_INVALID_CONFIGURATION, "problem has " + std::to_string(n) + " variables; the batch takes " +
                                               std::to_string(s->cfg.n_max));
  if (p->prog.n_slots > s->cfg.slots_max)
    return fail(CMN_INVALID_CONFIGURATION, "problem program needs " + std::to_string(p->prog.n_slots) +
                                               " slots; the batch takes " + std::to_string(s->cfg.slots_max));
  uint64_t k = 0;
  while (k < s->cfg.K && s->busy[k]) ++k;
  if (k == s->cfg.K) return fail(CMN_OVER_BUDGET, "no free slot in the batch");
  BCK(cudaSetDevice(s->device));
  InstDesc d{};
  d.prog64 = p->d_prog64;
  d.prog32 = p->d_prog32;
  d.kinds = p->d_kinds;
  d.root_lb = p->d_root_lb;
  d.root_ub = p->d_root_ub;
  d.prog_len = (int32_t)p->prog.code64.size();
  d.n_vars = (int32_t)n;
  d.n_slots = p->prog.n_slots;
  d.sched = p->d_sched;
  d.g_max = p->d_sched ? p->prog.group_max : 1;
  if (s->cfg.precision == CMN_PRECISION_FP32_LAZY) {
    d.prog32p = p->d_prog32p;
    if (p->d_inc_seg != nullptr) {
      if (p->prog.inc_segments > s->cfg.seg_max)
        return fail(CMN_INVALID_CONFIGURATION, "problem program has " + std::to_string(p->prog.inc_segments) +
                                                   " sum-chain segments; the batch takes " +
                                                   std::to_string(s->cfg.seg_max) + " (max_segments)");
      d.inc_seg = p->d_inc_seg;
      d.inc_off = p->d_inc_off;
      d.inc_pcs = p->d_inc_pcs;
      d.inc_segments = p->prog.inc_segments;
    }
  }
  d.active = 1;
  d.iter_limit = opts->iter_limit;
  d.batch_iter_limit = opts->batch_iter_limit;
  d.tolerance = opts->tolerance;
  s->h_desc[k] = d;
  // pageable source: the copy is staged before the call returns
  BCK(cudaMemcpyAsync(s->b.desc + k, &s->h_desc[k], sizeof(InstDesc), cudaMemcpyHostToDevice, s->stream));
  BCK(s->upload_order());
  const double gub0 = opts->has_known_primal ? opts->known_primal_bound : DBL_MAX;
  BCK(batch_init_slot(s->cfg, s->b, k, gub0, s->stream));
  s->prob[k] = p;
  s->opts[k] = *opts;
  s->busy[k] = 1;
  s->h_st[k].done = 0;
  s->fresh = false;
  s->t_add[k] = Clock::now();
  s->elapsed_ms[k] = -1.0;
  *slot = k;
  return CMN_OK;
}

extern "C" cmn_status cmn_batch_step(cmn_batch* s, uint64_t max_iterations, uint64_t* running)
{
  if (!s) return fail(CMN_INVALID_CONFIGURATION, "null batch");
  BCK(cudaSetDevice(s->device));
  const Clock::time_point t0 = Clock::now();
  cmn_status st = s->pull();
  if (st != CMN_OK) return st;
  uint64_t done_iters = 0, burst = 1;
  while (s->running() > 0 && (max_iterations == 0 || done_iters < max_iterations)) {
    uint64_t k = burst;
    if (max_iterations) k = std::min<uint64_t>(k, max_iterations - done_iters);
    s->fresh = false;
    for (uint64_t i = 0; i < k; ++i) BCK(cudaGraphLaunch(s->exec, s->stream));
    done_iters += k;
    st = s->pull();
    if (st != CMN_OK) return st;
    const double ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
    if (ms < 50.0 && burst < 64) burst *= 2;
  }
  if (running) *running = s->running();
  return CMN_OK;
}

extern "C" cmn_status cmn_batch_launch(cmn_batch* s, uint64_t iterations)
{
  if (!s) return fail(CMN_INVALID_CONFIGURATION, "null batch");
  BCK(cudaSetDevice(s->device));
  s->fresh = false;
  for (uint64_t i = 0; i < iterations; ++i) BCK(cudaGraphLaunch(s->exec, s->stream));
  return CMN_OK;
}

extern "C" cmn_status cmn_batch_query(cmn_batch* s, int32_t* idle)
{
  if (!s || !idle) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  BCK(cudaSetDevice(s->device));
  const cudaError_t e = cudaStreamQuery(s->stream);
  if (e == cudaErrorNotReady) {
    *idle = 0;
    return CMN_OK;
  }
  BCK(e);
  *idle = 1;
  return CMN_OK;
}

extern "C" cmn_status cmn_batch_sync(cmn_batch* s, uint64_t* running)
{
  if (!s) return fail(CMN_INVALID_CONFIGURATION, "null batch");
  BCK(cudaSetDevice(s->device));
  cmn_status st = s->pull();
  if (st != CMN_OK) return st;
  if (running) *running = s->running();
  return CMN_OK;
}

extern "C" cmn_status cmn_batch_totals(cmn_batch* s, cmn_counters* sum, uint64_t* running)
{
  if (!s || !sum) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  BCK(cudaSetDevice(s->device));
  cmn_status st = s->fresh ? CMN_OK : s->pull();
  if (st != CMN_OK) return st;
  constexpr int kN = (int)(sizeof(cmn_counters) / sizeof(uint64_t));
  uint64_t acc[kN] = {0};
  static_assert(sizeof(cmn_counters) == sizeof(acc), "cmn_counters holds uint64 fields only");
  for (uint64_t k = 0; k < s->cfg.K; ++k) {
    if (!s->busy[k]) continue;
    cmn_counters c = s->h_st[k].counters;
    c.iterations = s->h_st[k].iterations;
    c.expansions = s->h_st[k].expansions;
    uint64_t v[kN];
    std::memcpy(v, &c, sizeof v);
    for (int i = 0; i < kN; ++i) acc[i] += v[i];
  }
  std::memcpy(sum, acc, sizeof acc);
  if (running) *running = s->running();
  return CMN_OK;
}

extern "C" cmn_status cmn_batch_phase_ms(cmn_batch* s, double* ms5)
{
  if (!s || !ms5) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  BCK(cudaSetDevice(s->device));
  BCK(cudaEventSynchronize(s->marks[4]));
  float t = 0;
  for (int i = 0; i < 4; ++i) {
    BCK(cudaEventElapsedTime(&t, s->marks[i], s->marks[i + 1]));
    ms5[i] = t;
  }
  BCK(cudaEventElapsedTime(&t, s->marks[0], s->marks[4]));
  ms5[4] = t;
  return CMN_OK;
}

extern "C" uint64_t cmn_batch_slot_bytes(const cmn_batch* s)
{
  return s && s->cfg.K ? (s->alloc_bytes + s->cfg.K - 1) / s->cfg.K : 0;
}

extern "C" cmn_status cmn_batch_poll(const cmn_batch* s, uint64_t slot, int32_t* done)
{
  if (!s || !done) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  if (slot >= s->cfg.K || !s->busy[slot]) return fail(CMN_INVALID_CONFIGURATION, "slot not occupied");
  *done = s->h_st[slot].done ? 1 : 0;
  return CMN_OK;
}

extern "C" cmn_status cmn_batch_outcome(cmn_batch* s, uint64_t slot, cmn_outcome* out, double* best_point)
{
  if (!s || !out) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  if (slot >= s->cfg.K || !s->busy[slot]) return fail(CMN_INVALID_CONFIGURATION, "slot not occupied");
  BCK(cudaSetDevice(s->device));
  cmn_status st = s->fresh ? CMN_OK : s->pull();
  if (st != CMN_OK) return st;
  const InstState& d = s->h_st[slot];
  const double tol = s->opts[slot].tolerance;
  const bool pending_empty = d.pool_size == 0;
  const double frontier_min = pending_empty ? DBL_MAX : key_to_lb(d.pool_min_key);
  const bool found = d.gub < DBL_MAX;
  std::memset(out, 0, sizeof *out);
  // finalise_bounds (search/epilogue.hpp:89-127)
  const double dropped_min = d.dropped_lb_min;
  const bool lost_nothing = d.counters.dropped_viable == 0;
  out->proven_optimal =
      found && (d.converged || pending_empty || d.viable == 0) && gap_closed_host(d.gub, dropped_min, tol);
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
  out->viable = d.viable;
  out->dropped_lb_min = dropped_min;
  out->elapsed_ms = s->elapsed_ms[slot] >= 0
                        ? s->elapsed_ms[slot]
                        : std::chrono::duration<double, std::milli>(Clock::now() - s->t_add[slot]).count();
  out->counters = d.counters;
  out->counters.iterations = d.iterations;
  out->counters.expansions = d.expansions;
  if (best_point) {
    const int n = s->h_desc[slot].n_vars;
    BCK(cudaMemcpyAsync(best_point, s->b.best_point + slot * (uint64_t)s->cfg.n_max, sizeof(double) * n,
                        cudaMemcpyDeviceToHost, s->stream));
    BCK(cudaStreamSynchronize(s->stream));
  }
  return CMN_OK;
}

extern "C" cmn_status cmn_batch_frontier(cmn_batch* s, uint64_t slot, double* boxes, double* lower_bounds,
                                         uint32_t* depths, uint64_t room, uint64_t* count)
{
  if (!s || !count) return fail(CMN_INVALID_CONFIGURATION, "null argument");
  if (slot >= s->cfg.K || !s->busy[slot]) return fail(CMN_INVALID_CONFIGURATION, "slot not occupied");
  BCK(cudaSetDevice(s->device));
  cmn_status st = s->fresh ? CMN_OK : s->pull();
  if (st != CMN_OK) return st;
  const uint64_t L = s->h_st[slot].pool_size;
  *count = L;
  const uint64_t m = std::min(L, room);
  if (m == 0) return CMN_OK;
  const BatchCfg& c = s->cfg;
  const int n = s->h_desc[slot].n_vars;
  const size_t base = (size_t)slot * c.n_max * c.P;
  if (boxes) {
    std::vector<double> lo((size_t)n * m), hi((size_t)n * m);
    BCK(cudaMemcpy2DAsync(lo.data(), m * sizeof(double), s->b.lo + base, c.P * sizeof(double), m * sizeof(double), n,
                          cudaMemcpyDeviceToHost, s->stream));
    BCK(cudaMemcpy2DAsync(hi.data(), m * sizeof(double), s->b.hi + base, c.P * sizeof(double), m * sizeof(double), n,
                          cudaMemcpyDeviceToHost, s->stream));
    BCK(cudaStreamSynchronize(s->stream));
    for (uint64_t i = 0; i < m; ++i)
      for (int v = 0; v < n; ++v) {
        boxes[2 * (i * n + v)] = lo[(size_t)v * m + i];
        boxes[2 * (i * n + v) + 1] = hi[(size_t)v * m + i];
      }
  }
  if (lower_bounds)
    BCK(cudaMemcpyAsync(lower_bounds, s->b.lb + (size_t)slot * c.P, m * sizeof(double), cudaMemcpyDeviceToHost,
                        s->stream));
  if (depths)
    BCK(cudaMemcpyAsync(depths, s->b.depth + (size_t)slot * c.P, m * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                        s->stream));
  BCK(cudaStreamSynchronize(s->stream));
  return CMN_OK;
}

extern "C" cmn_status cmn_batch_release(cmn_batch* s, uint64_t slot)
{
  if (!s) return fail(CMN_INVALID_CONFIGURATION, "null batch");
  if (slot >= s->cfg.K || !s->busy[slot]) return fail(CMN_INVALID_CONFIGURATION, "slot not occupied");
  BCK(cudaSetDevice(s->device));
  s->h_desc[slot] = InstDesc{};
  BCK(cudaMemcpyAsync(s->b.desc + slot, &s->h_desc[slot], sizeof(InstDesc), cudaMemcpyHostToDevice, s->stream));
  BCK(s->upload_order());
  s->busy[slot] = 0;
  s->prob[slot] = nullptr;
  s->h_st[slot].done = 1;
  return CMN_OK;
}

extern "C" void* cmn_batch_stream(cmn_batch* s) { return s ? reinterpret_cast<void*>(s->stream) : nullptr; }

extern "C" uint64_t cmn_batch_kernels_per_iteration(const cmn_batch* s) { return s ? s->kernels_per_iter : 0; }

extern "C" cmn_status cmn_batch_solve(const cmn_batch_config* config, const cmn_problem* const* problems,
                                      const cmn_solve_options* opts, uint64_t count, cmn_outcome* outcomes,
                                      double* best_points, uint64_t point_stride)
{
  if (!config || (!problems && count) || !opts || (!outcomes && count))
    return fail(CMN_INVALID_CONFIGURATION, "null argument");
  cmn_batch* s = nullptr;
  cmn_status st = cmn_batch_create(config, &s);
  if (st != CMN_OK) return st;
  std::vector<uint64_t> owner(s->cfg.K, ~0ULL);  // slot -> problem index
  uint64_t next = 0, open = 0;
  while (st == CMN_OK && (next < count || open > 0)) {
    while (st == CMN_OK && next < count && open < s->cfg.K) {
      uint64_t slot = 0;
      st = cmn_batch_add(s, problems[next], &opts[next], &slot);
      if (st == CMN_OK) {
        owner[slot] = next++;
        ++open;
      }
    }
    if (st != CMN_OK) break;
    uint64_t running = 0;
    st = cmn_batch_step(s, next < count ? 8 : 0, &running);
    for (uint64_t k = 0; st == CMN_OK && k < s->cfg.K; ++k) {
      if (owner[k] == ~0ULL || !s->h_st[k].done) continue;
      const uint64_t i = owner[k];
      st = cmn_batch_outcome(s, k, &outcomes[i], best_points ? best_points + i * point_stride : nullptr);
      if (st == CMN_OK) st = cmn_batch_release(s, k);
      owner[k] = ~0ULL;
      --open;
    }
  }
  cmn_batch_destroy(s);
  return st;
}
