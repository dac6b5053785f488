// eval_kernels.cu -- the fused interval evaluator (a), the point sampler
// (b) and the incumbent ArgMin, over children decoded from parent boxes.
//
// One thread owns one child box.  The interval kernels keep no copy of the
// box: a variable is read from the parent's planes (the siblings of a
// parent read the same addresses, so those loads hit L1), except the
// child's few split variables, which sit in the thread's shared-memory
// column beside its program slots.  Shared memory per thread is then
// independent of the number of variables, which keeps enough warps resident
// to saturate the FP64 pipe.  The sampler stages each point in shared
// memory, plane-major ([plane][thread]) so every warp access is one
// conflict-free row.  Nothing is shared between threads, so the kernels
// need no barriers and a thread whose child is invalid simply skips it.
//
// Replaces graph/kernels.cuh:76-461 (broadcast/apply root kernels, one op
// kernel per DAG node, feasibility, extract, mask, gather) and the CUB
// ArgMin of graph/replay.cuh:439-474.
#include <cfloat>
#include <cstdint>

#include "eval_core.cuh"
#include "kernels.cuh"
#include "launch.hpp"

namespace cmn {

__device__ __forceinline__ void child_of(int log2C, uint64_t g, uint64_t& k, uint64_t& r)
{
  if (log2C < 0) {
    k = 0;
    r = g;
  } else {
    k = g >> log2C;
    r = g & ((1ULL << log2C) - 1ULL);
  }
}

// The variable source of child (k, r): the parent's planes `plo`/`phi`
// (FP64, or FP32 rounded outward) plus the child's split variables, decoded
// from the parent's FP64 bounds into this thread's columns olo/ohi/ovid.
// `dup` is set when a slot digit is at or past its domain size
// (region::is_duplicate_child).
template <typename T, typename S>
__device__ __forceinline__ ChildVars<T, S> child_vars(const EvalArgs& a, const S* plo, const S* phi, uint64_t k,
                                                      uint64_t r, T* olo, T* ohi, int32_t* ovid, int stride,
                                                      bool& dup)
{
  ChildVars<T, S> cv;
  cv.plo = plo + k;
  cv.phi = phi + k;
  cv.pstride = a.pstride;
  cv.mask = 0;
  cv.olo = olo;
  cv.ohi = ohi;
  cv.ovid = ovid;
  cv.count = 0;
  cv.stride = stride;
  dup = false;
  if (a.pinfo != nullptr) {
    const uint32_t count = a.pinfo[k].count;
    const SlotPlan* sp = a.slots + k * (uint64_t)a.max_slots;
    for (uint32_t j = 0; j < count; ++j) {
      const SlotPlan s = sp[j];
      const uint64_t part = slot_part(r, s);
      if (part >= s.dom) dup = true;
      double lo, hi;
      slot_bounds(s, a.plo[(uint64_t)s.vid * a.pstride + k], a.phi[(uint64_t)s.vid * a.pstride + k], part, lo, hi);
      olo[j * stride] = Widen<T, double>::lo(lo);
      ohi[j * stride] = Widen<T, double>::hi(hi);
      ovid[j * stride] = (int32_t)s.vid;
      cv.mask |= 1ULL << (s.vid & 63);
    }
    cv.count = (int)count;
  }
  return cv;
}

// Shared memory of the interval kernels, per thread: the program slots
// (lo, hi) and up to `max_slots` split variables (lo, hi, id).
size_t eval_smem_bytes(int n_slots, int max_slots, bool fp32, int threads)
{
  const size_t t = fp32 ? 4 : 8;
  return ((2 * t) * (size_t)(n_slots + max_slots) + 4 * (size_t)max_slots) * (size_t)threads;
}

// Writes the verdict of child g of parent k (kModes as in eval_children).
template <typename T, int kMode>
__device__ __forceinline__ void write_verdict(const EvalArgs& a, uint64_t g, uint64_t k, const Verdict<T>& v,
                                              double gub)
{
  double lb = (double)v.obj.lo;
  if (kMode == 5 && a.parent_lb == nullptr) {
    // the solver's lazy form: the parent's FP64 verdict runs beside this
    // pass, and lazy_fold_kernel folds it in and settles every state but
    // these two
    a.out_lb[g] = lb;
    a.out_flag[g] = v.excluded ? kChildInfeasible : kChildScreened;
    return;
  }
  if (kMode == 5) {
    // the parent's certified bound holds for every child box inside it
    const double plb = a.parent_lb[k];
    lb = plb > lb ? plb : lb;
    a.out_lb[g] = lb;
    // a survivor whose bound lies within the band below the incumbent goes
    // to the FP64 pass, which may prune it; below the band FP64 could not
    a.out_flag[g] = v.excluded  ? kChildInfeasible
                    : lb > gub  ? kChildDominated
                    : lb >= certify_floor(gub) ? kChildScreened
                                               : kChildEligible;
    return;
  }
  if (kMode == 3 && a.parent_lb != nullptr) {  // lazy form's certify pass
    const double plb = a.parent_lb[k];
    lb = plb > lb ? plb : lb;
  }
  if (kMode == 0) {
    a.out_lb[g] = lb;
    if (a.out_ub) a.out_ub[g] = (double)v.obj.hi;
    // FP64: the reference predicate; FP32: not proven violated
    a.out_flag[g] = (uint8_t)(sizeof(T) == 8 ? v.feasible : !v.excluded);
  } else if (kMode == 2) {
    a.out_lb[g] = lb;
    a.out_flag[g] = v.excluded ? kChildInfeasible : (lb > gub ? kChildDominated : kChildScreened);
  } else {
    a.out_lb[g] = lb;
    a.out_flag[g] = !v.feasible ? kChildInfeasible : (lb > gub ? kChildDominated : kChildEligible);
  }
}

// Aggregate bounder (backend/aggregate/kernels.cuh:32-47 mask and the
// replay's per-child Min/Max, replay.cuh:497-556), fused: region r belongs
// to child r / agg_m; infeasible regions count as lb = +inf, ub = -inf.
// Minimum and maximum follow the total order of lb_key.  A warp whose
// active lanes share one child combines them before one pair of atomics.
// Every lane of the warp calls this.
__device__ __forceinline__ void aggregate_fold(const EvalArgs& a, bool active, uint64_t r, const Verdict<double>& v)
{
  const unsigned c = active ? (unsigned)(r / a.agg_m) : 0xffffffffu;
  unsigned long long kmin = lb_key(active && v.feasible ? v.obj.lo : INFINITY);
  unsigned long long kmax = lb_key(active && v.feasible ? v.obj.hi : -INFINITY);
  const unsigned any = __ballot_sync(0xffffffffu, active);
  if (any == 0) return;
  const unsigned cmin = __reduce_min_sync(0xffffffffu, c);
  const unsigned cmax = __reduce_max_sync(0xffffffffu, active ? c : 0u);
  if (cmin == cmax) {
    for (int off = 16; off > 0; off >>= 1) {
      const unsigned long long a1 = __shfl_xor_sync(0xffffffffu, kmin, off);
      const unsigned long long b1 = __shfl_xor_sync(0xffffffffu, kmax, off);
      kmin = a1 < kmin ? a1 : kmin;
      kmax = b1 > kmax ? b1 : kmax;
    }
    if ((threadIdx.x & 31) == (unsigned)(__ffs(any) - 1)) {
      atomicMin(a.agg_keys + cmin, kmin);
      atomicMax(a.agg_keys + a.agg_k + cmin, kmax);
    }
  } else if (active) {
    atomicMin(a.agg_keys + c, kmin);
    atomicMax(a.agg_keys + a.agg_k + c, kmax);
  }
}

// ---- program staging through shared memory ----
// The FP64 passes with one lane per box (kMode 0: roles and the lazy form's
// verdict of the staged parents; kMode 1: the solver's bound) read their
// program from shared memory: a block streams it in tiles of kStageTile
// instructions with the bulk-copy engine (cp.async.bulk, completion on an
// mbarrier), double-buffered, every thread of the block stepping through
// the tiles together.  Against reading the program through the read-only
// cache (CMN_STAGE_PROGRAM=0; the words of a tile are the same for every
// thread, so L1 already hits 93-96 %) it measured 0.7 % faster on the
// n = 64 bound (146.0 against 147.0 ms per 2^20 boxes).
#ifndef CMN_STAGE_PROGRAM
#define CMN_STAGE_PROGRAM 1
#endif
constexpr int kStageTile = 256;                 // instructions per tile (4 KiB)
constexpr uint32_t kStageSpinLimit = 1u << 24;  // try_wait rounds before a tile counts as lost
// dynamic shared memory the staging adds after a block's own layout: two
// tiles, two mbarriers and a flag (EvalArgs::stage_at gives the offset)
constexpr size_t kStageBytes = 2 * kStageTile * sizeof(Instr) + 32;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_init_fence()
{
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// thread 0: one arrival that also announces the bytes the copy will land
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// `bytes` (a multiple of 16) from global `src` to shared `dst` (both 16-byte
// aligned); completion is counted on `bar`
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Bounded wait for phase `parity` of `bar`: false when it did not complete.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity)
{
  for (uint32_t i = 0; i < kStageSpinLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// kMode 0 or 1, one lane per box, program tiles staged in shared memory.
// The block's trip count over boxes is uniform, so every thread reaches the
// barriers; a thread without a (live) box only steps through the tiles.
template <typename T, int kMode, typename S, bool kFused = false>
__device__ void eval_children_staged(const EvalArgs& a, const S* plo, const S* phi, uint64_t total, double gub,
                                     const Tile<T>& t, T* olo, T* ohi, int32_t* ovid)
{
  static_assert(kMode == 0 || kMode == 1, "staged program: the one-lane FP64 passes");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Instr(*tiles)[kStageTile] = reinterpret_cast<Instr(*)[kStageTile]>(smem_raw + a.stage_at);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + a.stage_at + 2 * kStageTile * sizeof(Instr));
  int& lost = *reinterpret_cast<int*>(bars + 2);
  const int B = blockDim.x;
  const int len = a.prog_len;
  const int ntiles = (len + kStageTile - 1) / kStageTile;
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init_fence();
    lost = 0;
  }
  __syncthreads();
  uint32_t seq = 0;  // tiles this block has consumed; tile `seq` lands in buffer seq & 1
  auto issue = [&](int tile, uint32_t q) {
    const int n = min(kStageTile, len - tile * kStageTile);
    mbar_arrive_expect_tx(&bars[q & 1], (uint32_t)n * 16u);
    bulk_copy_g2s(tiles[q & 1], a.prog + (size_t)tile * kStageTile, (uint32_t)n * 16u, &bars[q & 1]);
  };
  for (uint64_t bb = (uint64_t)blockIdx.x * B; bb < total; bb += (uint64_t)gridDim.x * B) {
    const uint64_t g = bb + threadIdx.x;
    bool live = g < total;
    uint64_t k = 0, r = 0;
    ChildVars<T, S> cv = {};
    if (live) {
      child_of(a.log2C, g, k, r);
      if (kMode != 0 && a.pinfo != nullptr) {
        const ParentInfo pi = a.pinfo[k];
        if (pi.fathom || r >= pi.nreg) {
          a.out_flag[g] = kChildNone;
          live = false;
        }
      }
    }
    if (live) {
      bool dup;
      cv = child_vars<T, S>(a, plo, phi, k, r, olo, ohi, ovid, B, dup);
      if (kMode != 0 && dup) {
        a.out_flag[g] = kChildDuplicate;
        live = false;
      }
    }
    Verdict<T> out = verdict_init<T>();
    Iv<T> acc = {T(0), T(0)};
    if (threadIdx.x == 0 && ntiles > 0) issue(0, seq);
    for (int tile = 0; tile < ntiles; ++tile, ++seq) {
      if (!mbar_wait_bounded(&bars[seq & 1], (seq >> 1) & 1)) lost = 1;
      __syncthreads();
      if (lost) {
        // a tile never arrived: flag it, wait once more (bounded) for that
        // copy, the only one in flight, and stop this block
        if (threadIdx.x == 0) {
          if (a.error != nullptr) atomicExch(a.error, 1u);
          mbar_wait_bounded(&bars[seq & 1], (seq >> 1) & 1);
        }
        return;
      }
      // every thread has seen tile `seq`; buffer (seq + 1) & 1 was last read
      // in the previous round, before the barrier above
      if (threadIdx.x == 0 && tile + 1 < ntiles) issue(tile + 1, seq + 1);
      const int pc0 = tile * kStageTile, pc1 = min(len, pc0 + kStageTile);
      if (live)
        interval_range_from<T, ChildVars<T, S>, SharedCode, kFused>(SharedCode{tiles[seq & 1], pc0}, pc0, pc1, cv, t, out,
                                                             acc);
      __syncthreads();
    }
    if (live) write_verdict<T, kMode>(a, g, k, out, gub);
  }
}

// Groups of 2^lg consecutive lanes share one child: each lane runs its
// segments of the program and the group combines the verdicts.  The loop
// bound is per block, so every lane of a warp reaches the shuffles.
template <typename T, int kMode, typename S, bool kFused = false>
__device__ void eval_children_grouped(const EvalArgs& a, const S* plo, const S* phi, uint64_t total, double gub,
                                      bool pass_through, int lg, const Tile<T>& t, T* olo, T* ohi, int32_t* ovid)
{
  const int B = blockDim.x;
  const int G = 1 << lg;
  const int lane = threadIdx.x & (G - 1);
  const uint64_t per_block = (uint64_t)(B >> lg);
  for (uint64_t base = (uint64_t)blockIdx.x * per_block; base < total; base += (uint64_t)gridDim.x * per_block) {
    const uint64_t idx = base + (threadIdx.x >> lg);
    bool live = idx < total;
    uint64_t g = 0, k = 0, r = 0;
    if (live) {
      g = (kMode == 3) ? (uint64_t)a.list[idx] : idx;
      child_of(a.log2C, g, k, r);
      if (kMode != 0 && kMode != 4 && a.pinfo != nullptr) {
        const ParentInfo pi = a.pinfo[k];
        if (pi.fathom || r >= pi.nreg) {
          if (kMode != 3 && lane == 0) a.out_flag[g] = kChildNone;
          live = false;
        }
      }
    }
    if (live && pass_through) {
      bool dup = false;
      const uint32_t count = a.pinfo[k].count;
      const SlotPlan* sp = a.slots + k * (uint64_t)a.max_slots;
      for (uint32_t j = 0; j < count; ++j) dup = dup || (slot_part(r, sp[j]) >= sp[j].dom);
      if (lane == 0) a.out_flag[g] = dup ? kChildDuplicate : kChildScreened;
      live = false;
    }
    Verdict<T> v = verdict_init<T>();
    if (live) {
      bool dup;
      const ChildVars<T, S> cv = child_vars<T, S>(a, plo, phi, k, r, olo, ohi, ovid, B, dup);
      if (kMode != 0 && kMode != 4 && dup) {
        if (lane == 0) a.out_flag[g] = kChildDuplicate;
        live = false;
      } else if (lg > 0) {
        v = run_interval_lane<T, ChildVars<T, S>, kFused>(a.prog, a.sched, lg, lane, cv, t);
      } else {  // one lane per box (the aggregate fold's loop): the whole program
        v = run_interval<T, ChildVars<T, S>, kFused>(a.prog, a.prog_len, cv, t);
      }
    }
    v = group_verdict<T>(v, G);
    if constexpr (kMode == 4) {
      aggregate_fold(a, live && lane == 0, r, v);
    } else {
      if (live && lane == 0) write_verdict<T, kMode>(a, g, k, v, gub);
    }
  }
}

// kMode 0: role / raw boxes -> out_lb, out_ub, out_flag = feasible
// kMode 1: solver FP64 -> out_lb, out_flag = ChildState
// kMode 2: solver FP32 screen -> out_lb (FP32 bound), out_flag = ChildState
// kMode 3: solver FP64 certify of a child list
// kMode 4: aggregate bounder fold
// kMode 5: solver lazy form, FP32 -> out_lb = max(FP32 bound, parent's
//          certified bound), out_flag = ChildState
template <typename T, int kMode, typename S, bool kStaged = false, bool kFused = false>
__device__ __forceinline__ void eval_children(const EvalArgs& a, const S* plo, const S* phi)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* base = reinterpret_cast<T*>(smem_raw);
  const int B = blockDim.x;
  const int ms = a.pinfo != nullptr ? a.max_slots : 0;
  Tile<T> t;  // program slots only
  t.lo = nullptr;
  t.hi = nullptr;
  t.slo = base;
  t.shi = base + (size_t)a.n_slots * B;
  t.stride = B;
  t.tid = threadIdx.x;
  T* olo = base + (size_t)2 * a.n_slots * B + threadIdx.x;
  T* ohi = olo + (size_t)ms * B;
  int32_t* ovid = reinterpret_cast<int32_t*>(base + (size_t)2 * (a.n_slots + ms) * B) + threadIdx.x;

  if (a.done != nullptr && *a.done) return;
  uint64_t total;
  if (kMode == 3) total = *a.list_count;
  else total = a.n_children_dev ? *a.n_children_dev : a.n_children;
  const double gub = a.gub ? *a.gub : DBL_MAX;
  // screen switched off for this iteration: every child goes to the FP64
  // certify pass unevaluated (duplicates and empty slots still classified)
  const bool pass_through = kMode == 2 && a.use_screen != nullptr && *a.use_screen == 0;

  const int lg = a.sched != nullptr ? lanes_per_box(total, a.capacity, a.g_max) : 0;
  if (lg > 0 || kMode == 4) {  // the aggregate fold needs whole warps: the grouped loop, even at one lane
    eval_children_grouped<T, kMode, S, kFused>(a, plo, phi, total, gub, pass_through, lg, t, olo, ohi, ovid);
    return;
  }
  if constexpr (kStaged) {
    eval_children_staged<T, kMode, S, kFused>(a, plo, phi, total, gub, t, olo, ohi, ovid);
    return;
  }
  for (uint64_t idx = (uint64_t)blockIdx.x * B + threadIdx.x; idx < total; idx += (uint64_t)gridDim.x * B) {
    const uint64_t g = (kMode == 3) ? (uint64_t)a.list[idx] : idx;
    uint64_t k, r;
    child_of(a.log2C, g, k, r);
    if (kMode != 0 && a.pinfo != nullptr) {
      const ParentInfo pi = a.pinfo[k];
      if (pi.fathom || r >= pi.nreg) {
        if (kMode != 3) a.out_flag[g] = kChildNone;
        continue;
      }
    }
    if (pass_through) {
      bool dup = false;
      const uint32_t count = a.pinfo[k].count;
      const SlotPlan* sp = a.slots + k * (uint64_t)a.max_slots;
      for (uint32_t j = 0; j < count; ++j) dup = dup || (slot_part(r, sp[j]) >= sp[j].dom);
      a.out_flag[g] = dup ? kChildDuplicate : kChildScreened;
      continue;
    }
    bool dup;
    const ChildVars<T, S> cv = child_vars<T, S>(a, plo, phi, k, r, olo, ohi, ovid, B, dup);
    if (kMode != 0 && dup) {
      a.out_flag[g] = kChildDuplicate;
      continue;
    }
    const Verdict<T> v = run_interval<T, ChildVars<T, S>, kFused>(a.prog, a.prog_len, cv, t);
    write_verdict<T, kMode>(a, g, k, v, gub);
  }
}

// Lazy form, incremental children, pass 1: for every (segment s, parent
// k), the sum of segment s's chain terms that read none of k's split
// variables, over the parent's FP32 planes.  A warp covers 32 parents of
// one segment, so the instruction stream is the same across the warp and
// the parent planes are read coalesced.
__global__ void __launch_bounds__(kEvalThreads) inc_common_kernel(const EvalArgs a)
{
  if (a.done != nullptr && *a.done) return;
  const uint64_t E = *a.n_parents_dev;
  const uint64_t total = E * (uint64_t)a.inc_segments;
  for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t s = idx / E, k = idx - s * E;
    const ParentInfo pi = a.pinfo[k];
    if (pi.nreg == 0) continue;  // dropped on certification: no children
    const SlotPlan* sp = a.slots + k * (uint64_t)a.max_slots;
    uint64_t mask = 0;
    for (uint32_t j = 0; j < pi.count; ++j) mask |= 1ULL << (sp[j].vid & 63);
    ChildVars<float, float> pv;
    pv.plo = a.plo32 + k;
    pv.phi = a.phi32 + k;
    pv.pstride = a.pstride;
    pv.mask = 0;  // the parent's own bounds for every variable
    pv.count = 0;
    auto is_split = [&](int v) {
      if (!((mask >> (v & 63)) & 1ULL)) return false;
      for (uint32_t j = 0; j < pi.count; ++j)
        if (sp[j].vid == (uint32_t)v) return true;
      return false;
    };
    Iv<float> acc = {0.0f, 0.0f};
    const int b = __ldg(a.inc_seg + 3 * s), t = __ldg(a.inc_seg + 3 * s + 1);
    for (int pc = b; pc < t; ++pc) {
      const Instr cur = load_instr(a.prog, pc);
      const int code = cur.head & 7;
      const bool reads_var = code == kOpTerm || (cur.modes & 3) == kModeVar;
      if (reads_var && (is_split(cur.a) || (code == kOpTerm && is_split(cur.b)))) continue;
      acc = chain_add<float, ChildVars<float, float>>(acc, cur, pv);
    }
    a.inc_common[2 * (s * a.pstride + k)] = acc.lo;
    a.inc_common[2 * (s * a.pstride + k) + 1] = acc.hi;
  }
}

// A parent box's FP32 planes with one variable narrowed to one part of its
// slot (pass 2 of the incremental children).
struct PartVars {
  const float* plo;
  const float* phi;
  uint64_t pstride;
  int vid;
  Iv<float> val;
  __device__ __forceinline__ Iv<float> var(int v) const
  {
    if (v == vid) return val;
    const uint64_t off = (uint64_t)v * pstride;
    return {__ldg(plo + off), __ldg(phi + off)};
  }
};

// Whether variable v is the variable of one of slots 0..j-1.
__device__ __forceinline__ bool slot_var_before(const SlotPlan* sp, int j, int v)
{
  for (int q = 0; q < j; ++q)
    if (sp[q].vid == (uint32_t)v) return true;
  return false;
}

// Lazy form, incremental children, pass 2: for every (slot part u, parent
// k) -- part p of slot j -- and every segment s, the chain sum (from zero,
// in program order) of the segment's terms that read slot j's variable v
// and no variable of an earlier slot, with v over part p of its slot and
// every other variable, split at a later slot or not, over the parent's
// bounds.  A variable that an earlier slot already splits contributes
// nothing here.  Each child then adds, per segment, the part sum of each of
// its slots (eval_children_inc_kernel): a sibling shares each part sum with
// the siblings on the same part of that slot.
__global__ void __launch_bounds__(kEvalThreads) inc_parts_kernel(const EvalArgs a)
{
  if (a.done != nullptr && *a.done) return;
  const uint64_t E = *a.n_parents_dev;
  const uint64_t C = 1ULL << a.log2C;
  const int S = a.inc_segments;
  for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < E * C;
       idx += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t u = idx / E, k = idx - u * E;
    const ParentInfo pi = a.pinfo[k];
    if (pi.fathom || pi.nreg == 0) continue;  // no bounded children
    const SlotPlan* sp = a.slots + k * (uint64_t)a.max_slots;
    int j = -1;
    uint64_t p = 0, base = 0;
    for (uint32_t q = 0; q < pi.count; ++q) {
      const uint64_t w = sp[q].width;
      if (u < base + w) {
        j = (int)q;
        p = u - base;
        break;
      }
      base += w;
    }
    if (j < 0) continue;  // u beyond this parent's parts
    const SlotPlan sj = sp[j];
    const int vj = (int)sj.vid;
    const bool repeated = slot_var_before(sp, j, vj);
    PartVars pv;
    pv.plo = a.plo32 + k;
    pv.phi = a.phi32 + k;
    pv.pstride = a.pstride;
    pv.vid = vj;
    double lo, hi;
    slot_bounds(sj, a.plo[(uint64_t)vj * a.pstride + k], a.phi[(uint64_t)vj * a.pstride + k], p, lo, hi);
    pv.val = {Widen<float, double>::lo(lo), Widen<float, double>::hi(hi)};
    for (int s = 0; s < S; ++s) {
      Iv<float> acc = {0.0f, 0.0f};
      if (!repeated) {
        const int q0 = __ldg(a.inc_off + (uint64_t)vj * S + s), q1 = __ldg(a.inc_off + (uint64_t)vj * S + s + 1);
        for (int q = q0; q < q1; ++q) {
          const Instr cur = load_instr(a.prog, __ldg(a.inc_pcs + q));
          if ((cur.head & 7) == kOpTerm) {
            const int other = cur.a == vj ? cur.b : cur.a;
            if (other != vj && slot_var_before(sp, j, other)) continue;  // that slot's part sum has it
          }
          acc = chain_add<float, PartVars>(acc, cur, pv);
        }
      }
      const uint64_t at = 2 * (((uint64_t)s * C + u) * a.pstride + k);
      a.inc_parts[at] = acc.lo;
      a.inc_parts[at + 1] = acc.hi;
    }
  }
}

// Lazy form, incremental children, pass 3: each child starts every
// segment's chain from its parent's common sum, adds the part sum of each
// of its slots in slot order, then runs the segment's checks and objective.
// One lane per child; shared memory holds the child's split variables (as
// in eval_children, for the checks and the objective) and its slot parts.
__global__ void __launch_bounds__(kEvalThreads, CMN_EVAL_MIN_BLOCKS) eval_children_inc_kernel(const EvalArgs a)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* base = reinterpret_cast<float*>(smem_raw);
  const int B = blockDim.x;
  const int ms = a.max_slots;
  float* olo = base + threadIdx.x;
  float* ohi = olo + (size_t)ms * B;
  int32_t* ovid = reinterpret_cast<int32_t*>(base + (size_t)2 * ms * B) + threadIdx.x;
  uint32_t* opart = reinterpret_cast<uint32_t*>(base + (size_t)3 * ms * B) + threadIdx.x;
  if (a.done != nullptr && *a.done) return;
  const uint64_t total = a.n_children_dev ? *a.n_children_dev : a.n_children;
  const double gub = a.gub ? *a.gub : DBL_MAX;
  const int S = a.inc_segments;
  const uint64_t C = 1ULL << a.log2C;
  for (uint64_t g = (uint64_t)blockIdx.x * B + threadIdx.x; g < total; g += (uint64_t)gridDim.x * B) {
    uint64_t k, r;
    child_of(a.log2C, g, k, r);
    const ParentInfo pi = a.pinfo[k];
    if (pi.fathom || r >= pi.nreg) {
      a.out_flag[g] = kChildNone;
      continue;
    }
    bool dup;
    const ChildVars<float, float> cv = child_vars<float, float>(a, a.plo32, a.phi32, k, r, olo, ohi, ovid, B, dup);
    if (dup) {
      a.out_flag[g] = kChildDuplicate;
      continue;
    }
    {
      const SlotPlan* sp = a.slots + k * (uint64_t)a.max_slots;
      uint64_t pbase = 0;
      for (int j = 0; j < cv.count; ++j) {
        opart[j * B] = (uint32_t)(pbase + slot_part(r, sp[j]));
        pbase += sp[j].width;
      }
    }
    Verdict<float> v = verdict_init<float>();
    for (int s = 0; s < S; ++s) {
      Iv<float> acc = {a.inc_common[2 * ((uint64_t)s * a.pstride + k)],
                       a.inc_common[2 * ((uint64_t)s * a.pstride + k) + 1]};
      for (int j = 0; j < cv.count; ++j) {
        const uint64_t at = 2 * (((uint64_t)s * C + opart[j * B]) * a.pstride + k);
        acc = iv_add(acc, Iv<float>{a.inc_parts[at], a.inc_parts[at + 1]});
      }
      chain_tail<float, ChildVars<float, float>>(a.prog, __ldg(a.inc_seg + 3 * s + 1), __ldg(a.inc_seg + 3 * s + 2),
                                                 cv, acc, v);
    }
    write_verdict<float, 5>(a, g, k, v, gub);
  }
}

template <typename T, int kMode, bool kFused = false>
__global__ void __launch_bounds__(kEvalThreads, CMN_EVAL_MIN_BLOCKS) eval_children_kernel(const EvalArgs a)
{
  if constexpr (sizeof(T) == 4) {
    if (a.plo32 != nullptr) {
      eval_children<T, kMode, float>(a, a.plo32, a.phi32);
      return;
    }
  }
  eval_children<T, kMode, double, false, kFused>(a, a.plo, a.phi);
}

// The FP64 one-lane passes with their program staged in shared memory
// (kMode 0 and 1; EvalArgs::stage_at set by the launcher).
template <int kMode, bool kFused = false>
__global__ void __launch_bounds__(kEvalThreads, CMN_EVAL_MIN_BLOCKS) eval_children_staged_kernel(const EvalArgs a)
{
  eval_children<double, kMode, double, true, kFused>(a, a.plo, a.phi);
}

__device__ __forceinline__ void warp_min_cand(Cand& c)
{
  for (int off = 16; off > 0; off >>= 1) {
    Cand o;
    o.value = __shfl_down_sync(0xffffffffu, c.value, off);
    o.k = __shfl_down_sync(0xffffffffu, c.k, off);
    o.e = __shfl_down_sync(0xffffffffu, c.e, off);
    o.pad = 0;
    if (cand_less(o, c)) c = o;
  }
}

// Block-wide min of one Cand per thread; result valid in thread 0.
__device__ __forceinline__ Cand block_min_cand(Cand c)
{
  __shared__ Cand warp_best[32];
  warp_min_cand(c);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) warp_best[wid] = c;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  if (wid == 0) {
    Cand x = lane < nw ? warp_best[lane] : Cand{INFINITY, 0xffffffffu, 0, ~0ULL};
    warp_min_cand(x);
    c = x;
  }
  __syncthreads();
  return c;
}

__device__ __forceinline__ bool admissible(const SampleArgs& a, const Tile<double>& t)
{
  for (int v = 0; v < a.n_vars; ++v) {
    const double x = t.lo[v * t.stride + t.tid];
    if (!(x >= a.root_lb[v]) || !(x <= a.root_ub[v])) return false;
    if (a.var_kinds[v] != 0) {
      const double nearest = rint(x);
      if (fabs(__dsub_rn(x, nearest)) > 1e-6) return false;
    }
  }
  return true;
}

// The point of sample i of child (k, r), staged in this thread's column:
// every variable from its region bound (the parent's, narrowed by its slot).
__device__ __forceinline__ void stage_point(const SampleArgs& a, const Tile<double>& t, uint64_t k, uint64_t r,
                                            uint64_t i, uint64_t salt, bool fathom)
{
  const SlotPlan* sp = a.pinfo ? a.slots + k * (uint64_t)a.max_slots : nullptr;
  const uint32_t count = a.pinfo ? a.pinfo[k].count : 0;
  for (int v = 0; v < a.n_vars; ++v) {
    double lo = a.plo[(uint64_t)v * a.pstride + k];
    double hi = a.phi[(uint64_t)v * a.pstride + k];
    for (uint32_t j = 0; j < count; ++j) {
      if (sp[j].vid == (uint32_t)v) {
        const uint64_t part = slot_part(r, sp[j]);
        slot_bounds(sp[j], lo, hi, part, lo, hi);
        break;
      }
    }
    t.lo[v * t.stride + t.tid] = fathom ? lo : sample_value(a.var_kinds[v] != 0, lo, hi, (uint64_t)v, i, r, salt);
  }
}

// The chunk of children [32c, 32c + 32) of the lazy form: the child and
// sample with the smallest FP32 value (ties: the first child, then the
// first sample).  Returns false when no point of the chunk is feasible in
// FP32.
__device__ __forceinline__ bool chunk_pick(const Best32* __restrict__ cbest, uint64_t c, uint64_t total, uint64_t& g,
                                           uint64_t& i)
{
  float best = INFINITY;
  const uint64_t g0 = c << kChunkLog2;
  const uint64_t g1 = total < g0 + (1ULL << kChunkLog2) ? total : g0 + (1ULL << kChunkLog2);
  for (uint64_t x = g0; x < g1; ++x) {
    const Best32 b = cbest[x];
    if (b.value < best) {
      best = b.value;
      g = x;
      i = b.i;
    }
  }
  return best < INFINITY;
}

// Variables v = lane, lane + G, ... of the point of sample i of child
// (k, r), written into the group's column t.tid (see stage_point).
__device__ __forceinline__ void stage_point_part(const SampleArgs& a, const Tile<double>& t, uint64_t k, uint64_t r,
                                                 uint64_t i, uint64_t salt, bool fathom, int lane, int G)
{
  const SlotPlan* sp = a.pinfo ? a.slots + k * (uint64_t)a.max_slots : nullptr;
  const uint32_t count = a.pinfo ? a.pinfo[k].count : 0;
  for (int v = lane; v < a.n_vars; v += G) {
    double lo = a.plo[(uint64_t)v * a.pstride + k];
    double hi = a.phi[(uint64_t)v * a.pstride + k];
    for (uint32_t j = 0; j < count; ++j) {
      if (sp[j].vid == (uint32_t)v) {
        slot_bounds(sp[j], lo, hi, slot_part(r, sp[j]), lo, hi);
        break;
      }
    }
    t.lo[v * t.stride + t.tid] = fathom ? lo : sample_value(a.var_kinds[v] != 0, lo, hi, (uint64_t)v, i, r, salt);
  }
}

// Sampling with groups of 2^lg lanes per point (see eval_children_grouped):
// the G lanes of a group stage the point together into one shared-memory
// column (lane j writes variables j, j + G, ...), each runs its segments of
// the point program, and lane 0 of the group scores the combined result.
// A block holds blockDim.x >> lg_min columns, so a large point costs
// 8 * n_vars / G bytes per thread.  An item is a child (all its samples), or
// in the lazy form's chunk mode a chunk (the one point chunk_pick chose).
// The loop bound is per block, so every lane of a warp reaches the
// shuffles and warp barriers.
__device__ void sample_children_grouped(const SampleArgs& a, Tile<double> t, uint64_t total, uint64_t salt_base,
                                        double gub, int lg, Cand& best, unsigned long long& rejected)
{
  const int B = blockDim.x;
  const int G = 1 << lg;
  const int lane = threadIdx.x & (G - 1);
  t.tid = (int)((threadIdx.x & ~(unsigned)(G - 1)) >> a.lg_min);  // the group's column
  const bool chunked = a.cbest != nullptr;
  const uint64_t items = chunked ? (total + (1ULL << kChunkLog2) - 1) >> kChunkLog2 : total;
  const uint64_t per_block = (uint64_t)(B >> lg);
  const uint64_t S_loop = (a.exact || chunked) ? 1 : a.S;
  for (uint64_t base = (uint64_t)blockIdx.x * per_block; base < items; base += (uint64_t)gridDim.x * per_block) {
    const uint64_t item = base + (threadIdx.x >> lg);
    bool live = item < items;
    uint64_t g = item, i0 = 0, k = 0, r = 0;
    bool fathom = a.exact != 0;
    if (live && chunked) live = chunk_pick(a.cbest, item, total, g, i0);
    if (live) {
      child_of(a.log2C, g, k, r);
      uint64_t nreg = ~0ULL;
      if (a.pinfo != nullptr) {
        const ParentInfo pi = a.pinfo[k];
        nreg = pi.nreg;
        fathom = fathom || pi.fathom;
      }
      if (r >= nreg) live = false;
      if (live && !chunked && a.state != nullptr && !fathom) {
        const uint8_t st = a.state[g];
        live = a.sample_all ? (st != kChildNone) : (st == kChildEligible);
      }
    }
    const uint64_t salt = a.salt_base_dev ? salt_base + k + 1 : a.salt;
    const uint64_t S = fathom ? 1 : a.S;
    for (uint64_t j = 0; j < S_loop; ++j) {
      const uint64_t i = chunked ? i0 : j;
      const bool act = live && (chunked || j < S);
      if (act) stage_point_part(a, t, k, r, i, salt, fathom, lane, G);
      __syncwarp();
      PointVerdict pv;
      pv.obj = INFINITY;
      pv.feasible = true;
      pv.has_obj = false;
      if (act) pv = run_point_lane(a.prog, a.sched, lg, lane, t);
      pv = group_point_verdict(pv, G);
      if (act && lane == 0) {
        double value = (pv.feasible && !(pv.obj != pv.obj)) ? pv.obj : INFINITY;
        if (fathom && a.state != nullptr && value < INFINITY && !admissible(a, t)) {
          if (value < gub) ++rejected;
          value = INFINITY;
        }
        const Cand c = {value, (uint32_t)k, 0, r * S + i};
        if (value < INFINITY && cand_less(c, best)) best = c;
      }
      __syncwarp();  // the column is restaged next
    }
  }
}

// Point sampling (graph/subregion_sampler.cuh:133-199) and exact points
// (graph/kernels.cuh:131-172), point program, feasibility mask and the
// ArgMin over (value, parent, element) -- element = region * S + sample.
__global__ void __launch_bounds__(kEvalThreads) sample_children_kernel(const SampleArgs a)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* base = reinterpret_cast<double*>(smem_raw);
  const int B = blockDim.x;
  // one point column per 2^lg_min threads (slots follow the variables)
  const int cols = B >> a.lg_min;
  Tile<double> t;
  t.lo = base;
  t.hi = base;  // unused by the point program
  t.slo = base + (size_t)a.n_vars * cols;
  t.shi = t.slo;
  t.stride = cols;
  t.tid = threadIdx.x;

  if (a.done != nullptr && *a.done) {
    if (threadIdx.x == 0) a.block_best[blockIdx.x] = Cand{INFINITY, 0xffffffffu, 0, ~0ULL};
    return;
  }
  const uint64_t total = a.n_children_dev ? *a.n_children_dev : a.n_children;
  const uint64_t salt_base = a.salt_base_dev ? *a.salt_base_dev : 0;
  const double gub = a.gub ? *a.gub : DBL_MAX;
  Cand best = {INFINITY, 0xffffffffu, 0, ~0ULL};
  unsigned long long rejected = 0;

  const uint64_t chunks = (total + (1ULL << kChunkLog2) - 1) >> kChunkLog2;
  int lg = a.sched != nullptr ? lanes_per_box(a.cbest != nullptr ? chunks : total, a.capacity, a.g_max) : 0;
  if (lg < a.lg_min) lg = a.lg_min;
  if (lg > 0) sample_children_grouped(a, t, total, salt_base, gub, lg, best, rejected);
  if (lg == 0 && a.cbest != nullptr) {
    // lazy form: each chunk's FP32-best point, evaluated in FP64
    for (uint64_t c = (uint64_t)blockIdx.x * B + threadIdx.x; c < chunks; c += (uint64_t)gridDim.x * B) {
      uint64_t g = 0, i = 0;
      if (!chunk_pick(a.cbest, c, total, g, i)) continue;
      uint64_t k, r;
      child_of(a.log2C, g, k, r);
      bool fathom = a.exact != 0;
      if (a.pinfo != nullptr) fathom = fathom || a.pinfo[k].fathom;
      const uint64_t salt = a.salt_base_dev ? salt_base + k + 1 : a.salt;
      stage_point(a, t, k, r, i, salt, fathom);
      const PointVerdict pv = run_point_ordered(a.prog, a.prog_len, a.sched, t);
      double value = (pv.feasible && !(pv.obj != pv.obj)) ? pv.obj : INFINITY;
      if (fathom && a.state != nullptr && value < INFINITY && !admissible(a, t)) {
        if (value < gub) ++rejected;
        value = INFINITY;
      }
      const uint64_t S = fathom ? 1 : a.S;
      const Cand cand = {value, (uint32_t)k, 0, r * S + i};
      if (value < INFINITY && cand_less(cand, best)) best = cand;
    }
  }
  for (uint64_t g = (uint64_t)blockIdx.x * B + threadIdx.x; a.cbest == nullptr && lg == 0 && g < total;
       g += (uint64_t)gridDim.x * B) {
    uint64_t k, r;
    child_of(a.log2C, g, k, r);
    bool fathom = a.exact != 0;
    uint64_t nreg = ~0ULL;
    if (a.pinfo != nullptr) {
      const ParentInfo pi = a.pinfo[k];
      nreg = pi.nreg;
      fathom = fathom || pi.fathom;
    }
    if (r >= nreg) continue;
    if (a.state != nullptr && !fathom) {
      const uint8_t st = a.state[g];
      const bool take = a.sample_all ? (st != kChildNone) : (st == kChildEligible);
      if (!take) continue;
    }
    // child bounds per variable: parent bound, narrowed by its slot
    const SlotPlan* sp = a.pinfo ? a.slots + k * (uint64_t)a.max_slots : nullptr;
    const uint32_t count = a.pinfo ? a.pinfo[k].count : 0;
    const uint64_t salt = a.salt_base_dev ? salt_base + k + 1 : a.salt;
    const uint64_t S = fathom ? 1 : a.S;
    for (uint64_t i = 0; i < S; ++i) {
      // stage the point in the tile: every variable from its region bound
      for (int v = 0; v < a.n_vars; ++v) {
        double lo = a.plo[(uint64_t)v * a.pstride + k];
        double hi = a.phi[(uint64_t)v * a.pstride + k];
        for (uint32_t j = 0; j < count; ++j) {
          if (sp[j].vid == (uint32_t)v) {
            const uint64_t part = slot_part(r, sp[j]);
            slot_bounds(sp[j], lo, hi, part, lo, hi);
            break;
          }
        }
        t.lo[v * B + t.tid] =
            fathom ? lo : sample_value(a.var_kinds[v] != 0, lo, hi, (uint64_t)v, i, r, salt);
      }
      const PointVerdict pv = run_point_ordered(a.prog, a.prog_len, a.sched, t);
      double value = (pv.feasible && !(pv.obj != pv.obj)) ? pv.obj : INFINITY;
      if (fathom && a.state != nullptr && value < INFINITY && !admissible(a, t)) {
        if (value < gub) ++rejected;
        value = INFINITY;
      }
      const Cand c = {value, (uint32_t)k, 0, r * S + i};
      if (value < INFINITY && cand_less(c, best)) best = c;
    }
  }
  best = block_min_cand(best);
  if (threadIdx.x == 0) a.block_best[blockIdx.x] = best;
  if (a.rejected != nullptr) {
    for (int off = 16; off > 0; off >>= 1) rejected += __shfl_down_sync(0xffffffffu, rejected, off);
    if ((threadIdx.x & 31) == 0 && rejected) atomicAdd(a.rejected, rejected);
  }
}

// The lazy form's sample screen: every sampled child's S points (or its
// exact point) in FP32, keeping per child the smallest FP32 value and its
// sample index in cbest[g].  Children not sampled get +inf.  Groups of
// 2^lg_min lanes share a child and one shared-memory point column (lane j
// stages variables j, j + G, ... and runs its segments of the lane
// schedule), so a point of n variables costs 4n/G bytes per thread; with
// lg_min = 0 a lane evaluates its child alone.  The loop bound is per
// block, so every lane of a warp reaches the shuffles and barriers.
__global__ void __launch_bounds__(kEvalThreads) sample_screen_kernel(const SampleArgs a)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* base = reinterpret_cast<float*>(smem_raw);
  const int B = blockDim.x;
  const int lg = a.lg_min;
  const int G = 1 << lg;
  const int lane = threadIdx.x & (G - 1);
  const int cols = B >> lg;
  Tile<float> t;
  t.lo = base;
  t.hi = base;
  t.slo = base + (size_t)a.n_vars * cols;
  t.shi = t.slo;
  t.stride = cols;
  t.tid = threadIdx.x >> lg;
  if (a.done != nullptr && *a.done) return;
  const uint64_t total = a.n_children_dev ? *a.n_children_dev : a.n_children;
  const uint64_t salt_base = a.salt_base_dev ? *a.salt_base_dev : 0;
  const uint64_t per_block = (uint64_t)cols;
  const uint64_t S_loop = a.exact ? 1 : a.S;
  int32_t p0 = 0, p1 = a.prog_len;  // this lane's segments (lg > 0: the lane schedule)
  LaneSegs ls = {nullptr, 0, 0};
  if (lg > 0) ls = lane_segments(a.sched, lg, lane);
  for (uint64_t bb = (uint64_t)blockIdx.x * per_block; bb < total; bb += (uint64_t)gridDim.x * per_block) {
    const uint64_t g = bb + (threadIdx.x >> lg);
    Best32 best = {INFINITY, 0};
    bool live = g < total;
    uint64_t k = 0, r = 0;
    bool fathom = a.exact != 0;
    if (live) {
      child_of(a.log2C, g, k, r);
      uint64_t nreg = ~0ULL;
      if (a.pinfo != nullptr) {
        const ParentInfo pi = a.pinfo[k];
        nreg = pi.nreg;
        fathom = fathom || pi.fathom;
      }
      live = r < nreg;
      if (live && a.state != nullptr && !fathom) {
        const uint8_t st = a.state[g];
        live = a.sample_all ? (st != kChildNone) : (st == kChildEligible);
      }
    }
    const SlotPlan* sp = a.pinfo ? a.slots + k * (uint64_t)a.max_slots : nullptr;
    const uint32_t count = (live && a.pinfo) ? a.pinfo[k].count : 0;
    const uint64_t salt = a.salt_base_dev ? salt_base + k + 1 : a.salt;
    const uint64_t S = fathom ? 1 : a.S;
    for (uint64_t i = 0; i < S_loop; ++i) {
      const bool act = live && i < S;
      if (act) {
        for (int v = lane; v < a.n_vars; v += G) {
          double lo = a.plo[(uint64_t)v * a.pstride + k];
          double hi = a.phi[(uint64_t)v * a.pstride + k];
          for (uint32_t j = 0; j < count; ++j) {
            if (sp[j].vid == (uint32_t)v) {
              slot_bounds(sp[j], lo, hi, slot_part(r, sp[j]), lo, hi);
              break;
            }
          }
          const double x = fathom ? lo : sample_value(a.var_kinds[v] != 0, lo, hi, (uint64_t)v, i, r, salt);
          t.lo[v * cols + t.tid] = __double2float_rn(x);
        }
      }
      __syncwarp();
      PointVerdict32 pv;
      pv.obj = INFINITY;
      pv.feasible = true;
      pv.has_obj = false;
      if (act) {
        if (lg == 0 && a.sched != nullptr) {
          // level 0 of the lane schedule: the objective's segments last
          const LaneSegs l0 = lane_segments(a.sched, 0, 0);
          for (int j = l0.b; j < l0.e && pv.feasible; ++j)
            point_range32(a.prog, __ldg(l0.pairs + 2 * j), __ldg(l0.pairs + 2 * j + 1), t, pv);
        } else if (lg == 0) {
          point_range32(a.prog, p0, p1, t, pv);
        } else {
          for (int j = ls.b; j < ls.e && pv.feasible; ++j)
            point_range32(a.prog, __ldg(ls.pairs + 2 * j), __ldg(ls.pairs + 2 * j + 1), t, pv);
        }
      }
      for (int off = 1; off < G; off <<= 1) {  // the group's verdict
        const int f = __shfl_xor_sync(0xffffffffu, (int)pv.feasible, off);
        const int h = __shfl_xor_sync(0xffffffffu, (int)pv.has_obj, off);
        const float o = __shfl_xor_sync(0xffffffffu, pv.obj, off);
        pv.feasible = pv.feasible && f;
        if (!pv.has_obj && h) {
          pv.obj = o;
          pv.has_obj = true;
        }
      }
      const float value = (pv.feasible && !(pv.obj != pv.obj)) ? pv.obj : INFINITY;
      if (act && value < best.value) best = Best32{value, (uint32_t)i};
      __syncwarp();  // the column is restaged next
    }
    if (g < total && lane == 0) a.cbest[g] = best;
  }
}

// Final ArgMin over the per-block candidates (one block).
__global__ void reduce_cand_kernel(const Cand* __restrict__ block_best, int n, Cand* __restrict__ out)
{
  Cand best = {INFINITY, 0xffffffffu, 0, ~0ULL};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const Cand c = block_best[i];
    if (cand_less(c, best)) best = c;
  }
  best = block_min_cand(best);
  if (threadIdx.x == 0) *out = best;
}

// Witness of a candidate: the point the sampler (or the exact grid) drew
// for (parent k, element e).  One thread per variable.
__global__ void witness_kernel(const Cand* __restrict__ cand, const double* __restrict__ plo,
                               const double* __restrict__ phi, uint64_t pstride, const ParentInfo* __restrict__ pinfo,
                               const SlotPlan* __restrict__ slots, int max_slots, const int32_t* __restrict__ kinds,
                               int n_vars, uint64_t S, uint64_t salt, const uint64_t* __restrict__ salt_base_dev,
                               int exact, const uint32_t* __restrict__ write_flag, double* __restrict__ out)
{
  if (write_flag != nullptr && *write_flag == 0) return;
  const Cand c = *cand;
  const bool found = c.value < DBL_MAX;
  const uint64_t k = c.k;
  bool fathom = exact != 0;
  if (pinfo && found) fathom = fathom || pinfo[k].fathom;
  const uint64_t SS = fathom ? 1 : S;
  const uint64_t r = found ? c.e / SS : 0, i = found ? c.e % SS : 0;
  const uint64_t sl = salt_base_dev ? *salt_base_dev + k + 1 : salt;
  for (int v = threadIdx.x + blockIdx.x * blockDim.x; v < n_vars; v += blockDim.x * gridDim.x) {
    if (!found) {
      out[v] = __longlong_as_double(0x7ff8000000000000LL);
      continue;
    }
    double lo = plo[(uint64_t)v * pstride + k];
    double hi = phi[(uint64_t)v * pstride + k];
    if (pinfo) {
      const SlotPlan* sp = slots + k * (uint64_t)max_slots;
      const uint32_t count = pinfo[k].count;
      for (uint32_t j = 0; j < count; ++j) {
        if (sp[j].vid == (uint32_t)v) {
          const uint64_t part = slot_part(r, sp[j]);
          slot_bounds(sp[j], lo, hi, part, lo, hi);
          break;
        }
      }
    }
    out[v] = fathom ? lo : sample_value(kinds[v] != 0, lo, hi, (uint64_t)v, i, r, sl);
  }
}

// FMA throughput probe: 8 independent FMA chains per thread.
template <typename T>
__global__ void fma_peak_kernel(int iters, T* sink)
{
  T a0 = T(threadIdx.x) * T(1e-7), a1 = a0 + T(1), a2 = a0 + T(2), a3 = a0 + T(3);
  T a4 = a0 + T(4), a5 = a0 + T(5), a6 = a0 + T(6), a7 = a0 + T(7);
  const T m = T(0.999999), c = T(1e-9);
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, m, c);
    a1 = fma(a1, m, c);
    a2 = fma(a2, m, c);
    a3 = fma(a3, m, c);
    a4 = fma(a4, m, c);
    a5 = fma(a5, m, c);
    a6 = fma(a6, m, c);
    a7 = fma(a7, m, c);
  }
  sink[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

cudaError_t launch_fma_peak(int precision, int grid, int threads, int iters, void* sink, cudaStream_t s)
{
  if (precision == 0) fma_peak_kernel<double><<<grid, threads, 0, s>>>(iters, static_cast<double*>(sink));
  else fma_peak_kernel<float><<<grid, threads, 0, s>>>(iters, static_cast<float*>(sink));
  return cudaGetLastError();
}

// ---------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------

size_t sample_smem_bytes(int n_vars, int n_slots, int threads, int lg_min)
{
  return 8 * (size_t)(n_vars + n_slots) * (size_t)(threads >> lg_min);
}

int sample_lg_min(int n_vars, int n_slots, bool has_sched, int threads)
{
  if (!has_sched) return 0;  // shared slots: one column per thread
  int lg = 0;
  while (lg < 5 && sample_smem_bytes(n_vars, n_slots, threads, lg) > kSampleColumnBytes) ++lg;
  return lg;
}

// Kernel attributes are set once per device, before any launch, so that
// launches stay legal inside stream capture.
// The dynamic allowance is the opt-in maximum less the kernel's own static
// shared memory (the reduction scratch of the sampler).
template <typename K>
static cudaError_t allow_dynamic_smem(K kernel, int max_smem)
{
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              max_smem - (int)fa.sharedSizeBytes);
}

cudaError_t set_eval_kernel_attributes(int max_smem)
{
  cudaError_t e = allow_dynamic_smem(eval_children_kernel<double, 0>, max_smem);
  if (e == cudaSuccess) e = allow_dynamic_smem(eval_children_staged_kernel<0>, max_smem);
  if (e == cudaSuccess) e = allow_dynamic_smem(eval_children_staged_kernel<1>, max_smem);
  if (e == cudaSuccess) e = allow_dynamic_smem(eval_children_staged_kernel<0, true>, max_smem);
  if (e == cudaSuccess) e = allow_dynamic_smem(eval_children_kernel<double, 0, true>, max_smem);
  if (e == cudaSuccess) e = allow_dynamic_smem(eval_children_kernel<double, 1>, max_smem);
  if (e == cudaSuccess) e = allow_dynamic_smem(eval_children_kernel<double, 3>, max_smem);
  if (e == cudaSuccess) e = allow_dynamic_smem(eval_children_kernel<double, 4>, max_smem);
  if (e == cudaSuccess) e = allow_dynamic_smem(eval_children_kernel<float, 0>, max_smem);
  if (e == cudaSuccess) e = allow_dynamic_smem(eval_children_kernel<float, 2>, max_smem);
  if (e == cudaSuccess) e = allow_dynamic_smem(eval_children_kernel<float, 5>, max_smem);
  if (e == cudaSuccess) e = allow_dynamic_smem(sample_children_kernel, max_smem);
  if (e == cudaSuccess) e = allow_dynamic_smem(sample_screen_kernel, max_smem);
  return e;
}

int eval_kernel_occupancy(int mode, bool fp32, size_t smem, int threads)
{
  int blocks = 0;
  cudaError_t e;
  if (fp32) {
    e = mode == 0   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, eval_children_kernel<float, 0>, threads, smem)
        : mode == 5 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, eval_children_kernel<float, 5>, threads, smem)
                    : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, eval_children_kernel<float, 2>, threads, smem);
  } else {
    e = mode == 0 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, eval_children_kernel<double, 0>, threads, smem)
        : mode == 1
            ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, eval_children_kernel<double, 1>, threads, smem)
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, eval_children_kernel<double, 3>, threads, smem);
  }
  return e == cudaSuccess ? blocks : 1;
}

int sample_kernel_occupancy(size_t smem, int threads)
{
  int blocks = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, sample_children_kernel, threads, smem);
  return e == cudaSuccess ? blocks : 1;
}

template <typename T, int kMode, bool kFused = false>
static cudaError_t launch_eval_t(const EvalArgs& a, int grid, int threads, cudaStream_t s)
{
  size_t smem = eval_smem_bytes(a.n_slots, a.pinfo != nullptr ? a.max_slots : 0, sizeof(T) == 4, threads);
  EvalArgs b = a;
  b.stage_at = 0;
  if (CMN_STAGE_PROGRAM && sizeof(T) == 8 && (kMode == 0 || kMode == 1)) {
    // staged program tiles after the block's layout, when they still fit
    const size_t at = (smem + 127) & ~(size_t)127;
    if (at + kStageBytes <= (size_t)max_dynamic_smem()) {
      b.stage_at = at > 0 ? at : 128;
      smem = b.stage_at + kStageBytes;
    }
  }
  if constexpr (sizeof(T) == 8 && (kMode == 0 || kMode == 1)) {
    if (b.stage_at != 0) {
      eval_children_staged_kernel<kMode, kFused><<<grid, threads, smem, s>>>(b);
      return cudaGetLastError();
    }
  }
  eval_children_kernel<T, kMode, kFused><<<grid, threads, smem, s>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_inc(const EvalArgs& a, int grid, int threads, cudaStream_t s)
{
  inc_common_kernel<<<grid, threads, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  inc_parts_kernel<<<grid, threads, 0, s>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  eval_children_inc_kernel<<<grid, threads, inc_child_smem_bytes(a.max_slots, threads), s>>>(a);
  return cudaGetLastError();
}

size_t inc_child_smem_bytes(int max_slots, int threads)
{
  return (size_t)(8 + 4 + 4) * (size_t)max_slots * (size_t)threads;
}

cudaError_t launch_eval(const EvalArgs& a, int mode, bool fp32, int grid, int threads, cudaStream_t s)
{
  if (fp32) {
    if (mode == 0) return launch_eval_t<float, 0>(a, grid, threads, s);
    if (mode == 5) return launch_eval_t<float, 5>(a, grid, threads, s);
    return launch_eval_t<float, 2>(a, grid, threads, s);
  }
  if (mode == 0) return launch_eval_t<double, 0>(a, grid, threads, s);
  if (mode == 6) return launch_eval_t<double, 0, true>(a, grid, threads, s);
  if (mode == 1) return launch_eval_t<double, 1>(a, grid, threads, s);
  if (mode == 4) return launch_eval_t<double, 4>(a, grid, threads, s);
  return launch_eval_t<double, 3>(a, grid, threads, s);
}

size_t sample_screen_smem_bytes(int n_vars, int n_slots, int threads, int lg_min)
{
  return 4 * (size_t)(n_vars + n_slots) * (size_t)(threads >> lg_min);
}

int sample_screen_lg_min(int n_vars, int n_slots, bool has_sched, int threads)
{
  if (!has_sched) return 0;
  int lg = 0;
  while (lg < 5 && sample_screen_smem_bytes(n_vars, n_slots, threads, lg) > kSampleColumnBytes) ++lg;
  return lg;
}

cudaError_t launch_sample_screen(const SampleArgs& a, int grid, int threads, cudaStream_t s)
{
  sample_screen_kernel<<<grid, threads, sample_screen_smem_bytes(a.n_vars, a.n_slots, threads, a.lg_min), s>>>(a);
  return cudaGetLastError();
}

int sample_screen_occupancy(size_t smem, int threads)
{
  int blocks = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, sample_screen_kernel, threads, smem);
  return e == cudaSuccess ? blocks : 1;
}

cudaError_t launch_sample(const SampleArgs& a, int grid, int threads, cudaStream_t s)
{
  const size_t smem = sample_smem_bytes(a.n_vars, a.n_slots, threads, a.lg_min);
  sample_children_kernel<<<grid, threads, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_reduce_cand(const Cand* block_best, int n, Cand* out, cudaStream_t s)
{
  reduce_cand_kernel<<<1, 1024, 0, s>>>(block_best, n, out);
  return cudaGetLastError();
}

cudaError_t launch_witness(const Cand* cand, const double* plo, const double* phi, uint64_t pstride,
                           const ParentInfo* pinfo, const SlotPlan* slots, int max_slots, const int32_t* kinds,
                           int n_vars, uint64_t S, uint64_t salt, const uint64_t* salt_base_dev, int exact,
                           const uint32_t* write_flag, double* out, cudaStream_t s)
{
  const int threads = 128;
  const int grid = (n_vars + threads - 1) / threads;
  witness_kernel<<<grid, threads, 0, s>>>(cand, plo, phi, pstride, pinfo, slots, max_slots, kinds, n_vars, S, salt,
                                          salt_base_dev, exact, write_flag, out);
  return cudaGetLastError();
}

}  // namespace cmn
