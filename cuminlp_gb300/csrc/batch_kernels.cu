// batch_kernels.cu -- the multi-instance iteration (see batch.hpp).
//
// Per iteration: begin (thread per instance) -> select + gather + in-place
// compaction (block per instance, pool sorted in shared memory) -> branch
// (thread per parent) -> bound (one launch over all instances' children;
// FP64, or FP32 screen + FP64 certify) -> sample (one launch) -> finish
// (block per instance: ArgMin, incumbent and witness, prune, append kept
// children, evict above the cap, pool minimum, adaptive screen).
#include <algorithm>
#include <cfloat>
#include <cstdint>

#include "batch.hpp"
#include "eval_core.cuh"
#include "launch.hpp"
#include "policy.cuh"

namespace cmn {

namespace {

constexpr uint8_t kCertifiedBit = 0x80;  // set by the FP64 certify pass
constexpr int kMaxPerThread = kMiSortMax / kMiThreads;

__device__ __forceinline__ bool gap_closed_b(double gub, double bound, double tol)
{
  return __dsub_rn(gub, bound) <= __dmul_rn(tol, fmax(1.0, fabs(gub)));
}

__device__ __forceinline__ double key_to_lb_b(uint64_t k)
{
  const uint64_t u = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
  return __longlong_as_double((long long)u);
}

__device__ __forceinline__ uint64_t next_pow2(uint64_t x)
{
  uint64_t p = 1;
  while (p < x) p <<= 1;
  return p;
}

// exclusive rank of `f` among the block's threads (1024 threads)
__device__ __forceinline__ int block_rank(bool f, int& total)
{
  __shared__ int warp_tot[kMiThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned ball = __ballot_sync(0xffffffffu, f);
  if (lane == 0) warp_tot[wid] = __popc(ball);
  __syncthreads();
  int before = 0;
  total = 0;
  for (int w = 0; w < kMiThreads / 32; ++w) {
    if (w < wid) before += warp_tot[w];
    total += warp_tot[w];
  }
  __syncthreads();
  return before + __popc(ball & ((1u << lane) - 1u));
}

// ascending bitonic sort of (key, pos) pairs, n a power of two
__device__ void bitonic_sort(uint64_t* keys, uint32_t* pos, uint32_t n)
{
  for (uint32_t k = 2; k <= n; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t ixj = i ^ j;
        if (ixj > i) {
          const bool asc = (i & k) == 0;
          const uint64_t ka = keys[i], kb = keys[ixj];
          const uint32_t pa = pos[i], pb = pos[ixj];
          const bool b_less = kb < ka || (kb == ka && pb < pa);
          if (asc ? b_less : !b_less) {
            keys[i] = kb;
            keys[ixj] = ka;
            pos[i] = pb;
            pos[ixj] = pa;
          }
        }
      }
      __syncthreads();
    }
  }
}

__device__ __forceinline__ size_t plane(const BatchCfg& c, uint64_t slot, int v)
{
  return ((size_t)slot * c.n_max + v) * c.P;
}

__device__ __forceinline__ size_t splane(const BatchCfg& c, uint64_t slot, int v)
{
  return ((size_t)slot * c.n_max + v) * c.e_max;
}

// Stable in-place compaction of the marked entries among the first `n` of
// `slot`'s pool (marks in `keep`, new positions built in `newpos`).
__device__ void compact_pool(const BatchCfg& c, const BatchBufs& b, uint64_t slot, uint32_t n, int n_vars,
                             const uint8_t* keep, uint32_t* newpos, uint32_t* running)
{
  if (threadIdx.x == 0) *running = 0;
  __syncthreads();
  for (uint32_t base = 0; base < n; base += kMiThreads) {
    const uint32_t i = base + threadIdx.x;
    const bool f = i < n && keep[i];
    int total;
    const int r = block_rank(f, total);
    if (f) newpos[i] = *running + (uint32_t)r;
    __syncthreads();
    if (threadIdx.x == 0) *running += (uint32_t)total;
    __syncthreads();
  }
  double val[kMaxPerThread];
  for (int v = -1; v < 2 * n_vars; ++v) {
    // v = -1: lower bounds; then lo / hi planes
    double* arr = v < 0 ? b.lb + (size_t)slot * c.P : (v & 1 ? b.hi : b.lo) + plane(c, slot, v >> 1);
#pragma unroll
    for (int j = 0; j < kMaxPerThread; ++j) {
      const uint32_t i = threadIdx.x + j * kMiThreads;
      if (i < n && keep[i]) val[j] = arr[i];
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kMaxPerThread; ++j) {
      const uint32_t i = threadIdx.x + j * kMiThreads;
      if (i < n && keep[i]) arr[newpos[i]] = val[j];
    }
    __syncthreads();
  }
  uint32_t dv[kMaxPerThread];
  uint32_t* dep = b.depth + (size_t)slot * c.P;
#pragma unroll
  for (int j = 0; j < kMaxPerThread; ++j) {
    const uint32_t i = threadIdx.x + j * kMiThreads;
    if (i < n && keep[i]) dv[j] = dep[i];
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kMaxPerThread; ++j) {
    const uint32_t i = threadIdx.x + j * kMiThreads;
    if (i < n && keep[i]) dep[newpos[i]] = dv[j];
  }
  __syncthreads();
}

struct SortSmem {
  uint64_t* keys;
  uint32_t* pos;
  uint8_t* flag;
};

__device__ __forceinline__ SortSmem sort_smem(unsigned char* raw)
{
  SortSmem s;
  s.keys = reinterpret_cast<uint64_t*>(raw);
  s.pos = reinterpret_cast<uint32_t*>(s.keys + kMiSortMax);
  s.flag = reinterpret_cast<uint8_t*>(s.pos + kMiSortMax);
  return s;
}

// Marks the `k` smallest (key, position) entries among the first `n`.
__device__ void mark_smallest(const double* lb, uint32_t n, uint32_t k, const SortSmem& s)
{
  if (k >= n) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) s.flag[i] = 1;
    __syncthreads();
    return;
  }
  const uint32_t n2 = (uint32_t)next_pow2(n);
  for (uint32_t i = threadIdx.x; i < n2; i += blockDim.x) {
    s.keys[i] = i < n ? lb_key(lb[i]) : ~0ULL;
    s.pos[i] = i < n ? i : 0xffffffffu;
    if (i < n) s.flag[i] = 0;
  }
  __syncthreads();
  bitonic_sort(s.keys, s.pos, n2);
  for (uint32_t i = threadIdx.x; i < k; i += blockDim.x) s.flag[s.pos[i]] = 1;
  __syncthreads();
}

}  // namespace

// ---------------------------------------------------------------------
__global__ void batch_init_slot_kernel(const BatchCfg c, const BatchBufs b, uint64_t slot, double gub0)
{
  const InstDesc d = b.desc[slot];
  for (int v = threadIdx.x; v < c.n_max; v += blockDim.x) {
    if (v < d.n_vars) {
      b.lo[plane(c, slot, v)] = d.root_lb[v];
      b.hi[plane(c, slot, v)] = d.root_ub[v];
    }
    b.best_point[slot * c.n_max + v] = __longlong_as_double(0x7ff8000000000000LL);
  }
  if (threadIdx.x == 0) {
    InstState* s = &b.st[slot];
    memset(s, 0, sizeof(InstState));
    s->gub = gub0;
    s->glb = -DBL_MAX;
    s->dropped_lb_min = INFINITY;
    s->dropped_min_key = ~0ULL;
    s->pool_size = 1;
    s->viable = (-DBL_MAX <= gub0) ? 1 : 0;
    s->pool_min_key = lb_key(-DBL_MAX);
    s->use_screen = 1;
    s->counters.peak_frontier = 1;
    b.lb[slot * c.P] = -DBL_MAX;
    b.depth[slot * c.P] = 0;
  }
}

__global__ void batch_begin_kernel(const BatchCfg c, const BatchBufs b)
{
  const uint64_t slot = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= c.K) return;
  InstState& s = b.st[slot];
  const InstDesc& d = b.desc[slot];
  s.n_parents = 0;
  if (!d.active || s.done) return;
  const uint64_t L = s.pool_size;
  if (L == 0) {
    s.done = 1;
    return;
  }
  const double m = key_to_lb_b(s.pool_min_key);
  if (gap_closed_b(s.gub, m, d.tolerance)) {
    s.converged = 1;
    s.done = 1;
    return;
  }
  s.glb = m;
  if (s.expansions >= d.iter_limit || (d.batch_iter_limit && s.iterations >= d.batch_iter_limit)) {
    s.done = 1;
    return;
  }
  uint64_t E = L < c.e_max ? L : c.e_max;
  const uint64_t left = d.iter_limit - s.expansions;
  if (E > left) E = left;
  s.iterations += 1;
  s.n_parents = E;
  s.salt_base = s.expansions;
  s.expansions += E;
  s.counters.iterations = s.iterations;
  s.counters.expansions = s.expansions;
}

// select the E best parents, stage them, compact the rest in place
__global__ void __launch_bounds__(kMiThreads) batch_select_kernel(const BatchCfg c, const BatchBufs b)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ uint32_t running;
  const uint64_t slot = blockIdx.x;
  InstState* st = &b.st[slot];
  const uint32_t E = (uint32_t)st->n_parents;
  if (E == 0) return;
  const uint32_t L = (uint32_t)st->pool_size;
  const int n = b.desc[slot].n_vars;
  const SortSmem s = sort_smem(smem_raw);
  mark_smallest(b.lb + (size_t)slot * c.P, L, E, s);
  // gather the selected parents in pool order
  if (threadIdx.x == 0) running = 0;
  __syncthreads();
  for (uint32_t base = 0; base < L; base += kMiThreads) {
    const uint32_t i = base + threadIdx.x;
    const bool f = i < L && s.flag[i];
    int total;
    const int r = block_rank(f, total);
    if (f) {
      const uint32_t k = running + (uint32_t)r;
      for (int v = 0; v < n; ++v) {
        const double lo = b.lo[plane(c, slot, v) + i], hi = b.hi[plane(c, slot, v) + i];
        b.plo[splane(c, slot, v) + k] = lo;
        b.phi[splane(c, slot, v) + k] = hi;
        if (b.plo32 != nullptr) {
          b.plo32[splane(c, slot, v) + k] = __double2float_rd(lo);
          b.phi32[splane(c, slot, v) + k] = __double2float_ru(hi);
        }
      }
      b.pdepth[slot * c.e_max + k] = b.depth[(size_t)slot * c.P + i];
    }
    __syncthreads();
    if (threadIdx.x == 0) running += (uint32_t)total;
    __syncthreads();
  }
  // the unselected entries keep their order at the front of the pool
  for (uint32_t i = threadIdx.x; i < L; i += blockDim.x) s.flag[i] = !s.flag[i];
  __syncthreads();
  compact_pool(c, b, slot, L, n, s.flag, s.pos, &running);
  if (threadIdx.x == 0) {
    st->remaining = L - E;
    st->pool_size = L - E;
  }
}

__global__ void batch_branch_kernel(const BatchCfg c, const BatchBufs b)
{
  const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= c.K * c.e_max) return;
  const uint64_t slot = idx / c.e_max, k = idx % c.e_max;
  InstState* st = &b.st[slot];
  if (k >= st->n_parents) return;
  const InstDesc d = b.desc[slot];
  const size_t pk = slot * c.e_max + k;
  EnumCand* ec = reinterpret_cast<EnumCand*>(b.enum_scratch) + pk * c.n_max;
  BisCand* bc = reinterpret_cast<BisCand*>(b.bis_scratch) + pk * c.n_max;
  uint64_t* heap = b.heap_scratch + pk * c.n_max;
  SlotPlan* sp = b.slots + pk * c.max_slots;
  const PolicyParams pp = {c.log2C, c.max_cycle, c.enumerate_cap, c.relative};
  const ParentInfo pi =
      bisection_policy(b.plo + splane(c, slot, 0) + k, b.phi + splane(c, slot, 0) + k, c.e_max, d.n_vars, d.kinds,
                       pp, ec, bc, heap, sp);
  b.pinfo[pk] = pi;
  if (c.precision == CMN_PRECISION_FP32_LAZY) return;  // batch_drop_kernel counts after the verdict
  if (pi.fathom) {
    atomicAdd((unsigned long long*)&st->counters.fathomed, 1ULL);
    atomicAdd((unsigned long long*)&st->counters.fathomed_points, (unsigned long long)pi.nreg);
  } else {
    atomicAdd((unsigned long long*)&st->counters.bounded, (unsigned long long)pi.nreg);
  }
}

// Exclusive prefix of the live children per slot (n_parents << B), slots
// taken in `order`, into child_base[0..K]; child_base[K] is this
// iteration's live child count and child_base[K + 1] the most lanes any
// live instance can use per child.
//
// The lazy form's verdict takes its parents in warp runs: a run is one
// warp over 32 >> lg parents of one instance, 2^lg lanes per parent.  lg
// is chosen per instance: the capacity's lanes when few parents are live,
// and more for a long program, until a run is at most half of a warp's
// fair share of the verdict's work (the parents' program lengths over the
// grid's warps), within the lanes the instance's schedule has.  vrun gets
// the runs' exclusive prefix by `order` position and their total, vlg each
// position's lg, and the run ticket is reset.
__global__ void __launch_bounds__(1024) batch_live_kernel(const BatchCfg c, const BatchBufs b)
{
  __shared__ uint64_t wsum[32], wrun[32];
  __shared__ uint64_t carry, rcarry;
  __shared__ int gmax;
  __shared__ unsigned long long work, parents;
  if (threadIdx.x == 0) {
    carry = 0;
    rcarry = 0;
    gmax = 1;
    work = 0;
    parents = 0;
  }
  __syncthreads();
  const bool runs = b.vrun != nullptr;
  int my_gmax = 1;
  unsigned long long my_work = 0, my_par = 0;
  for (uint64_t i = threadIdx.x; i < c.K; i += 1024) {
    const uint64_t np = b.st[i].n_parents;
    if (np > 0 && b.desc[i].g_max > my_gmax) my_gmax = b.desc[i].g_max;
    my_work += np * (uint64_t)b.desc[i].prog_len;
    my_par += np;
  }
  atomicMax(&gmax, my_gmax);
  if (runs) {
    atomicAdd(&work, my_work);
    atomicAdd(&parents, my_par);
  }
  __syncthreads();
  int lg_cap = 0;
  unsigned long long half_share = 0;
  if (runs) {
    lg_cap = lanes_per_box(parents, c.eval_capacity, min(gmax, c.g_max));
    const unsigned long long warps = c.eval_capacity >> 5 > 0 ? c.eval_capacity >> 5 : 1;
    half_share = work / (64ULL * warps);  // (work / 32 lanes / warps) / 2
    if (half_share < 64) half_share = 64;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (uint64_t base = 0; base < c.K; base += 1024) {
    const uint64_t i = base + threadIdx.x;
    uint64_t v = 0, u = 0;
    int lgi = 0;
    if (i < c.K) {
      const uint32_t slot = b.order[i];
      const uint64_t np = b.st[slot].n_parents;
      v = np << c.log2C;
      if (runs && np > 0) {
        const InstDesc& d = b.desc[slot];
        int lim = 0;
        while (lim < 5 && (2 << lim) <= d.g_max) ++lim;
        int l = 0;
        while (l < lim && ((unsigned long long)d.prog_len >> l) > half_share) ++l;
        lgi = max(l, min(lg_cap, lim));
        u = ((np << lgi) + 31) >> 5;
      }
    }
    uint64_t x = v, y = u;
    for (int off = 1; off < 32; off <<= 1) {
      const uint64_t xa = __shfl_up_sync(0xffffffffu, x, off);
      const uint64_t ya = __shfl_up_sync(0xffffffffu, y, off);
      if (lane >= off) {
        x += xa;
        y += ya;
      }
    }
    if (lane == 31) {
      wsum[wid] = x;
      wrun[wid] = y;
    }
    __syncthreads();
    if (wid == 0) {
      uint64_t w = wsum[lane], z = wrun[lane];
      for (int off = 1; off < 32; off <<= 1) {
        const uint64_t wa = __shfl_up_sync(0xffffffffu, w, off);
        const uint64_t za = __shfl_up_sync(0xffffffffu, z, off);
        if (lane >= off) {
          w += wa;
          z += za;
        }
      }
      wsum[lane] = w;
      wrun[lane] = z;
    }
    __syncthreads();
    const uint64_t cy = carry, ry = rcarry;
    if (i < c.K) {
      b.child_base[i] = cy + (wid > 0 ? wsum[wid - 1] : 0) + x - v;
      if (runs) {
        b.vrun[i] = ry + (wid > 0 ? wrun[wid - 1] : 0) + y - u;
        b.vlg[i] = (uint8_t)lgi;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      carry = cy + wsum[31];
      rcarry = ry + wrun[31];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    b.child_base[c.K] = carry;
    b.child_base[c.K + 1] = (uint64_t)min(gmax, c.g_max);
    if (runs) {
      b.vrun[c.K] = rcarry;
      b.vrun[c.K + 1] = 0;
    }
  }
}

// Live child i -> its global index slot * child_stride + local.
__device__ __forceinline__ uint64_t live_child(const BatchCfg& c, const BatchBufs& b, uint64_t i)
{
  uint64_t lo = 0, hi = c.K;  // largest position with child_base[pos] <= i
  while (hi - lo > 1) {
    const uint64_t mid = (lo + hi) >> 1;
    if (__ldg(b.child_base + mid) <= i) lo = mid;
    else hi = mid;
  }
  return (uint64_t)__ldg(b.order + lo) * c.child_stride + (i - __ldg(b.child_base + lo));
}

// Lanes of a group of 2^lg that run instance d's program on one box: all of
// them over the instance's lane schedule, or lane 0 alone over the whole
// program when the instance has none (or takes fewer lanes).
template <typename T, typename V, bool kFused = false>
__device__ __forceinline__ Verdict<T> batch_lane_verdict(const InstDesc& d, const Instr* prog, int lg, int lane,
                                                         const V& vars, const Tile<T>& t)
{
  int li = 0;
  while (li < lg && (2 << li) <= d.g_max) ++li;
  if (d.sched == nullptr || li == 0) {
    if (lane == 0) return run_interval<T, V, kFused>(prog, d.prog_len, vars, t);
    return verdict_init<T>();
  }
  if (lane < (1 << li)) return run_interval_lane<T, V, kFused>(prog, d.sched, li, lane, vars, t);
  return verdict_init<T>();
}

__device__ __forceinline__ double child_bound(const BatchCfg& c, const BatchBufs& b, uint64_t slot, uint64_t k,
                                              uint64_t r, int v, const SlotPlan* sp, uint32_t count, double& hi)
{
  double lo = b.plo[splane(c, slot, v) + k];
  hi = b.phi[splane(c, slot, v) + k];
  for (uint32_t j = 0; j < count; ++j) {
    if (sp[j].vid == (uint32_t)v) {
      const uint64_t part = slot_part(r, sp[j]);
      slot_bounds(sp[j], lo, hi, part, lo, hi);
      break;
    }
  }
  return lo;
}

// ---- the lazy form over many instances (as the single-instance solver
// runs it: csrc/search_kernels.cu solver_iteration, csrc/eval_kernels.cu) ----
__device__ __forceinline__ size_t common_at(const BatchCfg& c, uint64_t slot, int s, uint64_t k)
{
  return 2 * (((size_t)slot * c.seg_max + s) * c.e_max + k);
}

__device__ __forceinline__ size_t part_at(const BatchCfg& c, uint64_t slot, int s, uint64_t u, uint64_t k)
{
  return 2 * ((((size_t)slot * c.seg_max + s) * ((size_t)1 << c.log2C) + u) * c.e_max + k);
}

// A parent's FP32 planes with one variable narrowed to one part of its slot.
struct BatchPartVars {
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

__device__ __forceinline__ bool slot_var_before_b(const SlotPlan* sp, int j, int v)
{
  for (int q = 0; q < j; ++q)
    if (sp[q].vid == (uint32_t)v) return true;
  return false;
}

// FP64 verdict of every staged parent (fused terms, as mode 6 of the
// single-instance evaluator): plb, pfeas.  Each warp draws warp runs
// (batch_live_kernel's layout: 32 >> lg parents of one instance, 2^lg
// lanes each over the program's lane schedule; the verdict is the same)
// from a ticket, longest program first, until none is left: a warp that
// finishes a short run takes the next, so the SMs end together and no
// long program waits on one lane.  The ticket is warp-uniform, so every
// lane of a warp reaches the shuffles.
__global__ void __launch_bounds__(kEvalThreads) batch_verdict_kernel(const BatchCfg c, const BatchBufs b)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* base = reinterpret_cast<double*>(smem_raw);
  const int B = blockDim.x;
  Tile<double> t;
  t.lo = nullptr;
  t.hi = nullptr;
  t.slo = base;
  t.shi = base + (size_t)c.slots_max * B;
  t.stride = B;
  t.tid = threadIdx.x;
  const uint64_t runs = b.vrun[c.K];
  unsigned long long* ticket = reinterpret_cast<unsigned long long*>(b.vrun + c.K + 1);
  const int wl = threadIdx.x & 31;
  for (;;) {
    unsigned long long w = 0;
    if (wl == 0) w = atomicAdd(ticket, 1ULL);
    w = __shfl_sync(0xffffffffu, w, 0);
    if (w >= runs) break;
    uint64_t pos = 0, hi = c.K;  // largest position with vrun[pos] <= w: it has runs
    while (hi - pos > 1) {
      const uint64_t mid = (pos + hi) >> 1;
      if (b.vrun[mid] <= w) pos = mid;
      else hi = mid;
    }
    const uint64_t slot = b.order[pos];
    const int lg = b.vlg[pos];
    const int G = 1 << lg;
    const int lane = wl & (G - 1);
    const uint64_t k = ((w - b.vrun[pos]) << (5 - lg)) + (uint64_t)(wl >> lg);
    const bool live = k < b.st[slot].n_parents;
    Verdict<double> v = verdict_init<double>();
    if (live) {
      const InstDesc& d = b.desc[slot];
      ChildVars<double, double> cv = {};
      cv.plo = b.plo + splane(c, slot, 0) + k;
      cv.phi = b.phi + splane(c, slot, 0) + k;
      cv.pstride = c.e_max;
      cv.mask = 0;
      cv.count = 0;
      cv.stride = B;
      v = batch_lane_verdict<double, ChildVars<double, double>, true>(d, d.prog64, lg, lane, cv, t);
    }
    if (lg > 0) v = group_verdict<double>(v, G);
    if (live && lane == 0) {
      b.plb[slot * c.e_max + k] = v.obj.lo;
      b.pfeas[slot * c.e_max + k] = (uint8_t)v.feasible;
    }
  }
}

// A box the verdict excludes (reference predicate, or bound above the
// incumbent) is not expanded; the expansion counters as lazy_drop_kernel.
__global__ void batch_drop_kernel(const BatchCfg c, const BatchBufs b)
{
  const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= c.K * c.e_max) return;
  const uint64_t slot = idx / c.e_max, k = idx % c.e_max;
  InstState* st = &b.st[slot];
  if (k >= st->n_parents) return;
  const size_t pk = slot * c.e_max + k;
  ParentInfo pi = b.pinfo[pk];
  unsigned long long dropped = 0;
  if (!b.pfeas[pk] || b.plb[pk] > st->gub) {
    pi = ParentInfo{0, 0, 0};
    b.pinfo[pk] = pi;
    dropped = 1;
  }
  atomicAdd((unsigned long long*)&st->counters.certified_fp64, 1ULL);
  if (dropped) atomicAdd((unsigned long long*)&st->counters.certify_pruned, 1ULL);
  if (pi.fathom) {
    atomicAdd((unsigned long long*)&st->counters.fathomed, 1ULL);
    atomicAdd((unsigned long long*)&st->counters.fathomed_points, (unsigned long long)pi.nreg);
  } else {
    atomicAdd((unsigned long long*)&st->counters.bounded, (unsigned long long)pi.nreg);
  }
}

// Common chain sums of every (instance, segment, parent) whose program has
// the incremental tables (inc_common_kernel per instance).
__global__ void __launch_bounds__(kEvalThreads) batch_inc_common_kernel(const BatchCfg c, const BatchBufs b)
{
  const uint64_t total = c.K * (uint64_t)c.seg_max * c.e_max;
  for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = idx % c.e_max, rest = idx / c.e_max;
    const int s = (int)(rest % (uint64_t)c.seg_max);
    const uint64_t slot = rest / (uint64_t)c.seg_max;
    if (k >= b.st[slot].n_parents) continue;
    const InstDesc& d = b.desc[slot];
    if (s >= d.inc_segments) continue;
    const ParentInfo pi = b.pinfo[slot * c.e_max + k];
    if (pi.nreg == 0 || pi.fathom) continue;  // no bounded children
    const SlotPlan* sp = b.slots + (slot * c.e_max + k) * c.max_slots;
    uint64_t mask = 0;
    for (uint32_t j = 0; j < pi.count; ++j) mask |= 1ULL << (sp[j].vid & 63);
    ChildVars<float, float> pv = {};
    pv.plo = b.plo32 + splane(c, slot, 0) + k;
    pv.phi = b.phi32 + splane(c, slot, 0) + k;
    pv.pstride = c.e_max;
    auto is_split = [&](int v) {
      if (!((mask >> (v & 63)) & 1ULL)) return false;
      for (uint32_t j = 0; j < pi.count; ++j)
        if (sp[j].vid == (uint32_t)v) return true;
      return false;
    };
    Iv<float> acc = {0.0f, 0.0f};
    const int pb = __ldg(d.inc_seg + 3 * s), pt = __ldg(d.inc_seg + 3 * s + 1);
    for (int pc = pb; pc < pt; ++pc) {
      const Instr cur = load_instr(d.prog32, pc);
      const int code = cur.head & 7;
      const bool reads_var = code == kOpTerm || (cur.modes & 3) == kModeVar;
      if (reads_var && (is_split(cur.a) || (code == kOpTerm && is_split(cur.b)))) continue;
      acc = chain_add<float, ChildVars<float, float>>(acc, cur, pv);
    }
    const size_t at = common_at(c, slot, s, k);
    b.inc_common[at] = acc.lo;
    b.inc_common[at + 1] = acc.hi;
  }
}

// Part sums of every (instance, slot part, parent) (inc_parts_kernel per
// instance), every segment of the instance's program.
__global__ void __launch_bounds__(kEvalThreads) batch_inc_parts_kernel(const BatchCfg c, const BatchBufs b)
{
  const uint64_t C = 1ULL << c.log2C;
  const uint64_t total = c.K * C * c.e_max;
  for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = idx % c.e_max, rest = idx / c.e_max;
    const uint64_t u = rest % C, slot = rest / C;
    if (k >= b.st[slot].n_parents) continue;
    const InstDesc& d = b.desc[slot];
    const int S = d.inc_segments;
    if (S == 0) continue;
    const ParentInfo pi = b.pinfo[slot * c.e_max + k];
    if (pi.fathom || pi.nreg == 0) continue;
    const SlotPlan* sp = b.slots + (slot * c.e_max + k) * c.max_slots;
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
    if (j < 0) continue;
    const SlotPlan sj = sp[j];
    const int vj = (int)sj.vid;
    const bool repeated = slot_var_before_b(sp, j, vj);
    BatchPartVars pv;
    pv.plo = b.plo32 + splane(c, slot, 0) + k;
    pv.phi = b.phi32 + splane(c, slot, 0) + k;
    pv.pstride = c.e_max;
    pv.vid = vj;
    double lo, hi;
    slot_bounds(sj, b.plo[splane(c, slot, vj) + k], b.phi[splane(c, slot, vj) + k], p, lo, hi);
    pv.val = {Widen<float, double>::lo(lo), Widen<float, double>::hi(hi)};
    for (int s = 0; s < S; ++s) {
      Iv<float> acc = {0.0f, 0.0f};
      if (!repeated) {
        const int q0 = __ldg(d.inc_off + (uint64_t)vj * S + s), q1 = __ldg(d.inc_off + (uint64_t)vj * S + s + 1);
        for (int q = q0; q < q1; ++q) {
          const Instr cur = load_instr(d.prog32, __ldg(d.inc_pcs + q));
          if ((cur.head & 7) == kOpTerm) {
            const int other = cur.a == vj ? cur.b : cur.a;
            if (other != vj && slot_var_before_b(sp, j, other)) continue;
          }
          acc = chain_add<float, BatchPartVars>(acc, cur, pv);
        }
      }
      const size_t at = part_at(c, slot, s, u, k);
      b.inc_parts[at] = acc.lo;
      b.inc_parts[at + 1] = acc.hi;
    }
  }
}

// A child's FP32 bound from its parent's common sums and its slots' part
// sums, then each segment's checks and objective (eval_children_inc_kernel).
__device__ Verdict<float> batch_inc_child(const BatchCfg& c, const BatchBufs& b, const InstDesc& d, uint64_t slot,
                                          uint64_t k, uint64_t r, const SlotPlan* sp, uint32_t count,
                                          const ChildVars<float, float>& cv, uint32_t* opart, int B)
{
  uint64_t pbase = 0;
  for (uint32_t j = 0; j < count; ++j) {
    opart[j * B] = (uint32_t)(pbase + slot_part(r, sp[j]));
    pbase += sp[j].width;
  }
  Verdict<float> v = verdict_init<float>();
  for (int s = 0; s < d.inc_segments; ++s) {
    const size_t ca = common_at(c, slot, s, k);
    Iv<float> acc = {b.inc_common[ca], b.inc_common[ca + 1]};
    for (uint32_t j = 0; j < count; ++j) {
      const size_t at = part_at(c, slot, s, opart[j * B], k);
      acc = iv_add(acc, Iv<float>{b.inc_parts[at], b.inc_parts[at + 1]});
    }
    chain_tail<float, ChildVars<float, float>>(d.prog32, __ldg(d.inc_seg + 3 * s + 1), __ldg(d.inc_seg + 3 * s + 2),
                                               cv, acc, v);
  }
  return v;
}

// The FP32 sample screen over every live child (sample_screen_kernel with
// one lane per child): per child its smallest FP32 sample value and that
// sample's index, +inf when none is feasible in FP32 or it is not sampled.
__global__ void __launch_bounds__(kEvalThreads) batch_screen_kernel(const BatchCfg c, const BatchBufs b)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* base = reinterpret_cast<float*>(smem_raw);
  const int B = blockDim.x;
  Tile<float> t;
  t.lo = base;
  t.hi = base;
  t.slo = base + (size_t)c.n_max * B;
  t.shi = t.slo;
  t.stride = B;
  t.tid = threadIdx.x;
  const uint64_t total = b.child_base[c.K];
  for (uint64_t idx = (uint64_t)blockIdx.x * B + threadIdx.x; idx < total; idx += (uint64_t)gridDim.x * B) {
    const uint64_t g = live_child(c, b, idx);
    const uint64_t slot = g / c.child_stride, local = g % c.child_stride;
    const uint64_t k = local >> c.log2C, r = local & ((1ULL << c.log2C) - 1ULL);
    const InstState* st = &b.st[slot];
    const ParentInfo pi = b.pinfo[slot * c.e_max + k];
    Best32 best = {INFINITY, 0};
    const bool fathom = pi.fathom != 0;
    bool live = r < pi.nreg;
    if (live && !fathom) {
      const uint8_t s8 = b.cstate[g] & 0x7f;
      live = c.sample_all ? (s8 != kChildNone) : (s8 == kChildEligible);
    }
    if (live) {
      const InstDesc& d = b.desc[slot];
      const SlotPlan* sp = b.slots + (slot * c.e_max + k) * c.max_slots;
      const uint64_t S = fathom ? 1 : c.S;
      const uint64_t salt = st->salt_base + k + 1;
      for (uint64_t i = 0; i < S; ++i) {
        for (int v = 0; v < d.n_vars; ++v) {
          double hi;
          const double lo = child_bound(c, b, slot, k, r, v, sp, pi.count, hi);
          const double x = fathom ? lo : sample_value(d.kinds[v] != 0, lo, hi, (uint64_t)v, i, r, salt);
          t.lo[v * B + t.tid] = __double2float_rn(x);
        }
        PointVerdict32 pv = {INFINITY, true, false};
        if (d.sched != nullptr) {
          const LaneSegs l0 = lane_segments(d.sched, 0, 0);
          for (int j = l0.b; j < l0.e && pv.feasible; ++j)
            point_range32(d.prog32p, __ldg(l0.pairs + 2 * j), __ldg(l0.pairs + 2 * j + 1), t, pv);
        } else {
          point_range32(d.prog32p, 0, d.prog_len, t, pv);
        }
        const float value = (pv.feasible && !(pv.obj != pv.obj)) ? pv.obj : INFINITY;
        if (value < best.value) best = Best32{value, (uint32_t)i};
      }
    }
    b.cbest[g] = best;
  }
}

// Lane of the n-th (from 0) set bit of m, -1 when m has fewer set bits.
__device__ __forceinline__ int nth_set_lane(unsigned m, int n)
{
  for (int i = 0; i < n && m != 0u; ++i) m &= m - 1u;
  return m != 0u ? __ffs((int)m) - 1 : -1;
}

// Each chunk of 32 consecutive children of an instance: its FP32-best
// sample (chunk_pick's order: smallest value, then first child, then first
// sample) evaluated again in FP64; only that value can become the
// incumbent (sample_children_kernel in chunk mode).  cval / ce of the
// chunk's other children are +inf.
//
// A warp takes 32 >> lg chunks per pass (lg from the live children and the
// grid, as the bound's lane groups) and scans each on one lane.  It then
// splits its 32 lanes evenly over the chunks whose pick is FP32-feasible:
// with q of them, a group of 2^lw lanes (2^lw * q <= 32) evaluates one
// point over its instance's lane schedule.  Most chunks of an instance
// with several constraints hold no feasible point, so the few that do get
// many lanes instead of running a long program on one.  The loop and the
// shuffles are warp-uniform: every lane of a warp takes the same passes.
__global__ void __launch_bounds__(kEvalThreads) batch_chunk_kernel(const BatchCfg c, const BatchBufs b)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* base = reinterpret_cast<double*>(smem_raw);
  const int B = blockDim.x;
  Tile<double> t;
  t.lo = base;
  t.hi = base;
  t.slo = base + (size_t)c.n_max * B;
  t.shi = t.slo;
  t.stride = B;
  t.tid = threadIdx.x;  // every lane stages its group's point in its own column
  const uint64_t per_slot = (c.child_stride + 31) >> 5;
  const uint64_t items = c.K * per_slot;
  const int lg = lanes_per_box((b.child_base[c.K] + 31) >> 5, c.sample_capacity, (int)b.child_base[c.K + 1]);
  const int lane = threadIdx.x & 31;
  const uint64_t per_warp = 32u >> lg;
  const uint64_t warps = (uint64_t)gridDim.x * (uint64_t)(B >> 5);
  for (uint64_t w0 = ((uint64_t)blockIdx.x * (uint64_t)(B >> 5) + (threadIdx.x >> 5)) * per_warp; w0 < items;
       w0 += warps * per_warp) {
    // (1) lane i < per_warp: the pick of chunk w0 + i
    bool need = false;
    uint64_t slot = 0, bg = 0;
    uint32_t bi = 0;
    if ((uint64_t)lane < per_warp && w0 + lane < items) {
      const uint64_t idx = w0 + lane;
      slot = idx / per_slot;
      const uint64_t ch = idx % per_slot;
      const uint64_t nch = b.st[slot].n_parents << c.log2C;
      const uint64_t g0 = ch << 5;
      if (g0 < nch) {
        const uint64_t g1 = nch < g0 + 32 ? nch : g0 + 32;
        const uint64_t cbase = slot * c.child_stride;
        float bv = INFINITY;
        for (uint64_t x = g0; x < g1; ++x) {
          b.cval[cbase + x] = INFINITY;
          const Best32 q = b.cbest[cbase + x];
          if (q.value < bv) {
            bv = q.value;
            bg = x;
            bi = q.i;
          }
        }
        if (bv < INFINITY) {
          const uint64_t k = bg >> c.log2C, r = bg & ((1ULL << c.log2C) - 1ULL);
          need = r < b.pinfo[slot * c.e_max + k].nreg;
        }
      }
    }
    // (2) the warp's lanes over the picks to evaluate; the barrier orders
    // the +inf stores above before a group leader's store of the value
    __syncwarp();
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (m == 0u) continue;
    const int q = __popc(m);
    int lw = 0;
    while ((q << (lw + 1)) <= 32) ++lw;
    const int G = 1 << lw, gl = lane & (G - 1);
    const int src = nth_set_lane(m, lane >> lw);
    const int from = src < 0 ? lane : src;
    slot = __shfl_sync(0xffffffffu, slot, from);
    bg = __shfl_sync(0xffffffffu, bg, from);
    bi = __shfl_sync(0xffffffffu, bi, from);
    const bool act = src >= 0;
    PointVerdict pv;
    pv.obj = INFINITY;
    pv.feasible = true;
    pv.has_obj = false;
    const InstDesc* d = act ? &b.desc[slot] : nullptr;
    const uint64_t k = bg >> c.log2C, r = bg & ((1ULL << c.log2C) - 1ULL);
    ParentInfo pi = {0, 0, 0};
    if (act) {
      pi = b.pinfo[slot * c.e_max + k];
      const bool fathom = pi.fathom != 0;
      const SlotPlan* sp = b.slots + (slot * c.e_max + k) * c.max_slots;
      const uint64_t salt = b.st[slot].salt_base + k + 1;
      for (int v = 0; v < d->n_vars; ++v) {
        double hi;
        const double lo = child_bound(c, b, slot, k, r, v, sp, pi.count, hi);
        t.lo[v * B + t.tid] = fathom ? lo : sample_value(d->kinds[v] != 0, lo, hi, (uint64_t)v, bi, r, salt);
      }
      int li = 0;
      while (li < lw && (2 << li) <= d->g_max) ++li;
      if (d->sched == nullptr || li == 0) {
        if (gl == 0) pv = run_point_ordered(d->prog64, d->prog_len, d->sched, t);
      } else if (gl < (1 << li)) {
        pv = run_point_lane(d->prog64, d->sched, li, gl, t);
      }
    }
    if (lw > 0) pv = group_point_verdict(pv, G);
    if (act && gl == 0) {
      InstState* st = &b.st[slot];
      const bool fathom = pi.fathom != 0;
      double value = (pv.feasible && !(pv.obj != pv.obj)) ? pv.obj : INFINITY;
      if (fathom && value < INFINITY) {
        bool ok = true;
        for (int v = 0; v < d->n_vars && ok; ++v) {
          const double x = t.lo[v * B + t.tid];
          if (!(x >= d->root_lb[v]) || !(x <= d->root_ub[v])) ok = false;
          else if (d->kinds[v] != 0 && fabs(__dsub_rn(x, rint(x))) > 1e-6) ok = false;
        }
        if (!ok) {
          if (value < st->gub) atomicAdd((unsigned long long*)&st->counters.witness_rejected, 1ULL);
          value = INFINITY;
        }
      }
      const uint64_t S = fathom ? 1 : c.S;
      const uint64_t cbase = slot * c.child_stride;
      b.cval[cbase + bg] = value;
      b.ce[cbase + bg] = r * S + bi;
    }
  }
}

// kMode 1: FP64 bound; 2: FP32 screen; 3: FP64 certify of the listed
// children; 5: the lazy form's FP32 child bound (incremental from the part
// sums when the instance's program has the tables, else its whole FP32
// program), the parent's certified bound folded in.  Variables come from
// the parent planes (FP32 copies for the FP32 passes) with the child's
// split variables in this thread's shared-memory column.  The launch walks
// only live children (child_base), with 2^lg lanes per child when there
// are few of them.
template <typename T, int kMode>
__global__ void __launch_bounds__(kEvalThreads, 4) batch_eval_kernel(const BatchCfg c, const BatchBufs b)
{
  using S = T;  // the screen reads the FP32 planes, the FP64 passes the FP64 planes
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* base = reinterpret_cast<T*>(smem_raw);
  const int B = blockDim.x;
  Tile<T> t;  // program slots only
  t.lo = nullptr;
  t.hi = nullptr;
  t.slo = base;
  t.shi = base + (size_t)c.slots_max * B;
  t.stride = B;
  t.tid = threadIdx.x;
  T* olo = base + (size_t)2 * c.slots_max * B + threadIdx.x;
  T* ohi = olo + (size_t)c.max_slots * B;
  int32_t* ovid = reinterpret_cast<int32_t*>(base + (size_t)2 * (c.slots_max + c.max_slots) * B) + threadIdx.x;
  // kMode 5: the child's slot parts (u_j), after the split variables
  uint32_t* opart = reinterpret_cast<uint32_t*>(ovid + (size_t)c.max_slots * B);
  const S* planes_lo;
  const S* planes_hi;
  if constexpr (sizeof(T) == 4) {
    planes_lo = b.plo32;
    planes_hi = b.phi32;
  } else {
    planes_lo = b.plo;
    planes_hi = b.phi;
  }
  const uint64_t total = kMode == 3 ? *b.list_count : b.child_base[c.K];
  const int lg = lanes_per_box(total, c.eval_capacity, (int)b.child_base[c.K + 1]);
  const int G = 1 << lg;
  const int lane = threadIdx.x & (G - 1);
  const uint64_t per_block = (uint64_t)(B >> lg);
  for (uint64_t bb = (uint64_t)blockIdx.x * per_block; bb < total; bb += (uint64_t)gridDim.x * per_block) {
    const uint64_t idx = bb + (threadIdx.x >> lg);
    bool live = idx < total;
    uint64_t g = 0, slot = 0, k = 0, r = 0;
    ParentInfo pi = {0, 1, 0};
    const InstState* st = nullptr;
    if (live) {
      g = kMode == 3 ? (uint64_t)b.list[idx] : live_child(c, b, idx);
      slot = g / c.child_stride;
      const uint64_t local = g % c.child_stride;
      k = local >> c.log2C;
      r = local & ((1ULL << c.log2C) - 1ULL);
      st = &b.st[slot];
      pi = b.pinfo[slot * c.e_max + k];
      if (pi.fathom || r >= pi.nreg) {
        if (kMode != 3 && lane == 0) b.cstate[g] = kChildNone;
        live = false;
      }
    }
    const SlotPlan* sp = b.slots + (slot * c.e_max + k) * c.max_slots;
    if (live && kMode == 2 && !st->use_screen) {
      bool dup = false;
      for (uint32_t j = 0; j < pi.count; ++j) dup = dup || (slot_part(r, sp[j]) >= sp[j].dom);
      if (lane == 0) b.cstate[g] = dup ? kChildDuplicate : kChildScreened;
      live = false;
    }
    Verdict<T> v = verdict_init<T>();
    if (live) {
      ChildVars<T, S> cv;
      cv.plo = planes_lo + splane(c, slot, 0) + k;
      cv.phi = planes_hi + splane(c, slot, 0) + k;
      cv.pstride = c.e_max;
      cv.mask = 0;
      cv.olo = olo;
      cv.ohi = ohi;
      cv.ovid = ovid;
      cv.count = (int)pi.count;
      cv.stride = B;
      bool dup = false;
      for (uint32_t j = 0; j < pi.count; ++j) {
        const SlotPlan sj = sp[j];
        const uint64_t part = slot_part(r, sj);
        if (part >= sj.dom) dup = true;
        double lo, hi;
        slot_bounds(sj, b.plo[splane(c, slot, sj.vid) + k], b.phi[splane(c, slot, sj.vid) + k], part, lo, hi);
        olo[j * B] = Widen<T, double>::lo(lo);
        ohi[j * B] = Widen<T, double>::hi(hi);
        ovid[j * B] = (int32_t)sj.vid;
        cv.mask |= 1ULL << (sj.vid & 63);
      }
      if (dup) {
        if (lane == 0) b.cstate[g] = kChildDuplicate;
        live = false;
      } else {
        const InstDesc& d = b.desc[slot];
        const Instr* prog = sizeof(T) == 4 ? d.prog32 : d.prog64;
        if constexpr (kMode == 5 && sizeof(T) == 4) {
          if (d.inc_segments > 0) {
            // the parent's common sum plus the part sum of each slot
            if (lane == 0) v = batch_inc_child(c, b, d, slot, k, r, sp, pi.count, cv, opart, B);
          } else {
            v = batch_lane_verdict<T, ChildVars<T, S>>(d, prog, lg, lane, cv, t);
          }
        } else {
          v = batch_lane_verdict<T, ChildVars<T, S>>(d, prog, lg, lane, cv, t);
        }
      }
    }
    if (lg > 0) v = group_verdict<T>(v, G);
    if (live && lane == 0) {
      double lb = (double)v.obj.lo;
      const double gub = st->gub;
      if (kMode == 5 || (kMode == 3 && c.precision == CMN_PRECISION_FP32_LAZY)) {
        // the parent's certified bound holds for every child box inside it
        const double plb = b.plb[slot * c.e_max + k];
        lb = plb > lb ? plb : lb;
      }
      b.clb[g] = lb;
      if (kMode == 2) {
        b.cstate[g] = v.excluded ? kChildInfeasible : (lb > gub ? kChildDominated : kChildScreened);
      } else if (kMode == 5) {
        // a survivor within the band below the incumbent goes to the FP64
        // pass, which may prune it; below the band FP64 could not
        b.cstate[g] = v.excluded     ? kChildInfeasible
                      : lb > gub     ? kChildDominated
                      : lb >= certify_floor(gub) ? kChildScreened
                                                 : kChildEligible;
      } else {
        const uint8_t sv = !v.feasible ? kChildInfeasible : (lb > gub ? kChildDominated : kChildEligible);
        b.cstate[g] = kMode == 3 ? (uint8_t)(sv | kCertifiedBit) : sv;
      }
    }
  }
}


// samples (or exact points of fathomed parents) of every live child: the
// best (value, element) per child.  With 2^lg lanes per child every lane
// stages the point in its own column and runs its share of the program.
__global__ void __launch_bounds__(kEvalThreads) batch_sample_kernel(const BatchCfg c, const BatchBufs b)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* base = reinterpret_cast<double*>(smem_raw);
  const int B = blockDim.x;
  Tile<double> t;
  t.lo = base;
  t.hi = base;
  t.slo = base + (size_t)c.n_max * B;
  t.shi = t.slo;
  t.stride = B;
  t.tid = threadIdx.x;
  const uint64_t total = b.child_base[c.K];
  const int lg = lanes_per_box(total, c.sample_capacity, (int)b.child_base[c.K + 1]);
  const int G = 1 << lg;
  const int lane = threadIdx.x & (G - 1);
  const uint64_t per_block = (uint64_t)(B >> lg);
  for (uint64_t bb = (uint64_t)blockIdx.x * per_block; bb < total; bb += (uint64_t)gridDim.x * per_block) {
    const uint64_t idx = bb + (threadIdx.x >> lg);
    bool live = idx < total;
    uint64_t g = 0, slot = 0, k = 0, r = 0;
    ParentInfo pi = {0, 0, 0};
    InstState* st = nullptr;
    bool fathom = false;
    if (live) {
      g = live_child(c, b, idx);
      slot = g / c.child_stride;
      const uint64_t local = g % c.child_stride;
      k = local >> c.log2C;
      r = local & ((1ULL << c.log2C) - 1ULL);
      st = &b.st[slot];
      if (lane == 0) b.cval[g] = INFINITY;
      pi = b.pinfo[slot * c.e_max + k];
      fathom = pi.fathom != 0;
      if (r >= pi.nreg) live = false;
      if (live && !fathom) {
        const uint8_t s8 = b.cstate[g] & 0x7f;
        live = c.sample_all ? (s8 != kChildNone) : (s8 == kChildEligible);
      }
    }
    const SlotPlan* sp = b.slots + (slot * c.e_max + k) * c.max_slots;
    const uint64_t S = fathom ? 1 : c.S;
    double best = INFINITY;
    uint64_t best_e = 0;
    for (uint64_t i = 0; i < c.S; ++i) {  // c.S bounds every box's S: the shuffles see every lane
      const bool act = live && i < S;
      PointVerdict pv;
      pv.obj = INFINITY;
      pv.feasible = true;
      pv.has_obj = false;
      const InstDesc* d = act ? &b.desc[slot] : nullptr;
      if (act) {
        const uint64_t salt = st->salt_base + k + 1;
        for (int v = 0; v < d->n_vars; ++v) {
          double hi;
          const double lo = child_bound(c, b, slot, k, r, v, sp, pi.count, hi);
          t.lo[v * B + t.tid] = fathom ? lo : sample_value(d->kinds[v] != 0, lo, hi, (uint64_t)v, i, r, salt);
        }
        int li = 0;
        while (li < lg && (2 << li) <= d->g_max) ++li;
        if (d->sched == nullptr || li == 0) {
          if (lane == 0) pv = run_point_ordered(d->prog64, d->prog_len, d->sched, t);
        } else if (lane < (1 << li)) {
          pv = run_point_lane(d->prog64, d->sched, li, lane, t);
        }
      }
      if (lg > 0) pv = group_point_verdict(pv, G);
      if (act && lane == 0) {
        double value = (pv.feasible && !(pv.obj != pv.obj)) ? pv.obj : INFINITY;
        if (fathom && value < INFINITY) {
          bool ok = true;
          for (int v = 0; v < d->n_vars && ok; ++v) {
            const double x = t.lo[v * B + t.tid];
            if (!(x >= d->root_lb[v]) || !(x <= d->root_ub[v])) ok = false;
            else if (d->kinds[v] != 0 && fabs(__dsub_rn(x, rint(x))) > 1e-6) ok = false;
          }
          if (!ok) {
            if (value < st->gub) atomicAdd((unsigned long long*)&st->counters.witness_rejected, 1ULL);
            value = INFINITY;
          }
        }
        if (value < best) {
          best = value;
          best_e = r * S + i;
        }
      }
    }
    if (live && lane == 0) {
      b.cval[g] = best;
      b.ce[g] = best_e;
    }
  }
}

// per instance: incumbent, prune, append kept children, evict, statistics
__global__ void __launch_bounds__(kMiThreads) batch_finish_kernel(const BatchCfg c, const BatchBufs b)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ uint32_t running;
  __shared__ Cand best_s;
  __shared__ unsigned long long cnt[10];
  __shared__ unsigned long long min_key_s;
  const uint64_t slot = blockIdx.x;
  InstState* st = &b.st[slot];
  const uint32_t E = (uint32_t)st->n_parents;
  if (E == 0) return;
  const InstDesc d = b.desc[slot];
  const int n = d.n_vars;
  const uint32_t nch = E << c.log2C;
  const uint64_t cbase = slot * c.child_stride;
  const double gub_old = st->gub;
  if (threadIdx.x < 10) cnt[threadIdx.x] = 0;
  if (threadIdx.x == 0) min_key_s = ~0ULL;

  // (1) ArgMin over (value, parent, element)
  Cand mine = {INFINITY, 0xffffffffu, 0, ~0ULL};
  for (uint32_t local = threadIdx.x; local < nch; local += blockDim.x) {
    const double v = b.cval[cbase + local];
    if (v < INFINITY) {
      const Cand cc = {v, local >> c.log2C, 0, b.ce[cbase + local]};
      if (cand_less(cc, mine)) mine = cc;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    Cand o;
    o.value = __shfl_down_sync(0xffffffffu, mine.value, off);
    o.k = __shfl_down_sync(0xffffffffu, mine.k, off);
    o.e = __shfl_down_sync(0xffffffffu, mine.e, off);
    o.pad = 0;
    if (cand_less(o, mine)) mine = o;
  }
  {
    __shared__ Cand wb[kMiThreads / 32];
    if ((threadIdx.x & 31) == 0) wb[threadIdx.x >> 5] = mine;
    __syncthreads();
    if (threadIdx.x == 0) {
      Cand bst = wb[0];
      for (int w = 1; w < kMiThreads / 32; ++w)
        if (cand_less(wb[w], bst)) bst = wb[w];
      best_s = bst;
    }
    __syncthreads();
  }
  const Cand best = best_s;
  const bool improved = best.value < gub_old;
  if (improved) {
    const uint64_t k = best.k;
    const size_t pk = slot * c.e_max + k;
    const ParentInfo pi = b.pinfo[pk];
    const SlotPlan* sp = b.slots + pk * c.max_slots;
    const bool fathom = pi.fathom != 0;
    const uint64_t S = fathom ? 1 : c.S;
    const uint64_t r = best.e / S, i = best.e % S;
    for (int v = threadIdx.x; v < n; v += blockDim.x) {
      double hi;
      const double lo = child_bound(c, b, slot, k, r, v, sp, pi.count, hi);
      b.best_point[slot * c.n_max + v] =
          fathom ? lo : sample_value(d.kinds[v] != 0, lo, hi, (uint64_t)v, i, r, st->salt_base + k + 1);
    }
    if (threadIdx.x == 0) {
      st->gub = best.value;
      st->best = best;
      st->have_best = 1;
    }
  }
  __syncthreads();
  const double gub = st->gub;

  // (2) verdict counts and (3) append kept children after the remaining pool
  const uint32_t remaining = (uint32_t)st->remaining;
  if (threadIdx.x == 0) running = 0;
  __syncthreads();
  unsigned long long l_dup = 0, l_inf = 0, l_dom = 0, l_kept = 0, l_smp = 0, l_valid = 0, l_excl = 0, l_cert = 0;
  for (uint32_t cb = 0; cb < nch; cb += kMiThreads) {
    const uint32_t local = cb + threadIdx.x;
    bool keep = false;
    if (local < nch) {
      const uint8_t raw = b.cstate[cbase + local];
      const uint64_t k = local >> c.log2C, r = local & ((1ULL << c.log2C) - 1ULL);
      const ParentInfo pi = b.pinfo[slot * c.e_max + k];
      if (!pi.fathom && r < pi.nreg) {
        const uint8_t s8 = raw & 0x7f;
        if (s8 != kChildNone) {
          if (c.sample_all || s8 == kChildEligible) ++l_smp;
          if (s8 != kChildDuplicate) {
            ++l_valid;
            if (s8 == kChildInfeasible || s8 == kChildDominated) ++l_excl;
            if (raw & kCertifiedBit) ++l_cert;
          }
          if (s8 == kChildDuplicate) ++l_dup;
          else if (s8 == kChildInfeasible) ++l_inf;
          else if (s8 == kChildDominated || s8 == kChildScreened || b.clb[cbase + local] > gub) ++l_dom;
          else {
            ++l_kept;
            keep = true;
          }
        }
      }
    }
    int total;
    const int rank = block_rank(keep, total);
    if (keep) {
      const uint32_t at = remaining + running + (uint32_t)rank;
      const uint64_t k = local >> c.log2C, r = local & ((1ULL << c.log2C) - 1ULL);
      const size_t pk = slot * c.e_max + k;
      const ParentInfo pi = b.pinfo[pk];
      const SlotPlan* sp = b.slots + pk * c.max_slots;
      for (int v = 0; v < n; ++v) {
        double hi;
        const double lo = child_bound(c, b, slot, k, r, v, sp, pi.count, hi);
        b.lo[plane(c, slot, v) + at] = lo;
        b.hi[plane(c, slot, v) + at] = hi;
      }
      b.lb[(size_t)slot * c.P + at] = b.clb[cbase + local];
      b.depth[(size_t)slot * c.P + at] = b.pdepth[pk] + 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) running += (uint32_t)total;
    __syncthreads();
  }
  atomicAdd(&cnt[0], l_dup);
  atomicAdd(&cnt[1], l_inf);
  atomicAdd(&cnt[2], l_dom);
  atomicAdd(&cnt[3], l_kept);
  atomicAdd(&cnt[4], l_smp);
  atomicAdd(&cnt[5], l_valid);
  atomicAdd(&cnt[6], l_excl);
  atomicAdd(&cnt[7], l_cert);
  __syncthreads();
  const uint32_t new_size = remaining + (uint32_t)cnt[3];

  // (4) above the cap: keep the `cap` best, fold the rest into the floor
  uint32_t final_size = new_size;
  if (new_size > c.cap) {
    const SortSmem s = sort_smem(smem_raw);
    const double* lbp = b.lb + (size_t)slot * c.P;
    mark_smallest(lbp, new_size, (uint32_t)c.cap, s);
    unsigned long long via = 0, dom = 0;
    uint64_t mk = ~0ULL;
    for (uint32_t i = threadIdx.x; i < new_size; i += blockDim.x) {
      if (s.flag[i]) continue;
      const double x = lbp[i];
      if (x <= gub) {
        ++via;
        const uint64_t kk = lb_key(x);
        mk = kk < mk ? kk : mk;
      } else {
        ++dom;
      }
    }
    atomicAdd(&cnt[8], via);
    atomicAdd(&cnt[9], dom);
    if (mk != ~0ULL) atomicMin(&min_key_s, (unsigned long long)mk);
    __syncthreads();
    compact_pool(c, b, slot, new_size, n, s.flag, s.pos, &running);
    final_size = (uint32_t)c.cap;
  }

  // (5) pool minimum and viable count
  uint64_t mk = ~0ULL;
  unsigned long long viable = 0;
  const double* lbp = b.lb + (size_t)slot * c.P;
  for (uint32_t i = threadIdx.x; i < final_size; i += blockDim.x) {
    const uint64_t kk = lb_key(lbp[i]);
    mk = kk < mk ? kk : mk;
    if (lbp[i] <= gub) ++viable;
  }
  __shared__ unsigned long long pool_min_s, viable_s;
  if (threadIdx.x == 0) {
    pool_min_s = ~0ULL;
    viable_s = 0;
  }
  __syncthreads();
  atomicMin(&pool_min_s, (unsigned long long)mk);
  atomicAdd(&viable_s, viable);
  __syncthreads();
  if (threadIdx.x == 0) {
    cmn_counters& ct = st->counters;
    ct.pruned_duplicate += cnt[0];
    ct.pruned_infeasible += cnt[1];
    ct.pruned_dominated += cnt[2];
    ct.enqueued += cnt[3];
    ct.sampled += cnt[4] * c.S;
    if (c.precision == CMN_PRECISION_FP32_SCREEN) {
      if (st->use_screen) ct.screened_fp32 += cnt[5];
      ct.certified_fp64 += cnt[7];
      if (cnt[5] > 0) {
        const unsigned long long x = st->use_screen ? cnt[5] - cnt[7] : cnt[6];
        st->use_screen = (x * 4 >= cnt[5]) ? 1 : 0;
      }
    } else if (c.precision == CMN_PRECISION_FP32_LAZY) {
      ct.screened_fp32 += cnt[5];   // every valid child is bounded in FP32
      ct.certified_fp64 += cnt[7];  // the band's FP64 pass (the parents: batch_drop_kernel)
    } else {
      ct.certified_fp64 += cnt[5];
    }
    ct.dropped_viable += cnt[8];
    ct.dropped_dominated += cnt[9];
    if (min_key_s < st->dropped_min_key) st->dropped_min_key = min_key_s;
    if (st->dropped_min_key != ~0ULL) st->dropped_lb_min = key_to_lb_b(st->dropped_min_key);
    st->pool_size = final_size;
    st->pool_min_key = pool_min_s;
    st->viable = viable_s;
    if (final_size > ct.peak_frontier) ct.peak_frontier = final_size;
  }
}

// ---------------------------------------------------------------------
// certify list (children the screen left open), stable over (slot, child)
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(512) batch_list_count_kernel(const BatchCfg c, const BatchBufs b)
{
  const uint64_t total = c.K * c.child_stride;
  const uint64_t i = (uint64_t)blockIdx.x * 512 + threadIdx.x;
  bool f = false;
  if (i < total) {
    const uint64_t slot = i / c.child_stride, k = (i % c.child_stride) >> c.log2C;
    f = k < b.st[slot].n_parents && b.cstate[i] == kChildScreened;
  }
  const int cnt = __syncthreads_count(f);
  if (threadIdx.x == 0) b.block_counts[blockIdx.x] = (uint32_t)cnt;
}

__global__ void batch_list_scan_kernel(const BatchCfg c, const BatchBufs b)
{
  __shared__ uint64_t carry;
  __shared__ uint32_t wsum[32];
  const uint64_t nblocks = (c.K * c.child_stride + 511) / 512;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (uint64_t base = 0; base < nblocks; base += blockDim.x) {
    const uint64_t i = base + threadIdx.x;
    const uint32_t v = i < nblocks ? b.block_counts[i] : 0;
    uint32_t x = v;
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
      uint32_t sw = lane < (int)(blockDim.x / 32) ? wsum[lane] : 0;
      for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, sw, off);
        if (lane >= off) sw += y;
      }
      wsum[lane] = sw;
    }
    __syncthreads();
    const uint64_t cy = carry;
    if (i < nblocks) b.block_offsets[i] = (uint32_t)(cy + (wid > 0 ? wsum[wid - 1] : 0) + x - v);
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = cy + wsum[blockDim.x / 32 - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) *b.list_count = carry;
}

__global__ void __launch_bounds__(512) batch_list_scatter_kernel(const BatchCfg c, const BatchBufs b)
{
  __shared__ int wt[16];
  const uint64_t total = c.K * c.child_stride;
  const uint64_t i = (uint64_t)blockIdx.x * 512 + threadIdx.x;
  bool f = false;
  if (i < total) {
    const uint64_t slot = i / c.child_stride, k = (i % c.child_stride) >> c.log2C;
    f = k < b.st[slot].n_parents && b.cstate[i] == kChildScreened;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned ball = __ballot_sync(0xffffffffu, f);
  if (lane == 0) wt[wid] = __popc(ball);
  __syncthreads();
  int before = 0;
  for (int w = 0; w < wid; ++w) before += wt[w];
  if (f) b.list[b.block_offsets[blockIdx.x] + before + __popc(ball & ((1u << lane) - 1u))] = (uint32_t)i;
}

// ---------------------------------------------------------------------
size_t batch_eval_smem(const BatchCfg& c, bool fp32)
{
  // FP32 (the screen, the lazy bound): slot parts after the split variables
  return ((fp32 ? 8 : 16) * (size_t)(c.slots_max + c.max_slots) + (fp32 ? 8 : 4) * (size_t)c.max_slots) *
         kEvalThreads;
}

size_t batch_sample_smem(const BatchCfg& c) { return 8 * (size_t)(c.n_max + c.slots_max) * kEvalThreads; }

// the lazy form's FP32 screen: one FP32 point column per thread
static size_t batch_screen_smem(const BatchCfg& c) { return 4 * (size_t)(c.n_max + c.slots_max) * kEvalThreads; }

// the lazy form's verdict: program slots (FP64 intervals) per thread
static size_t batch_verdict_smem(const BatchCfg& c) { return 16 * (size_t)c.slots_max * kEvalThreads; }

int batch_eval_occupancy(const BatchCfg& c, bool fp32)
{
  int n = 0;
  if (fp32)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_eval_kernel<float, 2>, kEvalThreads,
                                                  batch_eval_smem(c, true));
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_eval_kernel<double, 1>, kEvalThreads,
                                                  batch_eval_smem(c, false));
  return n;
}

int batch_sample_occupancy(const BatchCfg& c)
{
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_sample_kernel, kEvalThreads, batch_sample_smem(c));
  return n;
}

static size_t sort_smem_bytes() { return (size_t)kMiSortMax * (8 + 4 + 1); }

cudaError_t set_batch_kernel_attributes(int max_smem)
{
  const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, batch_select_kernel);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(batch_select_kernel, at, max_smem - (int)fa.sharedSizeBytes);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, batch_finish_kernel);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(batch_finish_kernel, at, max_smem - (int)fa.sharedSizeBytes);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(batch_eval_kernel<double, 1>, at, max_smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(batch_eval_kernel<float, 2>, at, max_smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(batch_eval_kernel<double, 3>, at, max_smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(batch_sample_kernel, at, max_smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(batch_eval_kernel<float, 5>, at, max_smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(batch_verdict_kernel, at, max_smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(batch_screen_kernel, at, max_smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(batch_chunk_kernel, at, max_smem);
  return e;
}

cudaError_t batch_init_slot(const BatchCfg& c, const BatchBufs& b, uint64_t slot, double gub0, cudaStream_t s)
{
  batch_init_slot_kernel<<<1, 128, 0, s>>>(c, b, slot, gub0);
  return cudaGetLastError();
}

static void mark(const cudaEvent_t* marks, int i, cudaStream_t s)
{
  if (marks) cudaEventRecordWithFlags(marks[i], s, cudaEventRecordExternal);
}

// Blocks for a grid-stride launch of `kernel` over `items` threads' worth
// of work: as many as stay resident on every SM, no more than the items
// need.
template <typename Kernel>
static int resident_grid(Kernel kernel, size_t smem, uint64_t items)
{
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, kEvalThreads, smem) != cudaSuccess) {
    (void)cudaGetLastError();
    n = 1;
  }
  const uint64_t need = (items + kEvalThreads - 1) / kEvalThreads;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)sm_count() * (uint64_t)std::max(1, n)));
}

BatchGrids batch_grids(const BatchCfg& c, int eval_grid)
{
  BatchGrids g;
  g.eval = eval_grid;
  g.inc_common = resident_grid(batch_inc_common_kernel, 0, c.K * (uint64_t)c.seg_max * c.e_max);
  g.inc_parts = resident_grid(batch_inc_parts_kernel, 0, c.K * (c.e_max << c.log2C));
  g.screen = resident_grid(batch_screen_kernel, batch_screen_smem(c), c.K * c.child_stride);
  return g;
}

cudaError_t batch_iteration(const BatchCfg& c, const BatchBufs& b, const BatchGrids& grids, cudaStream_t s,
                            const cudaEvent_t* marks)
{
  const int eval_grid = grids.eval;
  mark(marks, 0, s);
  const int kb = (int)((c.K + 255) / 256);
  batch_begin_kernel<<<kb, 256, 0, s>>>(c, b);
  batch_select_kernel<<<(int)c.K, kMiThreads, sort_smem_bytes(), s>>>(c, b);
  const uint64_t np = c.K * c.e_max;
  batch_branch_kernel<<<(int)((np + 127) / 128), 128, 0, s>>>(c, b);
  batch_live_kernel<<<1, 1024, 0, s>>>(c, b);
  mark(marks, 1, s);
  const bool fp32 = c.precision == CMN_PRECISION_FP32_SCREEN;
  const bool lazy = c.precision == CMN_PRECISION_FP32_LAZY;
  if (lazy) {
    // the FP64 verdict of the staged parents, the drop, then the FP32 child
    // bounds with each parent's certified bound folded in, and the band's
    // FP64 pass (the single-instance solver runs the verdict beside the
    // bounds; the states and counters are the same)
    batch_verdict_kernel<<<eval_grid, kEvalThreads, batch_verdict_smem(c), s>>>(c, b);
    const uint64_t np2 = c.K * c.e_max;
    batch_drop_kernel<<<(int)((np2 + 255) / 256), 256, 0, s>>>(c, b);
    batch_inc_common_kernel<<<grids.inc_common, kEvalThreads, 0, s>>>(c, b);
    batch_inc_parts_kernel<<<grids.inc_parts, kEvalThreads, 0, s>>>(c, b);
    batch_eval_kernel<float, 5><<<eval_grid, kEvalThreads, batch_eval_smem(c, true), s>>>(c, b);
    const int lg = (int)((c.K * c.child_stride + 511) / 512);
    batch_list_count_kernel<<<lg, 512, 0, s>>>(c, b);
    batch_list_scan_kernel<<<1, 1024, 0, s>>>(c, b);
    batch_list_scatter_kernel<<<lg, 512, 0, s>>>(c, b);
    batch_eval_kernel<double, 3><<<eval_grid, kEvalThreads, batch_eval_smem(c, false), s>>>(c, b);
    mark(marks, 2, s);
    batch_screen_kernel<<<grids.screen, kEvalThreads, batch_screen_smem(c), s>>>(c, b);
    batch_chunk_kernel<<<eval_grid, kEvalThreads, batch_sample_smem(c), s>>>(c, b);
    mark(marks, 3, s);
    batch_finish_kernel<<<(int)c.K, kMiThreads, sort_smem_bytes(), s>>>(c, b);
    mark(marks, 4, s);
    return cudaGetLastError();
  }
  if (fp32) {
    batch_eval_kernel<float, 2><<<eval_grid, kEvalThreads, batch_eval_smem(c, true), s>>>(c, b);
    const int lg = (int)((c.K * c.child_stride + 511) / 512);
    batch_list_count_kernel<<<lg, 512, 0, s>>>(c, b);
    batch_list_scan_kernel<<<1, 1024, 0, s>>>(c, b);
    batch_list_scatter_kernel<<<lg, 512, 0, s>>>(c, b);
    batch_eval_kernel<double, 3><<<eval_grid, kEvalThreads, batch_eval_smem(c, false), s>>>(c, b);
  } else {
    batch_eval_kernel<double, 1><<<eval_grid, kEvalThreads, batch_eval_smem(c, false), s>>>(c, b);
  }
  mark(marks, 2, s);
  batch_sample_kernel<<<eval_grid, kEvalThreads, batch_sample_smem(c), s>>>(c, b);
  mark(marks, 3, s);
  batch_finish_kernel<<<(int)c.K, kMiThreads, sort_smem_bytes(), s>>>(c, b);
  mark(marks, 4, s);
  return cudaGetLastError();
}

}  // namespace cmn
