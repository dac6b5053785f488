// search_kernels.cu -- the device half of the batched branch-and-bound:
// parent selection, the branching policy, prune + compaction (c) and the
// box pool with eviction (d).  Every kernel reads the iteration's sizes
// from SolverDev, so one captured graph replays any iteration.
//
// The reference keeps its frontier on the host: a binary heap of 40-byte
// nodes and a refcounted box history (search/frontier.hpp:152-338,
// search/history.hpp:20-137), pruned by an O(N) host loop after every
// launch (search/driver.hpp:303-352).  Here the frontier is a pool of SoA
// boxes in HBM; selection is a radix select on the lower-bound keys, and
// every compaction is a stable, deterministic block scan.
#include <cfloat>
#include <cstdint>

#include "eval_core.cuh"
#include "launch.hpp"
#include "policy.cuh"
#include "search.hpp"

namespace cmn {

__device__ __forceinline__ bool gap_closed_dev(double gub, double bound, double tol)
{
  return __dsub_rn(gub, bound) <= __dmul_rn(tol, fmax(1.0, fabs(gub)));
}

__device__ __forceinline__ double key_to_lb(uint64_t k)
{
  const uint64_t u = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
  return __longlong_as_double((long long)u);
}

// ---------------------------------------------------------------------
// init / begin / finish
// ---------------------------------------------------------------------
__global__ void init_kernel(const SolverCfg cfg, const SolverBufs b, const double* __restrict__ root_lb,
                            const double* __restrict__ root_ub, double gub0)
{
  const int t = threadIdx.x + blockIdx.x * blockDim.x;
  for (int v = t; v < cfg.n_vars; v += blockDim.x * gridDim.x) {  // the root box in store slot 0
    b.lo[v] = root_lb[v];
    b.hi[v] = root_ub[v];
  }
  if (t == 0) {
    SolverDev* d = b.dev;
    memset(d, 0, sizeof(SolverDev));
    d->gub = gub0;
    d->glb = -DBL_MAX;
    d->dropped_lb_min = INFINITY;
    d->dropped_min_key = ~0ULL;
    b.lb[0][0] = -DBL_MAX;
    b.slot[0][0] = 0;
    b.depth[0] = 0;
    d->free_top = cfg.pstride - 1;
    d->pool_size = 1;
    d->pool_min_key = lb_key(-DBL_MAX);
    d->pool_max_key = lb_key(-DBL_MAX);
    d->parity = 0;
    d->use_screen = 1;
    d->counters.peak_frontier = 1;
  }
}

// every store slot but the root's is free; pops take the low slots first
__global__ void free_init_kernel(const SolverCfg cfg, const SolverBufs b)
{
  const uint64_t n = cfg.pstride - 1;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    b.free_slots[i] = (uint32_t)(cfg.pstride - 1 - i);
}

// Top of the loop of search/driver.hpp:221-233: convergence of the least
// pending lower bound, the expansion budget, and this iteration's size.
__global__ void begin_kernel(const SolverCfg cfg, const SolverBufs b, int require_staged)
{
  SolverDev* d = b.dev;
  d->improved = 0;  // an iteration after the stop must not rewrite the witness
  if (d->done) return;
  const uint64_t L = d->pool_size;
  if (L == 0) {
    d->done = 1;
    return;
  }
  const double m = key_to_lb(d->pool_min_key);
  if (gap_closed_dev(d->gub, m, cfg.tolerance)) {
    d->converged = 1;
    d->done = 1;
    return;
  }
  d->glb = m;
  if (d->expansions >= cfg.iter_limit || (cfg.batch_iter_limit && d->iterations >= cfg.batch_iter_limit)) {
    d->done = 1;
    return;
  }
  uint64_t E = L < cfg.e_max ? L : cfg.e_max;
  const uint64_t left = cfg.iter_limit - d->expansions;
  if (E > left) E = left;
  // the previous iteration staged the E best entries of this pool already
  d->skip_select = (d->pre_valid && d->pre_k == E) ? 1u : 0u;
  if (require_staged && !d->skip_select) d->error = 1;
  d->pre_valid = 0;
  d->pre_k = 0;
  d->pre_count = 0;
  d->iterations += 1;
  d->n_parents = E;
  d->n_children = E << cfg.log2C;
  d->salt_base = d->expansions;
  d->expansions += E;
  d->certify_count = 0;
  d->iter_valid = 0;
  d->iter_excluded = 0;
  d->remaining = 0;
  d->kept = 0;
  d->new_size = 0;
  d->child_min_key = ~0ULL;
  d->child_max_key = 0;
  d->extent = 0;
  d->survivors = 0;
  d->evict = 0;
  d->improved = 0;
  d->counters.iterations = d->iterations;
  d->counters.expansions = d->expansions;
}

// ---------------------------------------------------------------------
// radix select of the k-th smallest lower-bound key
// ---------------------------------------------------------------------
// which = 0: the current pool (n = pool_size; one target, k = n_parents),
//            the first iteration only
// which = 1: the current buffer after the children were appended behind
//            the pool (n = extent), alive entries only; target 0 the cap
//            (when evicting), target 1 the next iteration's parents

// one of the two pool buffers without indexing the parameter arrays by a
// runtime value (which would copy them to local memory)
template <class T>
__device__ __forceinline__ T* parity_buf(T* const (&a)[2], uint32_t p)
{
  return p ? a[1] : a[0];
}

__device__ __forceinline__ const double* pool_lb(const SolverBufs& b) { return parity_buf(b.lb, b.dev->parity); }
__device__ __forceinline__ uint8_t* pool_sel(const SolverBufs& b) { return parity_buf(b.sel, b.dev->parity); }

__device__ __forceinline__ uint64_t rs_n(const SolverDev* d, int which)
{
  return which == 0 ? d->pool_size : d->extent;
}

// Number of select targets of a pass: which = 0 selects this iteration's
// parents; which = 1 selects the entries that stay under the cap (target 0)
// and, among them, the next iteration's parents (target 1).
__device__ __forceinline__ int n_targets(int which) { return which == 0 ? 1 : 2; }

__device__ __forceinline__ bool target_live(const RadixState& r)
{
  return r.active && !r.settled && r.bits_left != 0;
}

__global__ void radix_init_kernel(const SolverCfg cfg, const SolverBufs b, int which)
{
  SolverDev* d = b.dev;
  for (int t = 0; t < n_targets(which); ++t) {
    RadixState* rs = b.radix + t;
    uint64_t k;
    bool active;
    if (which == 0) {
      k = d->n_parents;
      active = !d->done && !d->skip_select && k < d->pool_size;
    } else if (t == 0) {
      k = cfg.cap;
      active = !d->done && d->evict && k < d->new_size;
    } else {
      k = d->pre_k;
      active = !d->done && k > 0 && k < d->new_size;
    }
    for (int i = threadIdx.x; i < kRadixBins; i += blockDim.x) rs->hist[i] = 0;
    if (threadIdx.x == 0) {
      const uint64_t lo = which == 0 ? d->pool_min_key : d->evict_lo_key;
      const uint64_t hi = which == 0 ? d->pool_max_key : d->evict_hi_key;
      const int common = lo <= hi ? ((lo ^ hi) == 0 ? 64 : __clzll((long long)(lo ^ hi))) : 0;
      const uint64_t top = common == 0 ? 0 : (~0ULL << (64 - common));
      rs->prefix = lo & top;
      rs->mask = top;
      rs->k = k;
      rs->less = 0;
      rs->active = active ? 1u : 0u;
      rs->settled = 0;
      rs->rank = active ? 1u : 0u;
      rs->bits_left = (uint32_t)(64 - common);
    }
  }
}

// One digit's histogram per live target over the entries inside its
// bucket, in one read of the keys. Each thread counts a run of equal bins
// in registers and adds it to the block's shared histogram only when the
// bin changes: converging lower bounds share most leading digits, so a pass
// makes few shared-memory atomics instead of one per entry on one address.
__global__ void radix_hist_kernel(const SolverCfg cfg, const SolverBufs b, int which)
{
  __shared__ uint32_t h[2][kRadixBins];
  const int T = n_targets(which);
  bool go[2] = {false, false};
  int shift[2] = {0, 0}, nb[2] = {1, 1};
  uint64_t prefix[2] = {0, 0}, mask[2] = {0, 0};
  for (int t = 0; t < T; ++t) {
    const RadixState& r = b.radix[t];
    go[t] = target_live(r);
    if (!go[t]) continue;
    const int bits = r.bits_left < (uint32_t)kRadixBits ? (int)r.bits_left : kRadixBits;
    shift[t] = (int)r.bits_left - bits;
    nb[t] = 1 << bits;
    prefix[t] = r.prefix;
    mask[t] = r.mask;
  }
  if (!go[0] && !go[1]) return;
  // while both targets sit in the same bucket (the first pass of a rebuild)
  // their histograms are the same: count once, add to both
  const bool same = go[0] && go[1] && prefix[0] == prefix[1] && mask[0] == mask[1] && shift[0] == shift[1];
  const bool count1 = go[1] && !same;
  const uint64_t n = rs_n(b.dev, which);
  if ((uint64_t)blockIdx.x * blockDim.x >= n) return;
  for (int t = 0; t < 2; ++t)
    for (int i = threadIdx.x; i < kRadixBins; i += blockDim.x) h[t][i] = 0;
  __syncthreads();
  const uint64_t* __restrict__ lb = reinterpret_cast<const uint64_t*>(pool_lb(b));
  const uint8_t* __restrict__ sel = which == 1 ? pool_sel(b) : nullptr;
  const int lane = threadIdx.x & 31;
  // each warp takes chunks of 32 x kHistUnroll consecutive entries and
  // issues all their loads before it bins them
  constexpr int kChunk = 32 * kHistUnroll;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x / 32);
  uint32_t run_bin[2] = {0, 0}, run[2] = {0, 0};
  for (uint64_t c = (uint64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); c * kChunk < n; c += warps) {
    uint64_t x[kHistUnroll];
    bool in[kHistUnroll];
#pragma unroll
    for (int u = 0; u < kHistUnroll; ++u) {
      const uint64_t i = c * kChunk + (uint64_t)u * 32 + lane;
      in[u] = i < n;
      x[u] = in[u] ? lb[i] : 0;
      if (sel != nullptr && in[u]) in[u] = sel[i] == kSelAlive;
    }
#pragma unroll
    for (int u = 0; u < kHistUnroll; ++u) {
      if (!in[u]) continue;
      const uint64_t key = bits_key(x[u]);
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        if (!(t == 0 ? go[0] : count1) || (key & mask[t]) != prefix[t]) continue;
        const uint32_t bin = (uint32_t)(key >> shift[t]) & (uint32_t)(nb[t] - 1);
        if (bin != run_bin[t]) {
          if (run[t]) atomicAdd(&h[t][run_bin[t]], run[t]);
          run_bin[t] = bin;
          run[t] = 0;
        }
        ++run[t];
      }
    }
  }
  for (int t = 0; t < 2; ++t)
    if (run[t]) atomicAdd(&h[t][run_bin[t]], run[t]);
  __syncthreads();
  for (int t = 0; t < T; ++t) {
    if (!go[t]) continue;
    const uint32_t* src = (t == 1 && same) ? h[0] : h[t];
    for (int i = threadIdx.x; i < nb[t]; i += blockDim.x)
      if (src[i]) atomicAdd(&b.radix[t].hist[i], src[i]);
  }
  (void)cfg;
}

// Picks the digit whose bin holds the k-th entry: a block scan over the
// bins (two per thread); block t serves target t. When the entries up to
// and including that bin are exactly k, the bin is taken whole and the
// search stops.
__global__ void __launch_bounds__(kPickThreads) radix_pick_kernel(const SolverBufs b)
{
  __shared__ uint64_t warp_sum[kPickThreads / 32];
  __shared__ int pick_d;
  __shared__ uint64_t pick_cum, pick_cnt;
  RadixState* rs = b.radix + blockIdx.x;
  if (!target_live(*rs)) return;
  const int bits = rs->bits_left < (uint32_t)kRadixBits ? (int)rs->bits_left : kRadixBits;
  const int shift = (int)rs->bits_left - bits;
  const int nb = 1 << bits;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const int b0 = 2 * t;
  const uint32_t c0 = b0 < nb ? rs->hist[b0] : 0u;
  const uint32_t c1 = b0 + 1 < nb ? rs->hist[b0 + 1] : 0u;
  if (t == 0) pick_d = -1;
  uint64_t x = (uint64_t)c0 + c1;
  for (int off = 1; off < 32; off <<= 1) {
    const uint64_t y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) warp_sum[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint64_t s = lane < kPickThreads / 32 ? warp_sum[lane] : 0;
    for (int off = 1; off < 32; off <<= 1) {
      const uint64_t y = __shfl_up_sync(0xffffffffu, s, off);
      if (lane >= off) s += y;
    }
    if (lane < kPickThreads / 32) warp_sum[lane] = s;  // inclusive
  }
  __syncthreads();
  const uint64_t incl = x + (wid > 0 ? warp_sum[wid - 1] : 0);
  const uint64_t excl = incl - c0 - c1;
  const uint64_t k = rs->k;
  if (excl < k && k <= incl) {  // exactly one thread holds the k-th entry
    if (excl + c0 >= k) {
      pick_d = b0;
      pick_cum = excl;
      pick_cnt = c0;
    } else {
      pick_d = b0 + 1;
      pick_cum = excl + c0;
      pick_cnt = c1;
    }
  }
  __syncthreads();
  if (b0 < nb) rs->hist[b0] = 0;
  if (b0 + 1 < nb) rs->hist[b0 + 1] = 0;
  if (t != 0) return;
  if (pick_d < 0) {  // fewer entries in the bucket than its rank: never expected
    b.dev->error = 1;
    rs->settled = 1;
    rs->rank = 0;
    return;
  }
  rs->less += pick_cum;
  rs->k = k - pick_cum;
  rs->prefix |= (uint64_t)pick_d << shift;
  rs->mask |= ((uint64_t)(nb - 1)) << shift;
  rs->bits_left = (uint32_t)shift;
  if (pick_cum + pick_cnt == k) {
    rs->settled = 1;
    rs->rank = 0;
  }
}

// ---------------------------------------------------------------------
// stable compaction: count -> scan -> scatter over tiles of kScanTile
// items; item j of thread t in tile T is T * kScanTile + j * kScanBlock + t,
// so every pass reads whole cache lines and keeps kScanItems loads in flight
// per thread.
// ---------------------------------------------------------------------
// first item of this thread in its block's tile, read once per kernel (the
// special registers are slow to re-read)
__device__ __forceinline__ uint64_t tile_first() { return (uint64_t)blockIdx.x * kScanTile + threadIdx.x; }

__device__ __forceinline__ uint64_t tile_item(uint64_t t0, int j) { return t0 + (uint64_t)j * kScanBlock; }

// Ranks of the flagged items of this block's tile in item order (for every
// item: the flagged items before it); returns the tile's flagged count. One
// call per kernel and table slot `S`.
template <int S = 0>
__device__ __forceinline__ int tile_ranks(const bool (&f)[kScanItems], int (&rank)[kScanItems])
{
  constexpr int kWarps = kScanBlock / 32;
  constexpr int kPer = kScanItems * kWarps / 32;  // table entries per lane of warp 0
  __shared__ int tab[kScanItems * kWarps];
  __shared__ int tile_total;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned ball[kScanItems];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    ball[j] = __ballot_sync(0xffffffffu, f[j]);
    if (lane == 0) tab[j * kWarps + wid] = __popc(ball[j]);
  }
  __syncthreads();
  if (wid == 0) {
    int v[kPer], sum = 0;
#pragma unroll
    for (int e = 0; e < kPer; ++e) {
      v[e] = tab[lane * kPer + e];
      sum += v[e];
    }
    int x = sum;
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x += y;
    }
    int run = x - sum;
#pragma unroll
    for (int e = 0; e < kPer; ++e) {
      tab[lane * kPer + e] = run;
      run += v[e];
    }
    if (lane == 31) tile_total = x;
  }
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) rank[j] = tab[j * kWarps + wid] + __popc(ball[j] & lt);
  return tile_total;
}

// tile_ranks of two flag sets with one pair of barriers
__device__ __forceinline__ void tile_ranks2(const bool (&f)[kScanItems], const bool (&g)[kScanItems],
                                            int (&rf)[kScanItems], int (&rg)[kScanItems])
{
  constexpr int kWarps = kScanBlock / 32;
  constexpr int kPer = kScanItems * kWarps / 32;
  __shared__ int tab[2][kScanItems * kWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned bf[kScanItems], bg[kScanItems];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    bf[j] = __ballot_sync(0xffffffffu, f[j]);
    bg[j] = __ballot_sync(0xffffffffu, g[j]);
    if (lane == 0) {
      tab[0][j * kWarps + wid] = __popc(bf[j]);
      tab[1][j * kWarps + wid] = __popc(bg[j]);
    }
  }
  __syncthreads();
  if (wid < 2) {  // warp 0 scans the first table, warp 1 the second
    int* t = tab[wid];
    int v[kPer], sum = 0;
#pragma unroll
    for (int e = 0; e < kPer; ++e) {
      v[e] = t[lane * kPer + e];
      sum += v[e];
    }
    int x = sum;
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x += y;
    }
    int run = x - sum;
#pragma unroll
    for (int e = 0; e < kPer; ++e) {
      t[lane * kPer + e] = run;
      run += v[e];
    }
  }
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    rf[j] = tab[0][j * kWarps + wid] + __popc(bf[j] & lt);
    rg[j] = tab[1][j * kWarps + wid] + __popc(bg[j] & lt);
  }
}

__device__ __forceinline__ uint64_t warp_min_u64(uint64_t m)
{
  for (int off = 16; off > 0; off >>= 1) {
    const uint64_t o = __shfl_xor_sync(0xffffffffu, m, off);
    m = o < m ? o : m;
  }
  return m;
}

__device__ __forceinline__ uint64_t warp_max_u64(uint64_t m)
{
  for (int off = 16; off > 0; off >>= 1) {
    const uint64_t o = __shfl_xor_sync(0xffffffffu, m, off);
    m = o > m ? o : m;
  }
  return m;
}

// Sum of `c` over the block (one call per kernel and slot `S`).
template <int S = 0>
__device__ __forceinline__ int tile_count(int c)
{
  __shared__ int tot;
  if (threadIdx.x == 0) tot = 0;
  __syncthreads();
  const int w = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0 && w) atomicAdd(&tot, w);
  __syncthreads();
  return tot;
}

// Block totals of per-thread counters, for thread 0 (one global atomic per
// block instead of one per warp: same-address atomics serialise in L2).
// Every thread of the block calls it.
template <int N>
__device__ __forceinline__ void block_sum(unsigned long long (&v)[N])
{
  __shared__ unsigned long long acc[N];
  if (threadIdx.x < N) acc[threadIdx.x] = 0;
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; ++k) {
    unsigned long long x = v[k];
    for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
    if ((threadIdx.x & 31) == 0 && x) atomicAdd(&acc[k], x);
  }
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = acc[k];
}

// Block maximum of `m`, for thread 0. Every thread of the block calls it.
__device__ __forceinline__ uint64_t block_max(uint64_t m)
{
  __shared__ unsigned long long acc;
  if (threadIdx.x == 0) acc = 0;
  __syncthreads();
  for (int off = 16; off > 0; off >>= 1) {
    const uint64_t o = __shfl_down_sync(0xffffffffu, m, off);
    m = o > m ? o : m;
  }
  if ((threadIdx.x & 31) == 0 && m != 0) atomicMax(&acc, (unsigned long long)m);
  __syncthreads();
  return acc;
}

// Block minimum of `m`, for thread 0. Every thread of the block calls it.
__device__ __forceinline__ uint64_t block_min(uint64_t m)
{
  __shared__ unsigned long long acc;
  if (threadIdx.x == 0) acc = ~0ULL;
  __syncthreads();
  for (int off = 16; off > 0; off >>= 1) {
    const uint64_t o = __shfl_down_sync(0xffffffffu, m, off);
    m = o < m ? o : m;
  }
  if ((threadIdx.x & 31) == 0 && m != ~0ULL) atomicMin(&acc, (unsigned long long)m);
  __syncthreads();
  return acc;
}

// Exclusive scan of the tile counts of `*n_items` items (one block of 1024
// threads); writes the total to *total_out when given.
__global__ void __launch_bounds__(1024) scan_kernel(const uint32_t* __restrict__ counts,
                                                    uint32_t* __restrict__ offsets,
                                                    const uint64_t* __restrict__ n_items,
                                                    uint64_t* __restrict__ total_out,
                                                    const uint32_t* __restrict__ active,
                                                    const uint32_t* __restrict__ skip,
                                                    const uint32_t* __restrict__ done)
{
  __shared__ uint64_t warp_sum[32];
  if (*done || (skip && *skip)) return;
  if (active && !*active) {
    if (threadIdx.x == 0 && total_out) *total_out = 0;
    return;
  }
  const uint64_t n = *n_items;
  const uint64_t nblocks = (n + kScanTile - 1) / kScanTile;
  // each thread sums a run of consecutive counts, the block scans the sums
  // once, and each thread writes its run's offsets: one pass, two barriers
  const uint32_t* src = counts;
  const uint64_t per = (nblocks + blockDim.x - 1) / blockDim.x;
  const uint64_t b0 = (uint64_t)threadIdx.x * per;
  const uint64_t b1 = b0 + per < nblocks ? b0 + per : nblocks;
  uint64_t sum = 0;
  for (uint64_t i = b0; i < b1; ++i) sum += src[i];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint64_t x = sum;
  for (int off = 1; off < 32; off <<= 1) {
    const uint64_t y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) warp_sum[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint64_t w = lane < (int)(blockDim.x / 32) ? warp_sum[lane] : 0;
    for (int off = 1; off < 32; off <<= 1) {
      const uint64_t y = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += y;
    }
    warp_sum[lane] = w;  // inclusive
  }
  __syncthreads();
  uint64_t run = x - sum + (wid > 0 ? warp_sum[wid - 1] : 0);
  if (threadIdx.x == blockDim.x - 1 && total_out) *total_out = run + sum;
  for (uint64_t i = b0; i < b1; ++i) {
    offsets[i] = (uint32_t)run;
    run += src[i];
  }
}

// ---- predicates / operations -----------------------------------------
struct KeptChild {
  SolverBufs b;
  __device__ uint64_t size() const { return b.dev->n_children; }
  __device__ bool operator()(uint64_t g) const
  {
    return b.cstate[g] == kChildEligible && !bits_lt(dbits(b.dev->gub), dbits(b.clb[g]));
  }
  __device__ bool skip() const { return b.dev->done != 0; }
};

struct ScreenedChild {
  SolverBufs b;
  __device__ uint64_t size() const { return b.dev->n_children; }
  __device__ bool operator()(uint64_t g) const { return b.cstate[g] == kChildScreened; }
  __device__ bool skip() const { return b.dev->done != 0; }
};

template <class P>
__global__ void __launch_bounds__(kScanBlock) count_kernel(const P pred, uint32_t* __restrict__ counts)
{
  const uint64_t t0 = tile_first();
  if (pred.skip()) return;
  const uint64_t n = pred.size();
  if ((uint64_t)blockIdx.x * kScanTile >= n) return;
  bool f[kScanItems];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint64_t i = tile_item(t0, j);
    f[j] = i < n && pred(i);
  }
  int c = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) c += f[j] ? 1 : 0;
  c = tile_count(c);
  if (threadIdx.x == 0) counts[blockIdx.x] = (uint32_t)c;
}

// Tile counts of the alive entries inside each ranked target's threshold
// bucket (target 0 into block_counts, target 1 into block_counts2).
__global__ void __launch_bounds__(kScanBlock) eq_count_kernel(const SolverCfg cfg, const SolverBufs b, int which)
{
  const uint64_t t0 = tile_first();
  const SolverDev* d = b.dev;
  const RadixState* rs = b.radix;
  const bool r0 = rs[0].rank != 0, r1 = which == 1 && rs[1].rank != 0;
  if (d->done || (!r0 && !r1)) return;
  const uint64_t n = rs_n(d, which);
  if ((uint64_t)blockIdx.x * kScanTile >= n) return;
  const uint64_t* __restrict__ lb = reinterpret_cast<const uint64_t*>(pool_lb(b));
  const uint8_t* __restrict__ sel = pool_sel(b);
  int c0 = 0, c1 = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint64_t i = tile_item(t0, j);
    if (i >= n || (which == 1 && sel[i] != kSelAlive)) continue;
    const uint64_t key = bits_key(lb[i]);
    c0 += (r0 && (key & rs[0].mask) == rs[0].prefix) ? 1 : 0;
    c1 += (r1 && (key & rs[1].mask) == rs[1].prefix) ? 1 : 0;
  }
  c0 = tile_count<0>(c0);
  c1 = tile_count<1>(c1);
  if (threadIdx.x == 0) {
    if (r0) b.block_counts[blockIdx.x] = (uint32_t)c0;
    if (r1) b.block_counts2[blockIdx.x] = (uint32_t)c1;
  }
  (void)cfg;
}

// The select decision of one target for one entry (`key` already masked).
struct TargetView {
  bool active, settled, ranked;
  uint64_t prefix, mask, k;
  __device__ explicit TargetView(const RadixState& r)
      : active(r.active != 0), settled(r.settled != 0), ranked(r.rank != 0), prefix(r.prefix), mask(r.mask), k(r.k)
  {
  }
  __device__ bool take(uint64_t key, bool eq, uint64_t eq_rank) const
  {
    if (!active) return true;
    if (eq) return settled || eq_rank < k;
    return (key & mask) < prefix;
  }
};

// Marks the k smallest (key, position) entries of each target: all keys
// below the threshold bucket, and the first `k` entries inside it in
// position order (all of them once the bucket is settled).
//   which = 0: marks this iteration's parents kSelParent and the others
//              kSelAlive, and writes the tile counts of the parents;
//   which = 1: marks alive entries outside the cap kSelEvicted (leaving the
//              parents' holes as they are) and folds them into the dropped
//              floor (search/budget.hpp:190-209); marks the next iteration's
//              parents among those that stay kSelNextParent; writes the tile
//              counts of the entries that stay and of the next parents.
__global__ void __launch_bounds__(kScanBlock, 2) mark_kernel(const SolverCfg cfg, const SolverBufs b, int which)
{
  const uint64_t t0 = tile_first();
  SolverDev* d = b.dev;
  if (which == 0 && d->skip_select) return;
  // the control words and the tile's entries are loaded together: a tile is
  // short, so a chain of dependent loads would set its duration
  const uint32_t done = d->done, skip = d->skip_select;
  const uint64_t n = rs_n(d, which);
  const uint64_t pre_k = d->pre_k;
  const uint64_t* __restrict__ lb = reinterpret_cast<const uint64_t*>(pool_lb(b));
  uint8_t* __restrict__ sel = pool_sel(b);
  uint64_t x[kScanItems];  // raw bits of the lower bounds
  uint8_t sv[kScanItems];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint64_t i = tile_item(t0, j);
    const bool inb = i < cfg.pstride;
    x[j] = inb ? lb[i] : 0;
    sv[j] = (which == 1 && inb) ? sel[i] : kSelAlive;
  }
  if (done || (which == 0 && skip)) return;
  if ((uint64_t)blockIdx.x * kScanTile >= n) return;
  const TargetView A(b.radix[0]);
  const bool pre = which == 1 && pre_k > 0;
  const TargetView B(b.radix[which == 1 ? 1 : 0]);
  const uint64_t gub = dbits(d->gub);
  bool alive[kScanItems], eqA[kScanItems], eqB[kScanItems];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    alive[j] = tile_item(t0, j) < n && sv[j] == kSelAlive;
    const uint64_t key = bits_key(x[j]);
    eqA[j] = A.active && alive[j] && (key & A.mask) == A.prefix;
    eqB[j] = pre && B.active && alive[j] && (key & B.mask) == B.prefix;
  }
  int rankA[kScanItems] = {}, rankB[kScanItems] = {};
  uint64_t baseA = 0, baseB = 0;
  if (A.ranked) {  // the same for the whole grid
    tile_ranks<0>(eqA, rankA);
    baseA = b.block_offsets[blockIdx.x];
  }
  if (pre && B.ranked) {
    tile_ranks<1>(eqB, rankB);
    baseB = b.block_offsets2[blockIdx.x];
  }
  int outA = 0, outB = 0;
  uint32_t viable = 0, dominated = 0;
  uint64_t mkey = ~0ULL;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    if (!alive[j]) continue;
    const uint64_t key = bits_key(x[j]);
    const bool ta = A.take(key, eqA[j], baseA + (uint64_t)rankA[j]);
    const bool tb = pre && ta && B.take(key, eqB[j], baseB + (uint64_t)rankB[j]);
    const uint64_t i = tile_item(t0, j);
    if (which == 0) {
      sel[i] = ta ? kSelParent : kSelAlive;
    } else if (!ta) {
      sel[i] = kSelEvicted;
      if (bits_le(x[j], gub)) {
        ++viable;
        mkey = key < mkey ? key : mkey;
      } else {
        ++dominated;
      }
    } else if (tb) {
      sel[i] = kSelNextParent;
    }
    outA += ta ? 1 : 0;
    outB += tb ? 1 : 0;
  }
  // the tile's counts and the eviction tallies, with one barrier
  struct Part {
    uint32_t a, b, viable, dominated;
    uint64_t mkey;
  };
  __shared__ Part part[kScanBlock / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  {
    const uint32_t pa = __reduce_add_sync(0xffffffffu, (uint32_t)outA);
    const uint32_t pb = __reduce_add_sync(0xffffffffu, (uint32_t)outB);
    const uint32_t pv = __reduce_add_sync(0xffffffffu, viable);
    const uint32_t pd = __reduce_add_sync(0xffffffffu, dominated);
    const uint64_t pm = warp_min_u64(mkey);
    if (lane == 0) part[wid] = Part{pa, pb, pv, pd, pm};
  }
  __syncthreads();
  if (wid != 0) return;
  const bool has = lane < kScanBlock / 32;
  const uint32_t ta = __reduce_add_sync(0xffffffffu, has ? part[lane].a : 0u);
  const uint32_t tb = __reduce_add_sync(0xffffffffu, has ? part[lane].b : 0u);
  const uint32_t tv = __reduce_add_sync(0xffffffffu, has ? part[lane].viable : 0u);
  const uint32_t td = __reduce_add_sync(0xffffffffu, has ? part[lane].dominated : 0u);
  const uint64_t tm = warp_min_u64(has ? part[lane].mkey : ~0ULL);
  if (lane != 0) return;
  b.block_counts[blockIdx.x] = ta;
  if (which == 1) b.block_counts2[blockIdx.x] = tb;
  if (which == 1 && A.active) {
    if (tv) atomicAdd((unsigned long long*)&d->counters.dropped_viable, (unsigned long long)tv);
    if (td) atomicAdd((unsigned long long*)&d->counters.dropped_dominated, (unsigned long long)td);
    if (tm != ~0ULL) atomicMin((unsigned long long*)&d->dropped_min_key, (unsigned long long)tm);
  }
}

// stage the box in store slot `s` as parent `pos` of the staging planes
__device__ __forceinline__ void stage_parent(const SolverCfg& cfg, const SolverBufs& b, uint64_t s, uint64_t pos)
{
  if (pos >= cfg.e_max) {  // more marks than parents: never written, flagged
    b.dev->error = 1;
    return;
  }
  // loads in groups ahead of the stores (the pointers do not alias)
  const double* __restrict__ slo = b.lo + s * (uint64_t)cfg.n_vars;
  const double* __restrict__ shi = b.hi + s * (uint64_t)cfg.n_vars;
  double* __restrict__ plo = b.plo;
  double* __restrict__ phi = b.phi;
  const uint32_t dep = b.depth[s];
  constexpr int kGroup = 8;
  for (int v0 = 0; v0 < cfg.n_vars; v0 += kGroup) {
    double l[kGroup], h[kGroup];
#pragma unroll
    for (int u = 0; u < kGroup; ++u)
      if (v0 + u < cfg.n_vars) {
        l[u] = slo[v0 + u];
        h[u] = shi[v0 + u];
      }
#pragma unroll
    for (int u = 0; u < kGroup; ++u)
      if (v0 + u < cfg.n_vars) {
        const uint64_t at = (uint64_t)(v0 + u) * cfg.e_max + pos;
        plo[at] = l[u];
        phi[at] = h[u];
        if (b.plo32 != nullptr) {
          b.plo32[at] = __double2float_rd(l[u]);
          b.phi32[at] = __double2float_ru(h[u]);
        }
      }
  }
  b.pdepth[pos] = dep;
}

// decode a kept child from its parent into a free store slot and append it
// behind the pool in the current buffer (position pool_size + pos)
struct AppendChild {
  SolverCfg cfg;
  SolverBufs b;
  __device__ void operator()(uint64_t g, uint64_t pos) const
  {
    const SolverDev* d = b.dev;
    if (pos >= d->free_top) {  // more children than free slots: never expected
      b.dev->error = 1;
      return;
    }
    const uint64_t s = b.free_slots[d->free_top - 1 - pos];
    const uint64_t at = d->pool_size + pos;
    const uint32_t p = d->parity;
    const uint64_t k = g >> cfg.log2C, r = g & ((1ULL << cfg.log2C) - 1ULL);
    // every load is issued before the stores it does not depend on: the
    // pointers do not alias, and without that each parent value would wait
    // for the store before it
    const double* __restrict__ plo = b.plo;
    const double* __restrict__ phi = b.phi;
    double* __restrict__ slo = b.lo + s * (uint64_t)cfg.n_vars;
    double* __restrict__ shi = b.hi + s * (uint64_t)cfg.n_vars;
    const ParentInfo pi = b.pinfo[k];
    const double clb = b.clb[g];
    const uint32_t dep = b.pdepth[k];
    constexpr int kGroup = 8;
    for (int v0 = 0; v0 < cfg.n_vars; v0 += kGroup) {
      double l[kGroup], h[kGroup];
#pragma unroll
      for (int u = 0; u < kGroup; ++u)
        if (v0 + u < cfg.n_vars) {
          l[u] = plo[(uint64_t)(v0 + u) * cfg.e_max + k];
          h[u] = phi[(uint64_t)(v0 + u) * cfg.e_max + k];
        }
#pragma unroll
      for (int u = 0; u < kGroup; ++u)
        if (v0 + u < cfg.n_vars) {
          slo[v0 + u] = l[u];
          shi[v0 + u] = h[u];
        }
    }
    const SlotPlan* sp = b.slots + k * (uint64_t)cfg.max_slots;
    for (uint32_t j = 0; j < pi.count; ++j) {
      const SlotPlan sj = sp[j];
      const uint64_t part = slot_part(r, sj);
      double lo, hi;
      slot_bounds(sj, plo[(uint64_t)sj.vid * cfg.e_max + k], phi[(uint64_t)sj.vid * cfg.e_max + k], part, lo, hi);
      slo[sj.vid] = lo;
      shi[sj.vid] = hi;
    }
    b.depth[s] = dep + 1;
    parity_buf(b.lb, p)[at] = clb;
    parity_buf(b.slot, p)[at] = (uint32_t)s;
    parity_buf(b.sel, p)[at] = kSelAlive;
  }
};

struct ListChild {
  SolverBufs b;
  __device__ void operator()(uint64_t g, uint64_t pos) const { b.list[pos] = (uint32_t)g; }
};

template <class P, class Op>
__global__ void __launch_bounds__(kScanBlock) scatter_kernel(const P pred, const Op op,
                                                             const uint32_t* __restrict__ offsets)
{
  const uint64_t t0 = tile_first();
  if (pred.skip()) return;
  const uint64_t n = pred.size();
  if ((uint64_t)blockIdx.x * kScanTile >= n) return;
  bool f[kScanItems];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint64_t i = tile_item(t0, j);
    f[j] = i < n && pred(i);
  }
  int rank[kScanItems];
  tile_ranks(f, rank);
  const uint64_t base = offsets[blockIdx.x];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j)
    if (f[j]) op(tile_item(t0, j), base + (uint64_t)rank[j]);
}

// Stages this iteration's parents (kSelParent entries of the pool, in
// position order) from the store into the parent planes, unless the
// previous iteration staged them.
__global__ void __launch_bounds__(kScanBlock) gather_parents_kernel(const SolverCfg cfg, const SolverBufs b,
                                                                    const uint32_t* __restrict__ offsets)
{
  const uint64_t t0 = tile_first();
  const SolverDev* d = b.dev;
  if (d->done || d->skip_select) return;
  const uint64_t n = d->pool_size;
  const uint64_t base = offsets[blockIdx.x];
  const uint8_t* __restrict__ sel = pool_sel(b);
  uint8_t sv[kScanItems];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint64_t i = tile_item(t0, j);
    sv[j] = i < cfg.pstride ? sel[i] : kSelAlive;
  }
  if ((uint64_t)blockIdx.x * kScanTile >= n) return;
  bool f[kScanItems];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) f[j] = tile_item(t0, j) < n && sv[j] == kSelParent;
  int rank[kScanItems];
  tile_ranks(f, rank);
  const uint32_t* slot = parity_buf(b.slot, d->parity);
#pragma unroll
  for (int j = 0; j < kScanItems; ++j)
    if (f[j]) stage_parent(cfg, b, slot[tile_item(t0, j)], base + (uint64_t)rank[j]);
}

// Moves the entries that stay, in order, to the other buffer (lower bound,
// store slot and mark), folds their keys into the pool's key range, lists
// the store slots of the next iteration's parents among them in order, and
// pushes the store slots of the others (this iteration's parents and the
// evicted) onto the free stack in position order.
__global__ void __launch_bounds__(kScanBlock, 2) copy_pool_kernel(const SolverCfg cfg, const SolverBufs b)
{
  const uint64_t t0 = tile_first();
  SolverDev* d = b.dev;
  // control words, the tile's entries and its offsets are loaded together
  const uint32_t done = d->done;
  const uint64_t n = d->extent;
  const uint64_t free_base = d->free_top;
  const uint32_t p = d->parity, q = 1 - p;
  const uint64_t* __restrict__ slb = reinterpret_cast<const uint64_t*>(parity_buf(b.lb, p));
  const uint32_t* __restrict__ sslot = parity_buf(b.slot, p);
  const uint8_t* __restrict__ ssel = parity_buf(b.sel, p);
  uint64_t* __restrict__ dlb = reinterpret_cast<uint64_t*>(parity_buf(b.lb, q));
  uint32_t* __restrict__ dslot = parity_buf(b.slot, q);
  uint8_t* __restrict__ dsel = parity_buf(b.sel, q);
  const uint64_t base = b.block_offsets[blockIdx.x];
  const uint64_t pbase = b.block_offsets2[blockIdx.x];
  bool f[kScanItems], g[kScanItems], in[kScanItems];
  uint64_t x[kScanItems];  // raw bits of the lower bounds
  uint32_t sl[kScanItems];
  uint8_t sv[kScanItems];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint64_t i = tile_item(t0, j);
    const bool inb = i < cfg.pstride;
    sv[j] = inb ? ssel[i] : kSelParent;
    x[j] = inb ? slb[i] : 0;
    sl[j] = inb ? sslot[i] : 0u;
  }
  if (done) return;
  if ((uint64_t)blockIdx.x * kScanTile >= n) return;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    in[j] = tile_item(t0, j) < n;
    f[j] = in[j] && (sv[j] == kSelAlive || sv[j] == kSelNextParent);
    g[j] = in[j] && sv[j] == kSelNextParent;
  }
  // the key range of the entries that stay, per warp before the barriers
  // of the ranks, for thread 0 after them
  __shared__ uint64_t part_min[kScanBlock / 32], part_max[kScanBlock / 32];
  {
    uint64_t mkey = ~0ULL, xkey = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j)
      if (f[j]) {
        const uint64_t k = bits_key(x[j]);
        mkey = k < mkey ? k : mkey;
        xkey = k > xkey ? k : xkey;
      }
    mkey = warp_min_u64(mkey);
    xkey = warp_max_u64(xkey);
    if ((threadIdx.x & 31) == 0) {
      part_min[threadIdx.x >> 5] = mkey;
      part_max[threadIdx.x >> 5] = xkey;
    }
  }
  int rank[kScanItems], prank[kScanItems];  // stayers / next parents before each item
  tile_ranks2(f, g, rank, prank);
  if (threadIdx.x == 0) {
    uint64_t mkey = ~0ULL, xkey = 0;
    for (int w = 0; w < kScanBlock / 32; ++w) {
      mkey = part_min[w] < mkey ? part_min[w] : mkey;
      xkey = part_max[w] > xkey ? part_max[w] : xkey;
    }
    if (mkey != ~0ULL) atomicMin((unsigned long long*)&d->pool_min_key, (unsigned long long)mkey);
    if (xkey != 0) atomicMax((unsigned long long*)&d->pool_max_key, (unsigned long long)xkey);
  }
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    if (!in[j]) continue;
    const uint64_t i = tile_item(t0, j);
    const uint64_t stay_before = base + (uint64_t)rank[j];
    if (f[j]) {
      dlb[stay_before] = x[j];
      dslot[stay_before] = sl[j];
      dsel[stay_before] = g[j] ? kSelParent : kSelAlive;
      if (g[j]) {
        const uint64_t pos = pbase + (uint64_t)prank[j];
        if (pos < cfg.e_max) b.pslot[pos] = sl[j];
        else d->error = 1;
      }
    } else {
      b.free_slots[free_base + (i - stay_before)] = sl[j];
    }
  }
}

// stages the next iteration's parents listed by the pool move
__global__ void stage_next_kernel(const SolverCfg cfg, const SolverBufs b)
{
  const SolverDev* d = b.dev;
  if (d->done) return;
  const uint64_t n = d->pre_count < cfg.e_max ? d->pre_count : cfg.e_max;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
    stage_parent(cfg, b, b.pslot[k], k);
}

// appends the kept children listed (in order) by the compaction, one thread
// per child so that each child's chain of dependent loads runs in parallel
__global__ void append_children_kernel(const SolverCfg cfg, const SolverBufs b)
{
  const SolverDev* d = b.dev;
  if (d->done) return;
  const uint64_t n = d->kept;
  const AppendChild op{cfg, b};
  for (uint64_t pos = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; pos < n; pos += (uint64_t)gridDim.x * blockDim.x)
    op(b.list[pos], pos);
}

// pool entries [start, start + count) in position order, unpacked from the
// store
__global__ void frontier_gather_kernel(const SolverCfg cfg, const SolverBufs b, uint64_t start, uint64_t count,
                                       double* __restrict__ boxes, uint32_t* __restrict__ depths)
{
  const uint32_t p = b.dev->parity;
  const uint32_t* slot = parity_buf(b.slot, p);
  const int n = cfg.n_vars;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t s = slot[start + i];
    if (boxes)
      for (int v = 0; v < n; ++v) {
        boxes[(i * n + v) * 2] = b.lo[s * (uint64_t)cfg.n_vars + v];
        boxes[(i * n + v) * 2 + 1] = b.hi[s * (uint64_t)cfg.n_vars + v];
      }
    if (depths) depths[i] = b.depth[s];
  }
}

// ---------------------------------------------------------------------
// branching: BisectionBudgetCompositionPolicy::choose per parent
// ---------------------------------------------------------------------
// kLocal > 0: the policy's per-parent scratch lives in this thread's local
// memory (n <= kLocal), which the hardware interleaves across the warp and
// caches in L1; otherwise in the global scratch arrays
template <int kLocal>
__global__ void branch_kernel(const SolverCfg cfg, const SolverBufs b)
{
  const SolverDev* d = b.dev;
  if (d->done) return;
  const uint64_t E = d->n_parents;
  const int n = cfg.n_vars;
  const PolicyParams pp = {cfg.log2C, cfg.max_cycle, cfg.enumerate_cap, cfg.relative};
  const bool lazy = cfg.precision == CMN_PRECISION_FP32_LAZY;
  uint64_t fathomed = 0, fathomed_points = 0, bounded = 0;
  EnumCand ec_local[kLocal > 0 ? kLocal : 1];
  BisCand bc_local[kLocal > 0 ? kLocal : 1];
  uint64_t heap_local[kLocal > 0 ? kLocal : 1];
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < E; k += (uint64_t)gridDim.x * blockDim.x) {
    EnumCand* ec = kLocal > 0 ? ec_local : reinterpret_cast<EnumCand*>(b.enum_scratch) + k * (uint64_t)n;
    BisCand* bc = kLocal > 0 ? bc_local : reinterpret_cast<BisCand*>(b.bis_scratch) + k * (uint64_t)n;
    uint64_t* heap = kLocal > 0 ? heap_local : b.heap_scratch + k * (uint64_t)n;
    SlotPlan* sp = b.slots + k * (uint64_t)cfg.max_slots;
    ParentInfo pi = bisection_policy(b.plo + k, b.phi + k, cfg.e_max, n, b.kinds, pp, ec, bc, heap, sp);
    b.pinfo[k] = pi;
    // lazy form: the box's FP64 verdict runs beside this kernel, and
    // lazy_drop_kernel applies it and counts afterwards
    if (lazy) continue;
    if (pi.fathom) {
      ++fathomed;
      fathomed_points += pi.nreg;
    } else {
      bounded += pi.nreg;
    }
  }
  if (lazy) return;  // every thread of the block takes this branch
  unsigned long long c[3] = {fathomed, fathomed_points, bounded};
  block_sum(c);
  if (threadIdx.x == 0) {
    if (c[0]) atomicAdd((unsigned long long*)&b.dev->counters.fathomed, c[0]);
    if (c[1]) atomicAdd((unsigned long long*)&b.dev->counters.fathomed_points, c[1]);
    if (c[2]) atomicAdd((unsigned long long*)&b.dev->counters.bounded, c[2]);
  }
}

// Lazy form, after the FP64 verdict of the staged parents (run beside the
// branching): a box that the reference predicate or the incumbent excludes
// is not expanded -- its plan becomes empty -- and the expansion counters
// are taken as branch_kernel takes them for the other forms.
__global__ void lazy_drop_kernel(const SolverCfg cfg, const SolverBufs b)
{
  const SolverDev* d = b.dev;
  if (d->done) return;
  const uint64_t E = d->n_parents;
  const double gub = d->gub;
  uint64_t fathomed = 0, fathomed_points = 0, bounded = 0, certified = 0, dropped = 0;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < E; k += (uint64_t)gridDim.x * blockDim.x) {
    ParentInfo pi = b.pinfo[k];
    ++certified;
    if (!b.pfeas[k] || b.plb[k] > gub) {
      pi = ParentInfo{0, 0, 0};
      b.pinfo[k] = pi;
      ++dropped;
    }
    if (pi.fathom) {
      ++fathomed;
      fathomed_points += pi.nreg;
    } else {
      bounded += pi.nreg;
    }
  }
  unsigned long long c[5] = {fathomed, fathomed_points, bounded, certified, dropped};
  block_sum(c);
  if (threadIdx.x == 0) {
    if (c[0]) atomicAdd((unsigned long long*)&b.dev->counters.fathomed, c[0]);
    if (c[1]) atomicAdd((unsigned long long*)&b.dev->counters.fathomed_points, c[1]);
    if (c[2]) atomicAdd((unsigned long long*)&b.dev->counters.bounded, c[2]);
    if (c[3]) atomicAdd((unsigned long long*)&b.dev->counters.certified_fp64, c[3]);
    if (c[4]) atomicAdd((unsigned long long*)&b.dev->counters.certify_pruned, c[4]);
  }
}

// Lazy form, per child, after lazy_drop_kernel: the FP32 pass wrote the
// child's own FP32 bound and, for a box it proved infeasible or a
// duplicate, the final state.  A child of a dropped parent has no box; for
// the others the parent's certified bound, which holds for every child box
// inside it, is folded in, and the state follows from the folded bound:
// above the incumbent, within the band below it (to the FP64 pass, which
// may prune it; below the band FP64 could not), or eligible.
__global__ void lazy_fold_kernel(const SolverCfg cfg, const SolverBufs b)
{
  const SolverDev* d = b.dev;
  if (d->done) return;
  const uint64_t total = d->n_children;
  const double gub = d->gub;
  const double floor_b = certify_floor(gub);
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total;
       g += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = g >> cfg.log2C, r = g & ((1ULL << cfg.log2C) - 1ULL);
    const ParentInfo pi = b.pinfo[k];
    if (pi.fathom || r >= pi.nreg) {
      b.cstate[g] = kChildNone;
      continue;
    }
    const uint8_t st = b.cstate[g];
    if (st == kChildInfeasible || st == kChildDuplicate) continue;
    const double plb = b.plb[k], lb32 = b.clb[g];
    const double lb = plb > lb32 ? plb : lb32;
    b.clb[g] = lb;
    b.cstate[g] = lb > gub ? kChildDominated : lb >= floor_b ? kChildScreened : kChildEligible;
  }
}

// ---------------------------------------------------------------------
// incumbent, prune accounting, pool finish
// ---------------------------------------------------------------------
__global__ void incumbent_kernel(const SolverBufs b, const Cand* __restrict__ best)
{
  SolverDev* d = b.dev;
  if (d->done) return;
  const Cand c = *best;
  d->improved = 0;
  if (c.value < DBL_MAX && c.value < d->gub) {
    d->gub = c.value;
    d->best = c;
    d->have_best = 1;
    d->improved = 1;
  }
}

// counts of this iteration's child verdicts (search/driver.hpp:319-350)
__global__ void prune_count_kernel(const SolverCfg cfg, const SolverBufs b)
{
  SolverDev* d = b.dev;
  if (d->done) return;
  const uint64_t n = d->n_children;
  const double gub = d->gub;
  unsigned long long dup = 0, inf = 0, dom = 0, kept = 0, sampled = 0;
  uint64_t mkey = ~0ULL, xkey = 0;  // key range of the children the pool takes
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (uint64_t)gridDim.x * blockDim.x) {
    const uint8_t s = b.cstate[g];
    if (s == kChildNone) continue;
    if (cfg.sample_all || s == kChildEligible) ++sampled;
    if (s == kChildDuplicate) ++dup;
    else if (s == kChildInfeasible) ++inf;
    else if (s == kChildDominated || bits_lt(dbits(gub), dbits(b.clb[g]))) ++dom;
    else ++kept;
    if (s == kChildEligible) {  // a superset of the kept children
      const uint64_t k = lb_key(b.clb[g]);
      mkey = k < mkey ? k : mkey;
      xkey = k > xkey ? k : xkey;
    }
  }
  unsigned long long c[5] = {dup, inf, dom, kept, sampled};
  block_sum(c);
  mkey = block_min(mkey);
  xkey = block_max(xkey);
  if (threadIdx.x == 0) {
    if (mkey != ~0ULL) atomicMin((unsigned long long*)&d->child_min_key, (unsigned long long)mkey);
    if (xkey != 0) atomicMax((unsigned long long*)&d->child_max_key, (unsigned long long)xkey);
    if (c[0]) atomicAdd((unsigned long long*)&d->counters.pruned_duplicate, c[0]);
    if (c[1]) atomicAdd((unsigned long long*)&d->counters.pruned_infeasible, c[1]);
    if (c[2]) atomicAdd((unsigned long long*)&d->counters.pruned_dominated, c[2]);
    if (c[3]) atomicAdd((unsigned long long*)&d->counters.enqueued, c[3]);
    if (c[4]) atomicAdd((unsigned long long*)&d->counters.sampled, c[4] * cfg.S);
  }
}

// FP64 evaluations of this iteration: every non-duplicate child in FP64
// mode, the certify list in the screened mode.
__global__ void eval_count_kernel(const SolverCfg cfg, const SolverBufs b)
{
  SolverDev* d = b.dev;
  if (d->done) return;
  const uint64_t n = d->n_children;
  const bool fp32 = cfg.precision == CMN_PRECISION_FP32_SCREEN;
  const bool lazy = cfg.precision == CMN_PRECISION_FP32_LAZY;
  unsigned long long valid = 0, excluded = 0;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (uint64_t)gridDim.x * blockDim.x) {
    const uint8_t s = b.cstate[g];
    if (s == kChildNone || s == kChildDuplicate) continue;
    ++valid;
    if (s == kChildInfeasible || s == kChildDominated) ++excluded;
  }
  unsigned long long c[2] = {valid, excluded};
  block_sum(c);
  if (threadIdx.x == 0) {
    if (c[0]) atomicAdd((unsigned long long*)&d->iter_valid, c[0]);
    if (c[1]) atomicAdd((unsigned long long*)&d->iter_excluded, c[1]);
    if (c[0] && ((fp32 && d->use_screen) || lazy)) atomicAdd((unsigned long long*)&d->counters.screened_fp32, c[0]);
    if (c[0] && !fp32 && !lazy) atomicAdd((unsigned long long*)&d->counters.certified_fp64, c[0]);
  }
}

// The screen stays on while it excludes at least a quarter of the children
// it sees, and comes back on once the FP64 verdicts would have excluded a
// quarter: it never changes a decision, only whether the work is done.
__global__ void screen_policy_kernel(const SolverCfg cfg, const SolverBufs b)
{
  SolverDev* d = b.dev;
  if (d->done || cfg.precision != CMN_PRECISION_FP32_SCREEN) return;
  const uint64_t v = d->iter_valid;
  const uint64_t x = d->use_screen ? v - d->certify_count : d->iter_excluded;
  if (v > 0) d->use_screen = (x * 4 >= v) ? 1 : 0;
}

__global__ void certify_count_kernel(const SolverBufs b)
{
  SolverDev* d = b.dev;
  if (d->done) return;
  d->counters.certified_fp64 += d->certify_count;
}

__global__ void size_kernel(const SolverCfg cfg, const SolverBufs b)
{
  SolverDev* d = b.dev;
  if (d->done) return;
  d->remaining = d->pool_size - d->n_parents;
  d->new_size = d->remaining + d->kept;
  d->extent = d->pool_size + d->kept;
  d->free_top -= d->kept;  // taken by the appended children
  d->evict = d->new_size > cfg.cap ? 1 : 0;
  // the next iteration's parents: its E (search/driver.hpp:221-233) over the
  // pool this iteration leaves
  const uint64_t next_L = d->evict ? cfg.cap : d->new_size;
  uint64_t E = next_L < cfg.e_max ? next_L : cfg.e_max;
  const uint64_t left = cfg.iter_limit > d->expansions ? cfg.iter_limit - d->expansions : 0;
  d->pre_k = E < left ? E : left;
  d->evict_lo_key = d->pool_min_key < d->child_min_key ? d->pool_min_key : d->child_min_key;
  d->evict_hi_key = d->pool_max_key > d->child_max_key ? d->pool_max_key : d->child_max_key;
  d->pool_min_key = ~0ULL;  // refilled by the move to the other buffer
  d->pool_max_key = 0;
}

__global__ void finish_kernel(const SolverCfg cfg, const SolverBufs b)
{
  SolverDev* d = b.dev;
  if (d->done) return;
  // the survivors were moved to the other buffer: exactly the cap when
  // evicting, otherwise every alive entry
  const uint64_t expect = d->evict ? cfg.cap : d->new_size;
  if (d->survivors != expect) d->error = 1;
  d->free_top += d->extent - d->survivors;  // the parents' and the evicted slots
  if (d->free_top + d->survivors != cfg.pstride) d->error = 1;
  if (d->pre_count != d->pre_k) d->error = 1;
  d->pre_valid = d->pre_k > 0 ? 1u : 0u;
  d->pool_size = d->survivors;
  d->parity = 1 - d->parity;
  if (d->dropped_min_key != ~0ULL) d->dropped_lb_min = key_to_lb(d->dropped_min_key);
  if (d->pool_size > d->counters.peak_frontier) d->counters.peak_frontier = d->pool_size;
}

__global__ void pool_min_kernel(const SolverBufs b, uint64_t* viable_out)
{
  SolverDev* d = b.dev;
  const uint64_t n = d->pool_size;
  const double* lb = parity_buf(b.lb, d->parity);
  const double gub = d->gub;
  uint64_t mkey = ~0ULL;
  unsigned long long viable = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = lb_key(lb[i]);
    mkey = k < mkey ? k : mkey;
    if (lb[i] <= gub) ++viable;
  }
  unsigned long long c[1] = {viable};
  block_sum(c);
  mkey = block_min(mkey);
  if (threadIdx.x == 0) {
    if (mkey != ~0ULL) atomicMin((unsigned long long*)&d->pool_min_key, (unsigned long long)mkey);
    if (viable_out && c[0]) atomicAdd((unsigned long long*)viable_out, c[0]);
  }
}

__global__ void pool_min_reset_kernel(const SolverBufs b, uint64_t* viable_out)
{
  b.dev->pool_min_key = ~0ULL;
  if (viable_out) *viable_out = 0;
}

// ---------------------------------------------------------------------
// host: enqueue one iteration
// ---------------------------------------------------------------------
static int tiles(uint64_t max_items) { return (int)((max_items + kScanTile - 1) / kScanTile); }

static void scan(const SolverBufs& b, const uint32_t* counts, uint32_t* offsets, const uint64_t* n_items_dev,
                 uint64_t* total_dev, const uint32_t* active, const uint32_t* skip, cudaStream_t s)
{
  scan_kernel<<<1, 1024, 0, s>>>(counts, offsets, n_items_dev, total_dev, active, skip, &b.dev->done);
}

template <class P>
static void compact(const P& pred, uint64_t max_items, const uint64_t* n_items_dev, uint64_t* total_dev,
                    const SolverBufs& b, cudaStream_t s)
{
  count_kernel<P><<<tiles(max_items), kScanBlock, 0, s>>>(pred, b.block_counts);
  scan(b, b.block_counts, b.block_offsets, n_items_dev, total_dev, nullptr, nullptr, s);
}

template <class P, class Op>
static void scatter(const P& pred, const Op& op, uint64_t max_items, cudaStream_t s, const SolverBufs& b)
{
  scatter_kernel<P, Op><<<tiles(max_items), kScanBlock, 0, s>>>(pred, op, b.block_offsets);
}

// which = 0: this iteration's parents (skipped when the previous iteration
// staged them); which = 1: the cap and the next iteration's parents
static void radix_select(const SolverCfg& cfg, const SolverBufs& b, int which, uint64_t max_items, cudaStream_t s)
{
  const int T = which == 0 ? 1 : 2;
  const uint32_t* skip = which == 0 ? &b.dev->skip_select : nullptr;
  radix_init_kernel<<<1, 256, 0, s>>>(cfg, b, which);
  const int grid = (int)std::min<uint64_t>((max_items + 255) / 256, 4096);
  // digits of up to 11 bits from below the keys' common leading bits;
  // the passes after the buckets settle or the bits run out return at once
  for (int p = 0; p < (64 + kRadixBits - 1) / kRadixBits; ++p) {
    radix_hist_kernel<<<grid, 256, 0, s>>>(cfg, b, which);
    radix_pick_kernel<<<T, kPickThreads, 0, s>>>(b);
  }
  // ranks among entries inside the threshold buckets, then the marks with
  // the tile counts of the entries the next compactions move
  const uint64_t* n_dev = which == 0 ? &b.dev->pool_size : &b.dev->extent;
  eq_count_kernel<<<tiles(max_items), kScanBlock, 0, s>>>(cfg, b, which);
  scan(b, b.block_counts, b.block_offsets, n_dev, nullptr, &b.radix[0].rank, skip, s);
  if (which == 1) scan(b, b.block_counts2, b.block_offsets2, n_dev, nullptr, &b.radix[1].rank, nullptr, s);
  mark_kernel<<<tiles(max_items), kScanBlock, 0, s>>>(cfg, b, which);
  scan(b, b.block_counts, b.block_offsets, n_dev, which == 0 ? nullptr : &b.dev->survivors, nullptr, skip, s);
  if (which == 1) scan(b, b.block_counts2, b.block_offsets2, n_dev, &b.dev->pre_count, nullptr, nullptr, s);
}

static void mark(const cudaEvent_t* marks, int i, cudaStream_t s)
{
  if (marks) cudaEventRecordWithFlags(marks[i], s, cudaEventRecordExternal);
}

cudaError_t solver_iteration(const SolverCfg& cfg, const SolverBufs& b, int eval_grid, int sample_grid,
                             cudaStream_t s, const SideStream& side, const cudaEvent_t* marks, bool with_select)
{
  const bool lazy = cfg.precision == CMN_PRECISION_FP32_LAZY;
  const uint64_t max_children = cfg.e_max << cfg.log2C;
  const uint64_t max_pool = cfg.pstride;
  mark(marks, 0, s);
  begin_kernel<<<1, 1, 0, s>>>(cfg, b, with_select ? 0 : 1);

  // (1) select the E best parents and stage them (after the first
  // iteration, the previous one staged them)
  if (with_select) {
    radix_select(cfg, b, 0, cfg.cap, s);
    gather_parents_kernel<<<tiles(cfg.cap), kScanBlock, 0, s>>>(cfg, b, b.block_offsets);
  }

  // (1b) lazy form: the FP64 verdict of every staged parent -- its bound
  // has been an FP32 one (with its own parent's FP64 bound folded in) since
  // it was appended.  It runs on the side stream, beside the branching and
  // the FP32 child bounds, which do not read it: the 2^-B share of boxes
  // it evaluates leaves part of the GPU idle on its own.
  if (lazy) {
    cudaError_t e = cudaEventRecord(side.fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(side.stream, side.fork, 0);
    if (e != cudaSuccess) return e;
    mark(marks, 5, side.stream);
    EvalArgs pa = {};
    pa.prog = b.prog64;
    pa.prog_len = cfg.prog_len;
    pa.n_vars = cfg.n_vars;
    pa.n_slots = cfg.n_slots;
    pa.log2C = 0;  // one "child" per parent: the parent box itself
    pa.plo = b.plo;
    pa.phi = b.phi;
    pa.pstride = cfg.e_max;
    pa.n_children_dev = &b.dev->n_parents;
    pa.done = &b.dev->done;
    pa.out_lb = b.plb;
    pa.out_flag = b.pfeas;
    pa.sched = b.sched;
    pa.g_max = cfg.g_max;
    pa.capacity = cfg.eval_capacity;
    pa.error = &b.dev->error;
    e = launch_eval(pa, 6, false, eval_grid, kEvalThreads, side.stream);
    if (e != cudaSuccess) return e;
    mark(marks, 6, side.stream);
    e = cudaEventRecord(side.join, side.stream);
    if (e != cudaSuccess) return e;
  }

  // (2) branch
  {
    const int grid = (int)std::min<uint64_t>((cfg.e_max + 127) / 128, 2048);
    if (cfg.n_vars <= 8) branch_kernel<8><<<grid, 128, 0, s>>>(cfg, b);
    else if (cfg.n_vars <= 32) branch_kernel<32><<<grid, 128, 0, s>>>(cfg, b);
    else branch_kernel<0><<<grid, 128, 0, s>>>(cfg, b);
  }
  mark(marks, 1, s);

  // (3) bound every child: FP64, or FP32 screen + FP64 certify
  EvalArgs ea = {};
  ea.n_vars = cfg.n_vars;
  ea.n_slots = cfg.n_slots;
  ea.log2C = cfg.log2C;
  ea.plo = b.plo;
  ea.phi = b.phi;
  ea.pstride = cfg.e_max;
  ea.pinfo = b.pinfo;
  ea.slots = b.slots;
  ea.max_slots = cfg.max_slots;
  ea.n_children_dev = &b.dev->n_children;
  ea.gub = &b.dev->gub;
  ea.done = &b.dev->done;
  ea.out_lb = b.clb;
  ea.out_flag = b.cstate;
  ea.error = &b.dev->error;
  ea.prog_len = cfg.prog_len;
  ea.sched = b.sched;
  ea.g_max = cfg.g_max;
  ea.capacity = cfg.eval_capacity;
  cudaError_t e;
  if (cfg.precision == CMN_PRECISION_FP32_SCREEN) {
    ea.prog = b.prog32;
    ea.plo32 = b.plo32;
    ea.phi32 = b.phi32;
    ea.use_screen = &b.dev->use_screen;
    e = launch_eval(ea, 2, true, eval_grid, kEvalThreads, s);
    if (e != cudaSuccess) return e;
    ScreenedChild sc{b};
    compact(sc, max_children, &b.dev->n_children, &b.dev->certify_count, b, s);
    scatter(sc, ListChild{b}, max_children, s, b);
    EvalArgs ca = ea;
    ca.prog = b.prog64;
    ca.plo32 = nullptr;
    ca.phi32 = nullptr;
    ca.list = b.list;
    ca.list_count = &b.dev->certify_count;
    e = launch_eval(ca, 3, false, eval_grid, kEvalThreads, s);
    if (e != cudaSuccess) return e;
  } else if (lazy) {
    ea.prog = b.prog32;
    ea.plo32 = b.plo32;
    ea.phi32 = b.phi32;
    ea.parent_lb = nullptr;  // folded in by lazy_fold_kernel
    if (cfg.inc) {
      ea.inc_segments = cfg.inc_segments;
      ea.n_parents_dev = &b.dev->n_parents;
      ea.inc_seg = b.inc_seg;
      ea.inc_off = b.inc_off;
      ea.inc_pcs = b.inc_pcs;
      ea.inc_common = b.inc_common;
      ea.inc_parts = b.inc_parts;
      e = launch_inc(ea, eval_grid, kEvalThreads, s);
    } else {
      e = launch_eval(ea, 5, true, eval_grid, kEvalThreads, s);
    }
    if (e != cudaSuccess) return e;
    mark(marks, 7, s);
    // join the parents' FP64 verdict: drop the boxes it excludes, fold the
    // certified bounds into their children
    e = cudaStreamWaitEvent(s, side.join, 0);
    if (e != cudaSuccess) return e;
    {
      const int pgrid = (int)std::min<uint64_t>((cfg.e_max + 255) / 256, 1024);
      lazy_drop_kernel<<<pgrid, 256, 0, s>>>(cfg, b);
      const int cgrid = (int)std::min<uint64_t>((max_children + 255) / 256, 2048);
      lazy_fold_kernel<<<cgrid, 256, 0, s>>>(cfg, b);
    }
    // the survivors within the band below the incumbent, in FP64
    ScreenedChild sc{b};
    compact(sc, max_children, &b.dev->n_children, &b.dev->certify_count, b, s);
    scatter(sc, ListChild{b}, max_children, s, b);
    EvalArgs ca = ea;
    ca.prog = b.prog64;
    ca.plo32 = nullptr;
    ca.phi32 = nullptr;
    ca.parent_lb = b.plb;
    ca.inc_segments = 0;
    ca.list = b.list;
    ca.list_count = &b.dev->certify_count;
    e = launch_eval(ca, 3, false, eval_grid, kEvalThreads, s);
    if (e != cudaSuccess) return e;
  } else {
    ea.prog = b.prog64;
    e = launch_eval(ea, 1, false, eval_grid, kEvalThreads, s);
    if (e != cudaSuccess) return e;
  }
  {
    const int grid = (int)std::min<uint64_t>((max_children + 255) / 256, 1024);
    eval_count_kernel<<<grid, 256, 0, s>>>(cfg, b);
    if (cfg.precision == CMN_PRECISION_FP32_SCREEN) {
      certify_count_kernel<<<1, 1, 0, s>>>(b);
      screen_policy_kernel<<<1, 1, 0, s>>>(cfg, b);
    } else if (cfg.precision == CMN_PRECISION_FP32_LAZY) {
      certify_count_kernel<<<1, 1, 0, s>>>(b);
    }
  }
  mark(marks, 2, s);

  // (4) sample, ArgMin, incumbent update and witness
  SampleArgs sa = {};
  sa.prog = b.prog64;
  sa.prog_len = cfg.prog_len;
  sa.n_vars = cfg.n_vars;
  sa.n_slots = cfg.n_slots;
  sa.log2C = cfg.log2C;
  sa.plo = b.plo;
  sa.phi = b.phi;
  sa.pstride = cfg.e_max;
  sa.pinfo = b.pinfo;
  sa.slots = b.slots;
  sa.max_slots = cfg.max_slots;
  sa.var_kinds = b.kinds;
  sa.root_lb = b.root_lb;
  sa.root_ub = b.root_ub;
  sa.n_children_dev = &b.dev->n_children;
  sa.S = cfg.S;
  sa.salt_base_dev = &b.dev->salt_base;
  sa.sample_all = cfg.sample_all;
  sa.state = b.cstate;
  sa.gub = &b.dev->gub;
  sa.done = &b.dev->done;
  sa.block_best = b.block_best;
  sa.rejected = (unsigned long long*)&b.dev->counters.witness_rejected;
  sa.sched = b.sched;
  sa.g_max = cfg.g_max;
  sa.capacity = cfg.sample_capacity;
  sa.lg_min = cfg.sample_lg_min;
  if (cfg.precision == CMN_PRECISION_FP32_LAZY) {
    // FP32 screen of every sample, then each chunk's best in FP64
    SampleArgs qa = sa;
    qa.lg_min = cfg.screen_lg_min;
    qa.prog = b.prog32p;
    qa.cbest = b.cbest;
    e = launch_sample_screen(qa, cfg.screen_grid, kEvalThreads, s);
    if (e != cudaSuccess) return e;
    sa.cbest = b.cbest;
  }
  e = launch_sample(sa, sample_grid, kEvalThreads, s);
  if (e != cudaSuccess) return e;
  Cand* best = b.block_best + b.n_block_best - 1;  // last entry holds the result
  e = launch_reduce_cand(b.block_best, sample_grid, best, s);
  if (e != cudaSuccess) return e;
  incumbent_kernel<<<1, 1, 0, s>>>(b, best);
  e = launch_witness(best, b.plo, b.phi, cfg.e_max, b.pinfo, b.slots, cfg.max_slots, b.kinds, cfg.n_vars, cfg.S, 0,
                     &b.dev->salt_base, 0, &b.dev->improved, b.best_point, s);
  if (e != cudaSuccess) return e;
  mark(marks, 3, s);

  // (5) prune with the new incumbent and rebuild the pool
  {
    const int grid = (int)std::min<uint64_t>((max_children + 255) / 256, 1024);
    prune_count_kernel<<<grid, 256, 0, s>>>(cfg, b);
  }
  // the kept children go behind the pool in the current buffer; the
  // parents stay there as holes until the one compaction below
  KeptChild kept{b};
  compact(kept, max_children, &b.dev->n_children, &b.dev->kept, b, s);
  scatter(kept, ListChild{b}, max_children, s, b);
  {
    const int grid = (int)std::min<uint64_t>((max_children + 255) / 256, 4096);
    append_children_kernel<<<grid, 256, 0, s>>>(cfg, b);
  }
  size_kernel<<<1, 1, 0, s>>>(cfg, b);

  // (6) over the cap: keep the `cap` best alive entries, fold the rest into
  // the floor; then move every alive entry to the other buffer in order
  radix_select(cfg, b, 1, max_pool, s);
  copy_pool_kernel<<<tiles(max_pool), kScanBlock, 0, s>>>(cfg, b);
  {
    const int grid = (int)std::min<uint64_t>((cfg.e_max + 255) / 256, 1024);
    stage_next_kernel<<<grid, 256, 0, s>>>(cfg, b);
  }
  finish_kernel<<<1, 1, 0, s>>>(cfg, b);
  mark(marks, 4, s);
  return cudaGetLastError();
}

cudaError_t solver_init(const SolverCfg& cfg, const SolverBufs& b, const double* root_lb_dev,
                        const double* root_ub_dev, double gub0, cudaStream_t s)
{
  init_kernel<<<1, 256, 0, s>>>(cfg, b, root_lb_dev, root_ub_dev, gub0);
  const int grid = (int)std::min<uint64_t>((cfg.pstride + 255) / 256, 4096);
  free_init_kernel<<<grid, 256, 0, s>>>(cfg, b);
  cudaMemsetAsync(b.sel[0], kSelAlive, cfg.pstride, s);
  cudaMemsetAsync(b.sel[1], kSelAlive, cfg.pstride, s);
  return cudaGetLastError();
}

cudaError_t solver_frontier_gather(const SolverCfg& cfg, const SolverBufs& b, uint64_t start, uint64_t count,
                                   double* boxes, uint32_t* depths, cudaStream_t s)
{
  if (count == 0) return cudaSuccess;
  const int grid = (int)std::min<uint64_t>((count + 255) / 256, 4096);
  frontier_gather_kernel<<<grid, 256, 0, s>>>(cfg, b, start, count, boxes, depths);
  return cudaGetLastError();
}

cudaError_t solver_pool_stats(const SolverCfg& cfg, const SolverBufs& b, uint64_t* viable_dev, cudaStream_t s)
{
  pool_min_reset_kernel<<<1, 1, 0, s>>>(b, viable_dev);
  const int grid = (int)std::min<uint64_t>((cfg.pstride + 255) / 256, 4096);
  pool_min_kernel<<<grid, 256, 0, s>>>(b, viable_dev);
  return cudaGetLastError();
}

}  // namespace cmn
