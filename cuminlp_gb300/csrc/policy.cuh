// policy.cuh -- BisectionBudgetCompositionPolicy::choose on the device
// (policy/bisection_budget.hpp:81-262), one thread per parent box.
//
// The reference orders its bisection candidates with the C++ library's
// make_heap / pop_heap / push_heap, so which of several equally wide
// variables is halved first is decided by that heap's layout; the hp_*
// functions restate the GCC libstdc++ heap algorithm (hole-based sift-down
// preferring the right child unless it is smaller, then a sift-up) so ties
// resolve exactly as in the reference.
#pragma once

#include <cstdint>

#include "../../include/cuminlp_gb300.h"
#include "kernels.cuh"

namespace cmn {

// The policy runs on the device (one thread per parent) and on the host
// (cmn_bisection_choose, for host-side drivers): the same source, with the
// round-to-nearest FP64 operations spelled once for both.
#ifdef __CUDA_ARCH__
#define CMN_POLICY_SUB(a, b) __dsub_rn((a), (b))
#define CMN_POLICY_DIV(a, b) __ddiv_rn((a), (b))
#define CMN_POLICY_D2U(x) __double2ull_rz(x)
#else
#define CMN_POLICY_SUB(a, b) ((a) - (b))
#define CMN_POLICY_DIV(a, b) ((a) / (b))
#define CMN_POLICY_D2U(x) ((unsigned long long)(x))
#endif

struct EnumCand {
  uint64_t vid, domain, bits;
  uint32_t kind, pad;
};
struct BisCand {
  uint64_t vid, bis;
  double live, orig;
  uint32_t kind, pad;
};

struct HeapCtx {
  const BisCand* c;
  int relative;
  __host__ __device__ double key(uint64_t i) const { return relative ? CMN_POLICY_DIV(c[i].live, c[i].orig) : c[i].live; }
  __host__ __device__ bool less(uint64_t a, uint64_t b) const { return key(a) < key(b); }
};

__host__ __device__ inline void hp_push_hole(uint64_t* f, int64_t hole, int64_t top, uint64_t value, const HeapCtx& h)
{
  int64_t parent = (hole - 1) / 2;
  while (hole > top && h.less(f[parent], value)) {
    f[hole] = f[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  f[hole] = value;
}

__host__ __device__ inline void hp_adjust(uint64_t* f, int64_t hole, int64_t len, uint64_t value, const HeapCtx& h)
{
  const int64_t top = hole;
  int64_t second = hole;
  while (second < (len - 1) / 2) {
    second = 2 * (second + 1);
    if (h.less(f[second], f[second - 1])) second--;
    f[hole] = f[second];
    hole = second;
  }
  if ((len & 1) == 0 && second == (len - 2) / 2) {
    second = 2 * (second + 1);
    f[hole] = f[second - 1];
    hole = second - 1;
  }
  hp_push_hole(f, hole, top, value, h);
}

__host__ __device__ inline void hp_make(uint64_t* f, int64_t len, const HeapCtx& h)
{
  if (len < 2) return;
  int64_t parent = (len - 2) / 2;
  for (;;) {
    const uint64_t v = f[parent];
    hp_adjust(f, parent, len, v, h);
    if (parent == 0) return;
    parent--;
  }
}

__host__ __device__ inline uint64_t int_domain(double lb, double ub)
{
  const double lo = ceil(lb), hi = floor(ub);
  if (hi < lo) return 0;
  return (uint64_t)CMN_POLICY_D2U(CMN_POLICY_SUB(hi, lo)) + 1;
}

__host__ __device__ inline uint64_t bits_for(uint64_t d)
{
  const uint64_t eff = d == 0 ? 1 : d;
  uint64_t bits = 0, cap = 1;
  while (cap < eff) {
    cap <<= 1;
    ++bits;
  }
  return bits > 1 ? bits : 1;
}

struct PolicyParams {
  int B;                  // bisection budget: 2^B regions per composition
  int64_t max_cycle;      // slot cap (0 = 64)
  int64_t enumerate_cap;  // SearchCalibration::enumerate_cap
  int relative;           // RelativeBisectionBudget key
};

// Variable v of the parent box is (plo[v * stride], phi[v * stride]).
// `ec`, `bc`, `heap` are scratch of n entries; `sp` receives the slots.
__host__ __device__ inline ParentInfo bisection_policy(const double* __restrict__ plo, const double* __restrict__ phi,
                                              uint64_t stride, int n, const int32_t* __restrict__ kinds,
                                              const PolicyParams& pp, EnumCand* ec, BisCand* bc, uint64_t* heap,
                                              SlotPlan* sp)
{
  const int64_t cap = pp.max_cycle == 0 ? 64 : pp.max_cycle;
  int64_t ne = 0, nb = 0, live = 0;
  for (int v = 0; v < n; ++v)
    if (phi[(uint64_t)v * stride] > plo[(uint64_t)v * stride]) ++live;
  for (int v = 0; v < n && ne + nb < cap; ++v) {
    const double lb = plo[(uint64_t)v * stride], ub = phi[(uint64_t)v * stride];
    if (!(ub > lb)) continue;
    const double w = CMN_POLICY_SUB(ub, lb);
    const int vk = kinds[v];
    if (vk == CMN_VAR_BINARY) {
      ec[ne] = {(uint64_t)v, 2, bits_for(2), (uint32_t)CMN_SLOT_BINARY_ENUMERATE, 0};
      ++ne;
    } else if (vk == CMN_VAR_INTEGER) {
      const uint64_t dd = int_domain(lb, ub);
      const uint64_t dm = dd > 1 ? dd : 1;
      if (pp.enumerate_cap == 0 || dm <= (uint64_t)pp.enumerate_cap) {
        ec[ne] = {(uint64_t)v, dd, bits_for(dd), (uint32_t)CMN_SLOT_INTEGER_ENUMERATE, 0};
        ++ne;
      } else {
        bc[nb] = {(uint64_t)v, 0, w, w, (uint32_t)CMN_SLOT_INTEGER_PARTITION, 0};
        ++nb;
      }
    } else {
      bc[nb] = {(uint64_t)v, 0, w, w, (uint32_t)CMN_SLOT_CONTINUOUS, 0};
      ++nb;
    }
  }
  ParentInfo pi;
  if (ne + nb == 0) {
    pi.count = 0;
    pi.nreg = 1;
    pi.fathom = 1;
    return pi;
  }
  for (int64_t i = 1; i < ne; ++i) {  // stable insertion sort by cost
    const EnumCand x = ec[i];
    int64_t j = i - 1;
    while (j >= 0 && x.bits < ec[j].bits) {
      ec[j + 1] = ec[j];
      --j;
    }
    ec[j + 1] = x;
  }
  uint64_t remaining = (uint64_t)pp.B;
  int64_t taken = 0;
  for (; taken < ne; ++taken) {
    if (ec[taken].bits > remaining) break;
    remaining -= ec[taken].bits;
  }
  for (int64_t i = taken; i < ne; ++i) {
    if (ec[i].kind == CMN_SLOT_INTEGER_ENUMERATE) {
      const uint64_t v = ec[i].vid;
      const double w = CMN_POLICY_SUB(phi[v * stride], plo[v * stride]);
      bc[nb] = {v, 0, w, w, (uint32_t)CMN_SLOT_INTEGER_PARTITION, 0};
      ++nb;
    }
  }
  for (int64_t i = 0; i < nb; ++i) heap[i] = (uint64_t)i;
  const HeapCtx h = {bc, pp.relative};
  hp_make(heap, nb, h);
  uint64_t spent = 0;
  for (; spent < remaining && nb > 0; ++spent) {
    // pop_heap, halve the top, push_heap
    if (nb > 1) {
      const uint64_t v = heap[nb - 1];
      heap[nb - 1] = heap[0];
      hp_adjust(heap, 0, nb - 1, v, h);
    }
    BisCand* c = &bc[heap[nb - 1]];
    c->live = CMN_POLICY_DIV(c->live, 2.0);
    ++c->bis;
    hp_push_hole(heap, nb - 1, 0, heap[nb - 1], h);
  }
  for (uint64_t q = spent; q < remaining; ++q) {
    int64_t widest = 0;
    for (int64_t i = 1; i < taken; ++i)
      if (ec[i].bits > ec[widest].bits) widest = i;
    ++ec[widest].bits;
  }
  uint32_t count = 0;
  bool all_enum = true;
  for (int64_t i = 0; i < taken; ++i) {
    sp[count] = {1ULL << ec[i].bits, 0, ec[i].domain, (uint32_t)ec[i].vid, ec[i].kind};
    ++count;
  }
  for (int64_t i = 0; i < nb; ++i) {
    if (bc[i].bis == 0) continue;
    const uint64_t w = 1ULL << bc[i].bis;
    sp[count] = {w, 0, w, (uint32_t)bc[i].vid, bc[i].kind};
    all_enum = false;
    ++count;
  }
  uint64_t running = 1;
  for (uint32_t j = 0; j < count; ++j) {
    sp[j].prefix = running;
    running *= sp[j].width;
    sp[j].step = slot_step(sp[j].kind, plo[(uint64_t)sp[j].vid * stride], phi[(uint64_t)sp[j].vid * stride], sp[j].width);
  }
  pi.count = count;
  pi.nreg = running;
  pi.fathom = (live <= (int64_t)count && all_enum) ? 1 : 0;
  return pi;
}

}  // namespace cmn
