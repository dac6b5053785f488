// fp64_emu.cuh -- IEEE 754 binary64 add, subtract and multiply with
// directed rounding (toward -inf / +inf), computed on the integer pipe.
//
// GB300 issues FP64 instructions at a small fraction of its integer rate,
// and the interval evaluator is bound by the FP64 pipe while most of its
// issue slots sit idle. Moving the round-up half of each interval
// operation to integer arithmetic lets both pipes work at once.
//
// The integer path handles normal operands whose result is normal; zeros,
// subnormals, infinities, NaNs, exact cancellation to zero, underflow and
// overflow take the FP64 instruction instead. Within its domain the
// integer path is exact by construction: the significand product or sum
// is formed exactly (128-bit product; sums with 10 guard bits and a sticky
// bit), then truncated and, when inexact, incremented in magnitude if the
// rounding direction points away from zero (IEEE 754-2008, 4.3.2).
#pragma once

#include <cstdint>

// The integer path compiles for the host as well, where a CPU test checks
// it against the host's FPU in each rounding mode.
#define CMN_EMU_HD __host__ __device__ __forceinline__

namespace cmn {
namespace emu {

constexpr uint64_t kM52 = (1ULL << 52) - 1;
constexpr uint64_t kAbs = 0x7fffffffffffffffULL;

__device__ __forceinline__ uint64_t bits(double x) { return (uint64_t)__double_as_longlong(x); }
__device__ __forceinline__ double from_bits(uint64_t u) { return __longlong_as_double((long long)u); }

CMN_EMU_HD uint64_t umul64hi(uint64_t a, uint64_t b)
{
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

CMN_EMU_HD int clz64(uint64_t x)  // x != 0
{
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

// exponent field in [1, 2046]: a normal number
CMN_EMU_HD bool normal_exp(uint32_t e) { return e - 1u < 2046u; }

// Packs sign, biased exponent e and significand m in [2^52, 2^53] after
// rounding; false when the result is not normal.
CMN_EMU_HD bool pack(uint32_t sign, int e, uint64_t m, uint64_t& r)
{
  if (m >> 53) {  // the increment carried out: m was 2^53 - 1
    m >>= 1;
    e += 1;
  }
  if (e <= 0 || e >= 2047) return false;
  r = ((uint64_t)sign << 63) | ((uint64_t)e << 52) | (m & kM52);
  return true;
}

// Rounding of the integer path: toward -inf, toward +inf, to nearest even.
enum Round { kDown = 0, kUp = 1, kNearest = 2 };

// a * b rounded in direction `mode`.
CMN_EMU_HD bool mul_round(uint64_t a, uint64_t b, int mode, uint64_t& r)
{
  const uint32_t ea = (uint32_t)(a >> 52) & 0x7ff, eb = (uint32_t)(b >> 52) & 0x7ff;
  if (!normal_exp(ea) || !normal_exp(eb)) return false;
  const uint64_t A = (a & kM52) | (1ULL << 52), B = (b & kM52) | (1ULL << 52);
  const uint64_t hi = umul64hi(A, B), lo = A * B;  // the exact product, < 2^106
  const uint32_t sign = (uint32_t)((a ^ b) >> 63);
  int e = (int)ea + (int)eb - 1023;
  uint64_t m;
  bool half, below;  // the first discarded bit, and any discarded bit after it
  if (hi >> 41) {  // product in [2^105, 2^106)
    m = (hi << 11) | (lo >> 53);
    half = (lo >> 52) & 1;
    below = (lo & ((1ULL << 52) - 1)) != 0;
    e += 1;
  } else {  // [2^104, 2^105)
    m = (hi << 12) | (lo >> 52);
    half = (lo >> 51) & 1;
    below = (lo & ((1ULL << 51) - 1)) != 0;
  }
  bool inc;
  if (mode == kNearest) {
    inc = half && (below || (m & 1));  // ties to even
  } else {
    const bool away = mode == kUp ? sign == 0 : sign != 0;
    inc = (half || below) && away;
  }
  m += inc ? 1 : 0;
  return pack(sign, e, m, r);
}

// a * b rounded toward +inf (up) or -inf (!up).
CMN_EMU_HD bool mul_dir(uint64_t a, uint64_t b, bool up, uint64_t& r)
{
  return mul_round(a, b, up ? kUp : kDown, r);
}

// a + b rounded toward +inf (up) or -inf (!up).
CMN_EMU_HD bool add_dir(uint64_t a, uint64_t b, bool up, uint64_t& r)
{
  uint32_t ea = (uint32_t)(a >> 52) & 0x7ff, eb = (uint32_t)(b >> 52) & 0x7ff;
  if (!normal_exp(ea) || !normal_exp(eb)) return false;
  if ((b & kAbs) > (a & kAbs)) {  // |a| >= |b|
    const uint64_t t = a;
    a = b;
    b = t;
    const uint32_t te = ea;
    ea = eb;
    eb = te;
  }
  const uint32_t sa = (uint32_t)(a >> 63), sb = (uint32_t)(b >> 63);
  const uint64_t A = ((a & kM52) | (1ULL << 52)) << 10;  // leading bit at 62, 10 guard bits
  const uint64_t B0 = ((b & kM52) | (1ULL << 52)) << 10;
  const uint32_t d = ea - eb;
  uint64_t Bs;
  bool sticky;
  if (d >= 64) {
    Bs = 0;
    sticky = true;
  } else {
    Bs = B0 >> d;
    sticky = d != 0 && (B0 << (64 - d)) != 0;
  }
  int e = (int)ea;
  uint64_t S;
  if (sa == sb) {
    S = A + Bs;  // < 2^64
    if (S >> 63) {
      sticky = sticky || (S & 1);
      S >>= 1;
      e += 1;
    }
  } else {
    // floor of the exact magnitude A - (Bs + f), f in [0, 1) known nonzero
    // when sticky; with sticky, d > 10 and the result keeps its leading bit
    // at 62 or 61, so the shift below is at most one and the truncation
    // argument holds (floor(M / 2^9) == floor(floor(M) / 2^9))
    S = A - Bs - (sticky ? 1 : 0);
    if (S == 0) return false;  // exact cancellation: the sign of zero is the instruction's
    const int L = clz64(S) - 1;
    S <<= L;
    e -= L;
  }
  uint64_t m = S >> 10;
  const bool inexact = sticky || (S & 1023) != 0;
  const bool away = up ? sa == 0 : sa != 0;
  m += (inexact && away) ? 1 : 0;
  return pack(sa, e, m, r);
}

// The FP64 instructions for everything outside the integer path; kept out
// of line so that the common path does not issue them.
static __device__ __noinline__ double hw_add_ru(double a, double b) { return __dadd_ru(a, b); }
static __device__ __noinline__ double hw_add_rd(double a, double b) { return __dadd_rd(a, b); }
static __device__ __noinline__ double hw_sub_ru(double a, double b) { return __dsub_ru(a, b); }
static __device__ __noinline__ double hw_sub_rd(double a, double b) { return __dsub_rd(a, b); }
static __device__ __noinline__ double hw_mul_ru(double a, double b) { return __dmul_ru(a, b); }
static __device__ __noinline__ double hw_mul_rd(double a, double b) { return __dmul_rd(a, b); }
static __device__ __noinline__ double hw_mul_rn(double a, double b) { return __dmul_rn(a, b); }

__device__ __forceinline__ double add_ru(double a, double b)
{
  uint64_t r;
  return add_dir(bits(a), bits(b), true, r) ? from_bits(r) : hw_add_ru(a, b);
}
__device__ __forceinline__ double add_rd(double a, double b)
{
  uint64_t r;
  return add_dir(bits(a), bits(b), false, r) ? from_bits(r) : hw_add_rd(a, b);
}
__device__ __forceinline__ double sub_ru(double a, double b)
{
  uint64_t r;
  return add_dir(bits(a), bits(b) ^ (1ULL << 63), true, r) ? from_bits(r) : hw_sub_ru(a, b);
}
__device__ __forceinline__ double sub_rd(double a, double b)
{
  uint64_t r;
  return add_dir(bits(a), bits(b) ^ (1ULL << 63), false, r) ? from_bits(r) : hw_sub_rd(a, b);
}
__device__ __forceinline__ double mul_ru(double a, double b)
{
  uint64_t r;
  return mul_dir(bits(a), bits(b), true, r) ? from_bits(r) : hw_mul_ru(a, b);
}
__device__ __forceinline__ double mul_rd(double a, double b)
{
  uint64_t r;
  return mul_dir(bits(a), bits(b), false, r) ? from_bits(r) : hw_mul_rd(a, b);
}
__device__ __forceinline__ double mul_rn(double a, double b)
{
  uint64_t r;
  return mul_round(bits(a), bits(b), kNearest, r) ? from_bits(r) : hw_mul_rn(a, b);
}

}  // namespace emu
}  // namespace cmn
