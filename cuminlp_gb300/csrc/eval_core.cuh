// eval_core.cuh -- device arithmetic and the fused DAG interpreter.
//
// Interval operators return the tightest enclosure under IEEE-754 directed
// rounding (the semantics of the reference's interval library for the
// operator set of graph/ops.cuh:24-355).  They use the CUDA directed
// rounding intrinsics only (__dadd_rd, __dmul_ru, __fmul_rd, ...), never
// plain expressions, so no FMA contraction can change a bound.
//
// The multiplication picks the extreme corner products from the operand
// sign classes (two products; four only when both operands straddle zero),
// instead of forming all eight directed products.  Sign classes come from
// the sign bits (integer pipe), leaving the FP64 pipe to the products.
#pragma once

#include <cstdint>

#include "fp64_emu.cuh"
#include "kernels.cuh"
#include "program.h"

namespace cmn {

template <typename T>
struct Iv {
  T lo, hi;
};

template <typename T>
struct Arith;

// Which FP64 operations run on the integer pipe (fp64_emu.cuh) instead of
// the FP64 pipe, so that the two pipes share the work (both give the IEEE
// result bit for bit): bit 0 interval add and subtract rounded up, bit 1
// interval products rounded up outside the fused terms, bit 2 interval
// multiply rounded down, bits 3 and 4 the point evaluation's variable and
// coefficient products (round to nearest), bits 5 and 6 the fused terms'
// variable and coefficient interval products rounded up.
#ifndef CMN_FP64_EMU
#define CMN_FP64_EMU (2 | 8 | 32 | 64)
#endif

template <>
struct Arith<double> {
  static __device__ __forceinline__ double add_rd(double a, double b) { return __dadd_rd(a, b); }
  static __device__ __forceinline__ double add_ru(double a, double b)
  {
    return (CMN_FP64_EMU & 1) ? emu::add_ru(a, b) : __dadd_ru(a, b);
  }
  static __device__ __forceinline__ double sub_rd(double a, double b) { return __dsub_rd(a, b); }
  static __device__ __forceinline__ double sub_ru(double a, double b)
  {
    return (CMN_FP64_EMU & 1) ? emu::sub_ru(a, b) : __dsub_ru(a, b);
  }
  static __device__ __forceinline__ double mul_rd(double a, double b)
  {
    return (CMN_FP64_EMU & 4) ? emu::mul_rd(a, b) : __dmul_rd(a, b);
  }
  static __device__ __forceinline__ double mul_ru(double a, double b) { return __dmul_ru(a, b); }
  static __device__ __forceinline__ double div_rd(double a, double b) { return __ddiv_rd(a, b); }
  static __device__ __forceinline__ double div_ru(double a, double b) { return __ddiv_ru(a, b); }
  static __device__ __forceinline__ double sqrt_rd(double a) { return __dsqrt_rd(a); }
  static __device__ __forceinline__ double sqrt_ru(double a) { return __dsqrt_ru(a); }
  static __device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
  static __device__ __forceinline__ double sqrt_rn(double a) { return __dsqrt_rn(a); }
  // sign bit set (negative, -0 or negative NaN)
  static __device__ __forceinline__ bool sgn(double x) { return __double2hiint(x) < 0; }
  static __device__ __forceinline__ bool is_zero(double x)
  {
    return ((__double2hiint(x) & 0x7fffffff) | __double2loint(x)) == 0;
  }
  // a > b for two non-negative values (sign bit clear), on the integer pipe
  static __device__ __forceinline__ bool gt_nonneg(double a, double b)
  {
    return __double_as_longlong(a) > __double_as_longlong(b);
  }
  static __device__ __forceinline__ double inf() { return __longlong_as_double(0x7ff0000000000000LL); }
  static __device__ __forceinline__ double nan() { return __longlong_as_double(0x7ff8000000000000LL); }
};

template <>
struct Arith<float> {
  static __device__ __forceinline__ float add_rd(float a, float b) { return __fadd_rd(a, b); }
  static __device__ __forceinline__ float add_ru(float a, float b) { return __fadd_ru(a, b); }
  static __device__ __forceinline__ float sub_rd(float a, float b) { return __fsub_rd(a, b); }
  static __device__ __forceinline__ float sub_ru(float a, float b) { return __fsub_ru(a, b); }
  static __device__ __forceinline__ float mul_rd(float a, float b) { return __fmul_rd(a, b); }
  static __device__ __forceinline__ float mul_ru(float a, float b) { return __fmul_ru(a, b); }
  static __device__ __forceinline__ float div_rd(float a, float b) { return __fdiv_rd(a, b); }
  static __device__ __forceinline__ float div_ru(float a, float b) { return __fdiv_ru(a, b); }
  static __device__ __forceinline__ float sqrt_rd(float a) { return __fsqrt_rd(a); }
  static __device__ __forceinline__ float sqrt_ru(float a) { return __fsqrt_ru(a); }
  static __device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
  static __device__ __forceinline__ float sqrt_rn(float a) { return __fsqrt_rn(a); }
  static __device__ __forceinline__ bool sgn(float x) { return __float_as_int(x) < 0; }
  static __device__ __forceinline__ bool is_zero(float x) { return (__float_as_int(x) & 0x7fffffff) == 0; }
  static __device__ __forceinline__ bool gt_nonneg(float a, float b)
  {
    return __float_as_int(a) > __float_as_int(b);
  }
  static __device__ __forceinline__ float inf() { return __int_as_float(0x7f800000); }
  static __device__ __forceinline__ float nan() { return __int_as_float(0x7fc00000); }
};

// x*y for interval endpoints: a zero factor gives +0 even against an
// infinite bound (IEEE 1788), never NaN.
template <typename T>
__device__ __forceinline__ T emul_rd(T x, T y)
{
  using A = Arith<T>;
  return (A::is_zero(x) | A::is_zero(y)) ? T(0) : A::mul_rd(x, y);
}
template <typename T>
__device__ __forceinline__ T emul_ru(T x, T y)
{
  using A = Arith<T>;
  return (A::is_zero(x) | A::is_zero(y)) ? T(0) : A::mul_ru(x, y);
}
// emul_ru with the product on the integer pipe when kInt (FP64 only)
template <typename T, bool kInt>
__device__ __forceinline__ T emul_ru_sel(T x, T y)
{
  if constexpr (kInt && sizeof(T) == 8) {
    using A = Arith<T>;
    return (A::is_zero(x) | A::is_zero(y)) ? T(0) : emu::mul_ru(x, y);
  } else {
    return emul_ru(x, y);
  }
}

template <typename T>
__device__ __forceinline__ Iv<T> iv_add(Iv<T> a, Iv<T> b)
{
  return {Arith<T>::add_rd(a.lo, b.lo), Arith<T>::add_ru(a.hi, b.hi)};
}

template <typename T>
__device__ __forceinline__ Iv<T> iv_sub(Iv<T> a, Iv<T> b)
{
  return {Arith<T>::sub_rd(a.lo, b.hi), Arith<T>::sub_ru(a.hi, b.lo)};
}

template <typename T>
__device__ __forceinline__ Iv<T> iv_neg(Iv<T> a)
{
  return {-a.hi, -a.lo};
}

// Tightest product.  Sign classes: pos (lo has no sign bit), neg (hi has
// the sign bit), mixed otherwise.  A zero endpoint may land in either
// class; the chosen corner products then differ only in the sign of a zero.
template <typename T, bool kIntUp = (CMN_FP64_EMU & 2) != 0>
__device__ __forceinline__ Iv<T> iv_mul(Iv<T> a, Iv<T> b)
{
  using A = Arith<T>;
  const bool ap = !A::sgn(a.lo), an = A::sgn(a.hi);
  const bool bp = !A::sgn(b.lo), bn = A::sgn(b.hi);
  const bool am = !ap && !an, bm = !bp && !bn;
  const T la = ap ? (bp ? a.lo : a.hi) : (an ? (bn ? a.hi : a.lo) : (bn ? a.hi : a.lo));
  const T lb = ap ? b.lo : (an ? b.hi : (bn ? b.lo : b.hi));
  const T ua = ap ? (bn ? a.lo : a.hi) : (an ? (bp ? a.hi : a.lo) : (bn ? a.lo : a.hi));
  const T ub = ap ? b.hi : (an ? b.lo : (bn ? b.lo : b.hi));
  Iv<T> r = {emul_rd(la, lb), emul_ru_sel<T, kIntUp>(ua, ub)};
  const bool mm = am && bm;
  if (__any_sync(__activemask(), mm)) {
    const T l2 = emul_rd(a.hi, b.lo);
    const T u2 = emul_ru_sel<T, kIntUp>(a.lo, b.lo);
    if (mm) {
      r.lo = l2 < r.lo ? l2 : r.lo;
      r.hi = u2 > r.hi ? u2 : r.hi;
    }
  }
  return r;
}

// iv_mul(c, p) for a coefficient interval c: when c's two ends carry the
// same sign bit (always in FP64, where c is a point), iv_mul's corner
// choice depends on the sign bits of c and of one end of p only, so the
// same two products come out with fewer selects. A coefficient pair that
// straddles a sign change takes iv_mul itself.
template <typename T, bool kIntUp = (CMN_FP64_EMU & 2) != 0>
__device__ __forceinline__ Iv<T> iv_scale(Iv<T> c, Iv<T> p)
{
  using A = Arith<T>;
  const bool cp = !A::sgn(c.lo), cn = A::sgn(c.hi);
  if (cp) {  // c >= 0, iv_mul's class "pos" for a
    return {emul_rd(A::sgn(p.lo) ? c.hi : c.lo, p.lo), emul_ru_sel<T, kIntUp>(A::sgn(p.hi) ? c.lo : c.hi, p.hi)};
  }
  if (cn) {  // c <= 0, class "neg"
    return {emul_rd(A::sgn(p.hi) ? c.hi : c.lo, p.hi), emul_ru_sel<T, kIntUp>(A::sgn(p.lo) ? c.lo : c.hi, p.lo)};
  }
  return iv_mul<T, kIntUp>(c, p);
}

template <typename T, bool kIntUp = (CMN_FP64_EMU & 2) != 0>
__device__ __forceinline__ Iv<T> iv_sqr(Iv<T> a)
{
  using A = Arith<T>;
  const bool p = !A::sgn(a.lo), n = A::sgn(a.hi);
  const T mlo = -a.lo;
  const T mag = A::gt_nonneg(mlo, a.hi) ? mlo : a.hi;  // mixed: both >= 0
  const T lo_op = p ? a.lo : (n ? a.hi : T(0));
  const T hi_op = p ? a.hi : (n ? a.lo : mag);
  return {emul_rd(lo_op, lo_op), emul_ru_sel<T, kIntUp>(hi_op, hi_op)};
}

template <typename T>
__device__ __forceinline__ T tmin(T a, T b) { return a < b ? a : b; }
template <typename T>
__device__ __forceinline__ T tmax(T a, T b) { return a > b ? a : b; }

template <typename T>
__device__ Iv<T> iv_div(Iv<T> a, Iv<T> b)
{
  using A = Arith<T>;
  Iv<T> r;
  if (b.lo > T(0) || b.hi < T(0)) {
    const T l1 = A::div_rd(a.lo, b.lo), l2 = A::div_rd(a.lo, b.hi);
    const T l3 = A::div_rd(a.hi, b.lo), l4 = A::div_rd(a.hi, b.hi);
    const T u1 = A::div_ru(a.lo, b.lo), u2 = A::div_ru(a.lo, b.hi);
    const T u3 = A::div_ru(a.hi, b.lo), u4 = A::div_ru(a.hi, b.hi);
    r.lo = tmin(tmin(l1, l2), tmin(l3, l4));
    r.hi = tmax(tmax(u1, u2), tmax(u3, u4));
    return r;
  }
  if (b.lo == T(0) && b.hi == T(0)) return {A::nan(), A::nan()};
  if (b.lo == T(0)) {
    if (a.lo >= T(0)) return {A::div_rd(a.lo, b.hi), A::inf()};
    if (a.hi <= T(0)) return {-A::inf(), A::div_ru(a.hi, b.hi)};
  } else if (b.hi == T(0)) {
    if (a.lo >= T(0)) return {-A::inf(), A::div_ru(a.lo, b.lo)};
    if (a.hi <= T(0)) return {A::div_rd(a.hi, b.lo), A::inf()};
  }
  return {-A::inf(), A::inf()};
}

template <typename T>
__device__ __forceinline__ Iv<T> iv_sqrt(Iv<T> a)
{
  using A = Arith<T>;
  if (a.hi < T(0)) return {A::nan(), A::nan()};
  return {a.lo > T(0) ? A::sqrt_rd(a.lo) : T(0), A::sqrt_ru(a.hi)};
}

template <typename T>
__device__ __forceinline__ Iv<T> iv_abs(Iv<T> a)
{
  if (a.lo >= T(0)) return a;
  if (a.hi <= T(0)) return {-a.hi, -a.lo};
  return {T(0), tmax(-a.lo, a.hi)};
}

template <typename T>
__device__ __forceinline__ T powu_rd(T a, int k)
{
  T r = T(1), base = a;
  while (k > 0) {
    if (k & 1) r = emul_rd(r, base);
    k >>= 1;
    if (k > 0) base = emul_rd(base, base);
  }
  return r;
}

template <typename T>
__device__ __forceinline__ T powu_ru(T a, int k)
{
  T r = T(1), base = a;
  while (k > 0) {
    if (k & 1) r = emul_ru(r, base);
    k >>= 1;
    if (k > 0) base = emul_ru(base, base);
  }
  return r;
}

template <typename T>
__device__ Iv<T> iv_pown(Iv<T> a, int k)
{
  if (k == 0) return {T(1), T(1)};
  if (k == 1) return a;
  if (k == 2) {
    // same classes as the oracle's sqr for pown(x, 2)
    return iv_sqr(a);
  }
  if (k < 0) {
    Iv<T> one = {T(1), T(1)};
    return iv_div(one, iv_pown(a, -k));
  }
  if ((k & 1) == 0) {
    const T mig = a.lo > T(0) ? a.lo : (a.hi < T(0) ? -a.hi : T(0));
    const T mag = tmax(a.lo < T(0) ? -a.lo : a.lo, a.hi < T(0) ? -a.hi : a.hi);
    return {powu_rd(mig, k), powu_ru(mag, k)};
  }
  return {a.lo >= T(0) ? powu_rd(a.lo, k) : -powu_ru(-a.lo, k),
          a.hi >= T(0) ? powu_ru(a.hi, k) : -powu_rd(-a.hi, k)};
}

// ---- transcendental enclosures ----
// Exp, Log, Sin, Cos, Tanh and Pow bound their range by CUDA's math
// functions at the interval's ends (and at the interior extrema of Sin and
// Cos), each result moved outward by kTransWiden ulps: the CUDA math
// library's documented maximum errors are 1-2 ulps in double and 1-4 ulps in
// float for these functions, so the widened result encloses the exact
// value.  These enclosures are sound but not tightest, and no reference
// result pins them bit for bit.
template <typename T>
struct Trans;
template <>
struct Trans<double> {
  static constexpr int kWiden = 3;
  static __device__ __forceinline__ double exp(double x) { return ::exp(x); }
  static __device__ __forceinline__ double log(double x) { return ::log(x); }
  static __device__ __forceinline__ double sin(double x) { return ::sin(x); }
  static __device__ __forceinline__ double cos(double x) { return ::cos(x); }
  static __device__ __forceinline__ double tanh(double x) { return ::tanh(x); }
  static __device__ __forceinline__ double pow(double x, double y) { return ::pow(x, y); }
  static __device__ __forceinline__ double next(double x, double dir) { return ::nextafter(x, dir); }
  static __device__ __forceinline__ double pi_lo() { return 3.141592653589793; }
  static __device__ __forceinline__ double pi_hi() { return 3.1415926535897936; }
};
template <>
struct Trans<float> {
  static constexpr int kWiden = 5;
  static __device__ __forceinline__ float exp(float x) { return ::expf(x); }
  static __device__ __forceinline__ float log(float x) { return ::logf(x); }
  static __device__ __forceinline__ float sin(float x) { return ::sinf(x); }
  static __device__ __forceinline__ float cos(float x) { return ::cosf(x); }
  static __device__ __forceinline__ float tanh(float x) { return ::tanhf(x); }
  static __device__ __forceinline__ float pow(float x, float y) { return ::powf(x, y); }
  static __device__ __forceinline__ float next(float x, float dir) { return ::nextafterf(x, dir); }
  static __device__ __forceinline__ float pi_lo() { return 3.14159250f; }
  static __device__ __forceinline__ float pi_hi() { return 3.14159274f; }
};

template <typename T>
__device__ __forceinline__ T widen_down(T x)
{
  if (x != x) return x;
  for (int i = 0; i < Trans<T>::kWiden; ++i) x = Trans<T>::next(x, -Arith<T>::inf());
  return x;
}
template <typename T>
__device__ __forceinline__ T widen_up(T x)
{
  if (x != x) return x;
  for (int i = 0; i < Trans<T>::kWiden; ++i) x = Trans<T>::next(x, Arith<T>::inf());
  return x;
}
template <typename T>
__device__ __forceinline__ T clampv(T x, T lo, T hi) { return x < lo ? lo : (x > hi ? hi : x); }

template <typename T>
__device__ Iv<T> iv_exp(Iv<T> a)
{
  const T lo = widen_down(Trans<T>::exp(a.lo));
  return {lo < T(0) ? T(0) : lo, widen_up(Trans<T>::exp(a.hi))};
}

// log over the part of the interval inside its domain [0, inf)
template <typename T>
__device__ Iv<T> iv_log(Iv<T> a)
{
  if (a.hi < T(0)) return {Arith<T>::nan(), Arith<T>::nan()};
  const T lo = a.lo <= T(0) ? -Arith<T>::inf() : widen_down(Trans<T>::log(a.lo));
  const T hi = a.hi == T(0) ? -Arith<T>::inf() : widen_up(Trans<T>::log(a.hi));
  return {lo, hi};
}

template <typename T>
__device__ Iv<T> iv_tanh(Iv<T> a)
{
  return {clampv(widen_down(Trans<T>::tanh(a.lo)), T(-1), T(1)), clampv(widen_up(Trans<T>::tanh(a.hi)), T(-1), T(1))};
}

// sin (shift 1) or cos (shift 0): the ends, plus +-1 wherever an extremum
// (a multiple of pi for cos, pi/2 off it for sin) may lie in the interval;
// every multiple of pi is located with pi's enclosure, so near-misses count
// as hits
template <typename T>
__device__ Iv<T> iv_trig(Iv<T> a, bool is_sin)
{
  using A = Arith<T>;
  if (!(a.lo <= a.hi)) return {A::nan(), A::nan()};
  if (a.lo == -A::inf() || a.hi == A::inf()) return {T(-1), T(1)};
  const T f0 = is_sin ? Trans<T>::sin(a.lo) : Trans<T>::cos(a.lo);
  const T f1 = is_sin ? Trans<T>::sin(a.hi) : Trans<T>::cos(a.hi);
  T lo = widen_down(tmin(f0, f1)), hi = widen_up(tmax(f0, f1));
  const T pl = Trans<T>::pi_lo(), ph = Trans<T>::pi_hi();
  T tl = tmin(A::div_rd(a.lo, pl), A::div_rd(a.lo, ph));
  T th = tmax(A::div_ru(a.hi, pl), A::div_ru(a.hi, ph));
  if (is_sin) {
    tl = A::sub_rd(tl, T(0.5));
    th = A::sub_ru(th, T(0.5));
  }
  const T jl = ceil(widen_down(tl)), jh = floor(widen_up(th));
  if (!(jh - jl < T(2))) return {T(-1), T(1)};
  for (T j = jl; j <= jh; j = j + T(1)) {
    const T half = j * T(0.5);
    if (half == floor(half)) hi = T(1);  // even multiple: a maximum
    else lo = T(-1);                      // odd: a minimum
  }
  return {clampv(lo, T(-1), T(1)), clampv(hi, T(-1), T(1))};
}

// a^b for a clipped to [0, inf), enclosed as exp(b * log(a))
template <typename T>
__device__ Iv<T> iv_pow(Iv<T> a, Iv<T> b)
{
  if (a.hi < T(0)) return {Arith<T>::nan(), Arith<T>::nan()};
  const Iv<T> x = {a.lo < T(0) ? T(0) : a.lo, a.hi};
  return iv_exp(iv_mul(b, iv_log(x)));
}

template <typename T>
__device__ __forceinline__ Iv<T> iv_generic(uint8_t op, Iv<T> a, Iv<T> b, int k)
{
  switch (op) {
    case kGExp: return iv_exp(a);
    case kGLog: return iv_log(a);
    case kGSin: return iv_trig(a, true);
    case kGCos: return iv_trig(a, false);
    case kGTanh: return iv_tanh(a);
    case kGPow: return iv_pow(a, b);
    case kGAdd: return iv_add(a, b);
    case kGSub: return iv_sub(a, b);
    case kGMul: return iv_mul(a, b);
    case kGDiv: return iv_div(a, b);
    case kGSqr: return iv_sqr(a);
    case kGNeg: return iv_neg(a);
    case kGSqrt: return iv_sqrt(a);
    case kGPowN: return iv_pown(a, k);
    case kGAbs: return iv_abs(a);
    case kGMin: return {tmin(a.lo, b.lo), tmin(a.hi, b.hi)};
    case kGMax: return {tmax(a.lo, b.lo), tmax(a.hi, b.hi)};
    default: return {Arith<T>::nan(), Arith<T>::nan()};
  }
}

// Point arithmetic: one round-to-nearest operation per DAG node
// (graph/ops.cuh point overloads).
__device__ __forceinline__ double pt_generic(uint8_t op, double a, double b, int k)
{
  using A = Arith<double>;
  switch (op) {
    case kGAdd: return A::add_rn(a, b);
    case kGSub: return A::sub_rn(a, b);
    case kGMul: return A::mul_rn(a, b);
    case kGDiv: return A::div_rn(a, b);
    case kGSqr: return A::mul_rn(a, a);
    case kGNeg: return -a;
    case kGSqrt: return A::sqrt_rn(a);
    case kGPowN: return k == 2 ? A::mul_rn(a, a) : pow(a, (double)k);
    case kGAbs: return fabs(a);
    case kGMin: return fmin(a, b);
    case kGMax: return fmax(a, b);
    case kGExp: return exp(a);
    case kGLog: return log(a);
    case kGSin: return sin(a);
    case kGCos: return cos(a);
    case kGTanh: return tanh(a);
    case kGPow: return pow(a, b);
    default: return A::nan();
  }
}

// The value of one variable / slot for this thread: shared-memory planes,
// plane-major with `stride` entries per plane, this thread at `tid`.
template <typename T>
struct Tile {
  T* lo;  // n_vars planes
  T* hi;
  T* slo;  // program slots
  T* shi;
  int stride;
  int tid;
  __device__ __forceinline__ Iv<T> var(int v) const { return {lo[v * stride + tid], hi[v * stride + tid]}; }
  __device__ __forceinline__ Iv<T> slot(int s) const { return {slo[s * stride + tid], shi[s * stride + tid]}; }
  __device__ __forceinline__ void set_slot(int s, Iv<T> x) const
  {
    slo[s * stride + tid] = x.lo;
    shi[s * stride + tid] = x.hi;
  }
};

// Bound of storage type S as an interval endpoint of type T: identity, or
// FP64 -> FP32 rounded outward.
template <typename T, typename S>
struct Widen {
  __device__ static __forceinline__ T lo(S x) { return x; }
  __device__ static __forceinline__ T hi(S x) { return x; }
};
template <>
struct Widen<float, double> {
  __device__ static __forceinline__ float lo(double x) { return __double2float_rd(x); }
  __device__ static __forceinline__ float hi(double x) { return __double2float_ru(x); }
};

// The variables of one child box without a per-thread copy of the box: a
// variable is read from the parent's planes in global memory (siblings read
// the same addresses, so the loads hit L1), unless it is one of the child's
// split variables, whose narrowed bounds sit in this thread's shared-memory
// column.  `mask` has bit (v & 63) set for every split variable v, so an
// unsplit variable costs one test.
template <typename T, typename S>
struct ChildVars {
  const S* plo;  // the parent's bound of variable v at plo[v * pstride]
  const S* phi;
  uint64_t pstride;
  uint64_t mask;
  const T* olo;  // split slot j of this thread at olo[j * stride]
  const T* ohi;
  const int32_t* ovid;
  int count;
  int stride;
  __device__ __forceinline__ Iv<T> var(int v) const
  {
    if ((mask >> (v & 63)) & 1ULL) {
      for (int j = 0; j < count; ++j)
        if (ovid[j * stride] == v) return {olo[j * stride], ohi[j * stride]};
    }
    const uint64_t off = (uint64_t)v * pstride;
    return {Widen<T, S>::lo(__ldg(plo + off)), Widen<T, S>::hi(__ldg(phi + off))};
  }
};

__device__ __forceinline__ Instr load_instr(const Instr* prog, int pc)
{
  int4 raw = __ldg(reinterpret_cast<const int4*>(prog) + pc);
  Instr ins;
  memcpy(&ins, &raw, sizeof(Instr));
  return ins;
}

// Operand of an interval program.  FP64 constants are point intervals; FP32
// constants carry their outward-rounded pair.
template <typename T>
__device__ __forceinline__ Iv<T> const_of(const Instr& ins);
template <>
__device__ __forceinline__ Iv<double> const_of<double>(const Instr& ins)
{
  return {ins.c, ins.c};
}
template <>
__device__ __forceinline__ Iv<float> const_of<float>(const Instr& ins)
{
  return {ins.c32.clo, ins.c32.chi};
}

template <typename T, typename V>
__device__ __forceinline__ Iv<T> fetch(const V& vars, const Tile<T>& t, const Iv<T>& acc, const Instr& ins, int mode,
                                       int idx)
{
  switch (mode) {
    case kModeSlot: return t.slot(idx);
    case kModeVar: return vars.var(idx);
    case kModeAcc: return acc;
    default: return const_of<T>(ins);
  }
}

// Result of interpreting the program on one box.
template <typename T>
struct Verdict {
  Iv<T> obj;
  bool feasible;    // FP64: reference predicate (NaN lb -> infeasible)
  bool excluded;    // a constraint is proven violated (NaN never excludes)
  bool has_obj;     // this lane executed the objective (segmented runs)
};

template <typename T>
__device__ __forceinline__ Verdict<T> verdict_init()
{
  Verdict<T> out;
  out.obj = {Arith<T>::nan(), Arith<T>::nan()};
  out.feasible = true;
  out.excluded = false;
  out.has_obj = false;
  return out;
}

// The term t of a TERM instruction: x_a * x_b, sqr(x_a) or x_a, times the
// coefficient when it has one.
template <typename T, typename V>
__device__ __forceinline__ Iv<T> term_value(const Instr& cur, int sub, const V& vars)
{
  Iv<T> p;
  const int pk = sub & kTermPMask;
  if (pk == kTermProd) {
    p = iv_mul<T, (CMN_FP64_EMU & 32) != 0>(vars.var(cur.a), vars.var(cur.b));
  } else if (pk == kTermSqr) {
    p = iv_sqr<T, (CMN_FP64_EMU & 32) != 0>(vars.var(cur.a));
  } else {
    p = vars.var(cur.a);
  }
  if (sub & kTermHasC) p = iv_scale<T, (CMN_FP64_EMU & 64) != 0>(const_of<T>(cur), p);
  return p;
}

// The lazy form's FP64 verdict folds a term's coefficient into the chain
// add: acc (+|-) c * p with __fma_rd / __fma_ru, one rounding per bound
// instead of two (the product by c and the add).  The coefficient's sign
// picks the endpoint of p.  Sound, and tighter; not the reference's order
// of operations, so only the lazy form's own certification uses it.
template <typename T, bool kFused>
__device__ __forceinline__ bool fused_term(int sub)
{
  return kFused && sizeof(T) == 8 && (sub & kTermHasC) && !(sub & kTermInit);
}

// x_a * x_b, sqr(x_a) or x_a of a TERM instruction, before its coefficient.
template <typename T, typename V>
__device__ __forceinline__ Iv<T> term_product(const Instr& cur, int sub, const V& vars)
{
  const int pk = sub & kTermPMask;
  if (pk == kTermProd) return iv_mul<T, (CMN_FP64_EMU & 32) != 0>(vars.var(cur.a), vars.var(cur.b));
  if (pk == kTermSqr) return iv_sqr<T, (CMN_FP64_EMU & 32) != 0>(vars.var(cur.a));
  return vars.var(cur.a);
}

__device__ __forceinline__ Iv<double> fma_into(Iv<double> acc, double c, Iv<double> p, bool sub)
{
  const double cc = sub ? -c : c;
  const bool pos = cc >= 0.0;
  return {__fma_rd(cc, pos ? p.lo : p.hi, acc.lo), __fma_ru(cc, pos ? p.hi : p.lo, acc.hi)};
}

// A TERM's contribution: its value (term_value) added into / subtracted from
// / starting the chain, or, fused, its product folded in with fma_into.
template <typename T, typename V, bool kFused>
__device__ __forceinline__ Iv<T> term_operand(const Instr& cur, int sub, const V& vars)
{
  if (fused_term<T, kFused>(sub)) return term_product<T, V>(cur, sub, vars);
  return term_value<T, V>(cur, sub, vars);
}

template <typename T, bool kFused>
__device__ __forceinline__ Iv<T> term_apply(Iv<T> acc, const Instr& cur, int sub, Iv<T> p)
{
  if constexpr (kFused && sizeof(T) == 8) {
    if (fused_term<T, kFused>(sub)) return fma_into(acc, cur.c, p, (sub & kTermSub) != 0);
  }
  if (sub & kTermInit) return p;
  return (sub & kTermSub) ? iv_sub(acc, p) : iv_add(acc, p);
}

// Where the interval interpreter reads instruction pc: the program in
// global memory through the read-only cache, or a tile of it staged in
// shared memory (instructions [base, base + tile length) at tile[0..]).
struct GlobalCode {
  const Instr* prog;
  __device__ __forceinline__ Instr operator()(int pc) const { return load_instr(prog, pc); }
};
struct SharedCode {
  const Instr* tile;
  int base;
  __device__ __forceinline__ Instr operator()(int pc) const { return tile[pc - base]; }
};

// Interval interpretation of instructions [pc0, pc1) for this thread's box,
// continuing the accumulator `acc`: variables from `vars` (anything with
// var(v) -> Iv<T>), program slots in `t`.  Checks fold into `out` with AND /
// OR, so ranges may run in any order.
template <typename T, typename V, typename Code, bool kFused = false>
__device__ __forceinline__ void interval_range_from(const Code& code_at, int pc0, int pc1, const V& vars,
                                                    const Tile<T>& t, Verdict<T>& out, Iv<T>& acc)
{
  int pc = pc0;
  while (pc < pc1) {
    // two terms in a row: both products before the first add, so the two
    // interval products (and their variable loads) overlap
    if (pc + 2 <= pc1) {
      const Instr c0 = code_at(pc), c1 = code_at(pc + 1);
      if ((c0.head & 7) == kOpTerm && (c1.head & 7) == kOpTerm) {
        const int s0 = c0.head >> 3, s1 = c1.head >> 3;
        const Iv<T> p0 = term_operand<T, V, kFused>(c0, s0, vars);
        const Iv<T> p1 = term_operand<T, V, kFused>(c1, s1, vars);
        acc = term_apply<T, kFused>(acc, c0, s0, p0);
        acc = term_apply<T, kFused>(acc, c1, s1, p1);
        pc += 2;
        continue;
      }
    }
    const Instr cur = code_at(pc);
    ++pc;
    const int code = cur.head & 7;
    const int sub = cur.head >> 3;
    switch (code) {
      case kOpTerm: {
        acc = term_apply<T, kFused>(acc, cur, sub, term_operand<T, V, kFused>(cur, sub, vars));
        break;
      }
      case kOpGeneric: {
        const Iv<T> a = fetch(vars, t, acc, cur, cur.modes & 3, cur.a);
        const Iv<T> b = fetch(vars, t, acc, cur, (cur.modes >> 2) & 3, cur.b);
        t.set_slot(cur.dst, iv_generic<T>((uint8_t)sub, a, b, (int)(int16_t)cur.b));
        break;
      }
      case kOpStoreAcc:
        t.set_slot(cur.dst, acc);
        break;
      case kOpLoadAcc:
        acc = fetch(vars, t, acc, cur, cur.modes & 3, cur.a);
        break;
      case kOpConstToSlot:
        t.set_slot(cur.dst, const_of<T>(cur));
        break;
      case kOpCheck: {
        const Iv<T> v = fetch(vars, t, acc, cur, cur.modes & 3, cur.a);
        // rhs is kept in FP64 for both precisions; compare in FP64 exactly
        const double rhs = cur.c;
        const double lo = (double)v.lo, hi = (double)v.hi;
        if (sub == 0) {
          out.feasible = out.feasible && (lo <= rhs);
          out.excluded = out.excluded || (lo > rhs);
        } else {
          out.feasible = out.feasible && (lo <= rhs && rhs <= hi);
          out.excluded = out.excluded || (lo > rhs || hi < rhs);
        }
        break;
      }
      case kOpObjective:
        out.obj = fetch(vars, t, acc, cur, cur.modes & 3, cur.a);
        out.has_obj = true;
        break;
      default:
        break;
    }
  }
}

// The same from a zero accumulator, reading the program in global memory.
template <typename T, typename V, bool kFused = false>
__device__ __forceinline__ void interval_range(const Instr* __restrict__ prog, int pc0, int pc1, const V& vars,
                                               const Tile<T>& t, Verdict<T>& out)
{
  Iv<T> acc = {T(0), T(0)};
  interval_range_from<T, V, GlobalCode, kFused>(GlobalCode{prog}, pc0, pc1, vars, t, out, acc);
}

template <typename T, typename V, bool kFused = false>
__device__ Verdict<T> run_interval(const Instr* __restrict__ prog, int len, const V& vars, const Tile<T>& t)
{
  Verdict<T> out = verdict_init<T>();
  interval_range<T, V, kFused>(prog, 0, len, vars, t, out);
  return out;
}

// ---- incremental chain evaluation (the lazy form's FP32 children) ----
// acc <- acc + (the instruction's term) for a chain instruction (a TERM,
// whose kTermInit only means "first of its chain", or a LoadAcc), so a
// chain can be summed in any grouping of its terms: every partial sum is
// an outward-rounded enclosure of the exact one.
template <typename T, typename V>
__device__ __forceinline__ Iv<T> chain_add(Iv<T> acc, const Instr& cur, const V& vars)
{
  const int code = cur.head & 7, sub = cur.head >> 3;
  if (code == kOpTerm) {
    const Iv<T> p = term_value<T, V>(cur, sub, vars);
    return (sub & kTermSub) ? iv_sub(acc, p) : iv_add(acc, p);
  }
  const int mode = cur.modes & 3;  // LoadAcc: a variable or a constant
  return iv_add(acc, mode == kModeVar ? vars.var(cur.a) : const_of<T>(cur));
}

// The checks and objective [pc0, pc1) that read a chain's value `acc`
// (interval_range's kOpCheck / kOpObjective).
template <typename T, typename V>
__device__ __forceinline__ void chain_tail(const Instr* __restrict__ prog, int pc0, int pc1, const V& vars,
                                           Iv<T> acc, Verdict<T>& out)
{
  for (int pc = pc0; pc < pc1; ++pc) {
    const Instr cur = load_instr(prog, pc);
    const int code = cur.head & 7, sub = cur.head >> 3, mode = cur.modes & 3;
    const Iv<T> v = mode == kModeAcc ? acc : (mode == kModeVar ? vars.var(cur.a) : const_of<T>(cur));
    if (code == kOpCheck) {
      const double rhs = cur.c;
      const double lo = (double)v.lo, hi = (double)v.hi;
      if (sub == 0) {
        out.feasible = out.feasible && (lo <= rhs);
        out.excluded = out.excluded || (lo > rhs);
      } else {
        out.feasible = out.feasible && (lo <= rhs && rhs <= hi);
        out.excluded = out.excluded || (lo > rhs || hi < rhs);
      }
    } else if (code == kOpObjective) {
      out.obj = v;
      out.has_obj = true;
    }
  }
}

// Segments of `lane` in a group of 2^l lanes: [b, e) indexes the (pc0, pc1)
// pairs of the level's block of the lane schedule (Program::sched).
struct LaneSegs {
  const int32_t* pairs;
  int b, e;
};
__device__ __forceinline__ LaneSegs lane_segments(const int32_t* __restrict__ sched, int l, int lane)
{
  const int32_t* L = sched + __ldg(sched + l);
  LaneSegs s;
  s.b = __ldg(L + lane);
  s.e = __ldg(L + lane + 1);
  s.pairs = L + (1 << l) + 1;
  return s;
}

// One lane of a group of 2^l lanes that share a box: it runs its share of
// the program's segments (independent sum chains, each starting with an
// accumulator reset).  Every instruction performs the same roundings as in
// the whole-program run, so the group's combined verdict (group_verdict) is
// bit-identical to run_interval's.
template <typename T, typename V, bool kFused = false>
__device__ Verdict<T> run_interval_lane(const Instr* __restrict__ prog, const int32_t* __restrict__ sched, int l,
                                        int lane, const V& vars, const Tile<T>& t)
{
  Verdict<T> out = verdict_init<T>();
  const LaneSegs ls = lane_segments(sched, l, lane);
  for (int j = ls.b; j < ls.e; ++j)
    interval_range<T, V, kFused>(prog, __ldg(ls.pairs + 2 * j), __ldg(ls.pairs + 2 * j + 1), vars, t, out);
  return out;
}

// Combines the verdicts of a group of G consecutive lanes (G a power of two
// up to 32); every lane of the warp must call it with the same G.
template <typename T>
__device__ __forceinline__ Verdict<T> group_verdict(Verdict<T> v, int G)
{
  for (int off = 1; off < G; off <<= 1) {
    const int f = __shfl_xor_sync(0xffffffffu, (int)v.feasible, off);
    const int e = __shfl_xor_sync(0xffffffffu, (int)v.excluded, off);
    const int h = __shfl_xor_sync(0xffffffffu, (int)v.has_obj, off);
    const T lo = __shfl_xor_sync(0xffffffffu, v.obj.lo, off);
    const T hi = __shfl_xor_sync(0xffffffffu, v.obj.hi, off);
    v.feasible = v.feasible && f;
    v.excluded = v.excluded || e;
    if (!v.has_obj && h) {
      v.obj = {lo, hi};
      v.has_obj = true;
    }
  }
  return v;
}

// Lanes per box for `n` boxes: the largest power of two G <= g_max with
// n * G <= capacity (the threads the launch keeps resident), so a small
// frontier spreads each box over several lanes and a large one keeps one
// lane per box.
// Returns log2 of the group size.
__device__ __forceinline__ int lanes_per_box(uint64_t n, uint64_t capacity, int g_max)
{
  int l = 0;
  while ((1 << l) < g_max && n * (uint64_t)(2 << l) <= capacity) ++l;
  return l;
}

// Variables held in the tile's own planes.
template <typename T>
__device__ Verdict<T> run_interval(const Instr* __restrict__ prog, int len, const Tile<T>& t)
{
  return run_interval<T, Tile<T>>(prog, len, t, t);
}

// Point interpretation (FP64 round-to-nearest) for this thread's point,
// held in t.lo; slots use t.slo.  Feasibility follows the point predicates
// of graph/kernels.cuh:283-320 (LE exact; EQ abs 1e-8 / rel 1e-6).
__device__ __forceinline__ bool almost_equal(double a, double b)
{
  const double diff = fabs(__dsub_rn(a, b));
  if (diff <= 1e-8) return true;
  return diff <= __dmul_rn(1e-6, fmax(fabs(a), fabs(b)));
}

struct PointVerdict {
  double obj;
  bool feasible;
  bool has_obj;
};

__device__ __forceinline__ double pfetch(const Tile<double>& t, double acc, const Instr& ins, int mode, int idx)
{
  switch (mode) {
    case kModeSlot: return t.slo[idx * t.stride + t.tid];
    case kModeVar: return t.lo[idx * t.stride + t.tid];
    case kModeAcc: return acc;
    default: return ins.c;
  }
}

// the point evaluation's products (round to nearest), on the integer pipe
// as CMN_FP64_EMU selects: bit 3 the variable products, bit 4 the products
// by a coefficient
__device__ __forceinline__ double pt_mul_var(double a, double b)
{
  return (CMN_FP64_EMU & 8) ? emu::mul_rn(a, b) : __dmul_rn(a, b);
}
__device__ __forceinline__ double pt_mul_const(double c, double p)
{
  return (CMN_FP64_EMU & 16) ? emu::mul_rn(c, p) : __dmul_rn(c, p);
}

// One chain term of the FP64 point program: acc (+|-) [c *] (x_a [* x_b]),
// each operation rounded to nearest (the products as pt_mul_* give them).
// xb is read for every term: b == a for sqr(x_a) and x_a terms.
__device__ __forceinline__ double term64(double acc, const Instr& cur, double xa, double xb)
{
  using A = Arith<double>;
  const int sub = cur.head >> 3;
  const int pk = sub & kTermPMask;
  double p;
  if (pk == kTermProd) {
    p = pt_mul_var(xa, xb);
  } else if (pk == kTermSqr) {
    p = pt_mul_var(xa, xa);
  } else {
    p = xa;
  }
  if (sub & kTermHasC) p = pt_mul_const(cur.c, p);
  if (sub & kTermInit) return p;
  return (sub & kTermSub) ? A::sub_rn(acc, p) : A::add_rn(acc, p);
}

// Terms the FP64 point interpreter takes at once when the next
// instructions are all terms.
constexpr int kPointRun64 = 4;

__device__ __forceinline__ void point_range(const Instr* __restrict__ prog, int pc0, int pc1, const Tile<double>& t,
                                            PointVerdict& out)
{
  double acc = 0.0;
  int pc = pc0;
  while (pc < pc1) {
    // a run of kPointRun64 terms: their words and variables are loaded
    // before the first add, so the loads of a run overlap
    if (pc + kPointRun64 <= pc1) {
      Instr c[kPointRun64];
      int all = 0;
#pragma unroll
      for (int q = 0; q < kPointRun64; ++q) {
        c[q] = load_instr(prog, pc + q);
        all |= (c[q].head & 7) ^ kOpTerm;
      }
      if (all == 0) {
        double xa[kPointRun64], xb[kPointRun64];
#pragma unroll
        for (int q = 0; q < kPointRun64; ++q) {
          xa[q] = t.lo[c[q].a * t.stride + t.tid];
          xb[q] = t.lo[c[q].b * t.stride + t.tid];
        }
#pragma unroll
        for (int q = 0; q < kPointRun64; ++q) acc = term64(acc, c[q], xa[q], xb[q]);
        pc += kPointRun64;
        continue;
      }
    }
    const Instr cur = load_instr(prog, pc);
    ++pc;
    const int code = cur.head & 7;
    const int sub = cur.head >> 3;
    switch (code) {
      case kOpTerm:
        acc = term64(acc, cur, t.lo[cur.a * t.stride + t.tid], t.lo[cur.b * t.stride + t.tid]);
        break;
      case kOpGeneric: {
        const double a = pfetch(t, acc, cur, cur.modes & 3, cur.a);
        const double b = pfetch(t, acc, cur, (cur.modes >> 2) & 3, cur.b);
        t.slo[cur.dst * t.stride + t.tid] = pt_generic((uint8_t)sub, a, b, (int)(int16_t)cur.b);
        break;
      }
      case kOpStoreAcc:
        t.slo[cur.dst * t.stride + t.tid] = acc;
        break;
      case kOpLoadAcc:
        acc = pfetch(t, acc, cur, cur.modes & 3, cur.a);
        break;
      case kOpConstToSlot:
        t.slo[cur.dst * t.stride + t.tid] = cur.c;
        break;
      case kOpCheck: {
        const double v = pfetch(t, acc, cur, cur.modes & 3, cur.a);
        const bool ok = (sub == 0) ? (v <= cur.c) : almost_equal(v, cur.c);
        out.feasible = out.feasible && ok;
        // an infeasible point counts as +inf whatever the rest gives: stop
        if (!ok) return;
        break;
      }
      case kOpObjective:
        out.obj = pfetch(t, acc, cur, cur.modes & 3, cur.a);
        out.has_obj = true;
        break;
      default:
        break;
    }
  }
}

__device__ inline PointVerdict run_point(const Instr* __restrict__ prog, int len, const Tile<double>& t)
{
  PointVerdict out;
  out.obj = Arith<double>::nan();
  out.feasible = true;
  out.has_obj = false;
  point_range(prog, 0, len, t, out);
  return out;
}

// The whole point program on one lane: with a lane schedule, its level-0
// segment order (the objective's segments last, so an infeasible point
// stops early), else program order.
__device__ inline PointVerdict run_point_ordered(const Instr* __restrict__ prog, int len,
                                                 const int32_t* __restrict__ sched, const Tile<double>& t);

// One lane of a group sharing a point (see run_interval_lane).
__device__ inline PointVerdict run_point_lane(const Instr* __restrict__ prog, const int32_t* __restrict__ sched, int l,
                                              int lane, const Tile<double>& t)
{
  PointVerdict out;
  out.obj = Arith<double>::nan();
  out.feasible = true;
  out.has_obj = false;
  const LaneSegs ls = lane_segments(sched, l, lane);
  for (int j = ls.b; j < ls.e && out.feasible; ++j)
    point_range(prog, __ldg(ls.pairs + 2 * j), __ldg(ls.pairs + 2 * j + 1), t, out);
  return out;
}

__device__ inline PointVerdict run_point_ordered(const Instr* __restrict__ prog, int len,
                                                 const int32_t* __restrict__ sched, const Tile<double>& t)
{
  return sched != nullptr ? run_point_lane(prog, sched, 0, 0, t) : run_point(prog, len, t);
}

__device__ __forceinline__ PointVerdict group_point_verdict(PointVerdict v, int G)
{
  for (int off = 1; off < G; off <<= 1) {
    const int f = __shfl_xor_sync(0xffffffffu, (int)v.feasible, off);
    const int h = __shfl_xor_sync(0xffffffffu, (int)v.has_obj, off);
    const double o = __shfl_xor_sync(0xffffffffu, v.obj, off);
    v.feasible = v.feasible && f;
    if (!v.has_obj && h) {
      v.obj = o;
      v.has_obj = true;
    }
  }
  return v;
}

// ---- FP32 point evaluation: the lazy form's sample screen ----
// One round-to-nearest FP32 operation per DAG node, the point's variables
// and the program's constants rounded to nearest (Program::code32p);
// constraints by the point predicates on the FP32 values widened to FP64.
// It only ranks sample points: the point that wins a chunk is evaluated
// again in FP64 (point_range) before it can become the incumbent.
struct PointVerdict32 {
  float obj;
  bool feasible;
  bool has_obj;
};

// x^k by binary powering, round to nearest at every step (k > 0)
__device__ __forceinline__ float pt32_powu(float a, int k)
{
  float r = 1.0f, base = a;
  while (k > 0) {
    if (k & 1) r = __fmul_rn(r, base);
    k >>= 1;
    if (k > 0) base = __fmul_rn(base, base);
  }
  return r;
}

__device__ __forceinline__ float pt32_generic(uint8_t op, float a, float b, int k)
{
  switch (op) {
    case kGAdd: return __fadd_rn(a, b);
    case kGSub: return __fsub_rn(a, b);
    case kGMul: return __fmul_rn(a, b);
    case kGDiv: return __fdiv_rn(a, b);
    case kGSqr: return __fmul_rn(a, a);
    case kGNeg: return -a;
    case kGSqrt: return __fsqrt_rn(a);
    case kGPowN: return k == 0 ? 1.0f : (k > 0 ? pt32_powu(a, k) : __fdiv_rn(1.0f, pt32_powu(a, -k)));
    case kGAbs: return fabsf(a);
    case kGMin: return fminf(a, b);
    case kGMax: return fmaxf(a, b);
    case kGExp: return expf(a);
    case kGLog: return logf(a);
    case kGSin: return sinf(a);
    case kGCos: return cosf(a);
    case kGTanh: return tanhf(a);
    case kGPow: return powf(a, b);
    default: return Arith<float>::nan();
  }
}

__device__ __forceinline__ float pfetch32(const Tile<float>& t, float acc, const Instr& ins, int mode, int idx)
{
  switch (mode) {
    case kModeSlot: return t.slo[idx * t.stride + t.tid];
    case kModeVar: return t.lo[idx * t.stride + t.tid];
    case kModeAcc: return acc;
    default: return ins.c32.clo;
  }
}

// One chain term of the FP32 point program on one point: acc (+|-)
// [c *] (x_a [* x_b]), each operation rounded to nearest; `cbits` is the
// coefficient's bit pattern.
__device__ __forceinline__ float term32(float acc, int sub, float xa, float xb, int cbits)
{
  float p = (sub & kTermPMask) == kTermVar ? xa : __fmul_rn(xa, xb);
  if (sub & kTermHasC) p = __fmul_rn(__int_as_float(cbits), p);
  return (sub & kTermInit) ? p : ((sub & kTermSub) ? __fsub_rn(acc, p) : __fadd_rn(acc, p));
}

// Terms the point interpreters take at once when the next instructions are
// all terms: their words and variables are loaded before the first add, so
// the loads of a run overlap.
constexpr int kTermRun = 8;

__device__ __forceinline__ void point_range32(const Instr* __restrict__ prog, int pc0, int pc1, const Tile<float>& t,
                                              PointVerdict32& out)
{
  float acc = 0.0f;
  // this thread's point column: variable v at x[v * stride]
  const float* __restrict__ x = t.lo + t.tid;
  const int st = t.stride;
  const int4* __restrict__ code4 = reinterpret_cast<const int4*>(prog);
  int pc = pc0;
  while (pc < pc1) {
    // the common case first, straight from the instruction's words (head
    // in bits 0-7 of word 0, a and b in word 1, the coefficient in word 2):
    // a run of kTermRun terms, every load issued before the first add
    if (pc + kTermRun <= pc1) {
      int4 w[kTermRun];
      int all = 0;
#pragma unroll
      for (int q = 0; q < kTermRun; ++q) {
        w[q] = __ldg(code4 + pc + q);
        all |= (w[q].x & 7) ^ kOpTerm;
      }
      if (all == 0) {
        float xa[kTermRun], xb[kTermRun];
#pragma unroll
        for (int q = 0; q < kTermRun; ++q) {
          xa[q] = x[(int)((uint32_t)w[q].y & 0xffffu) * st];
          xb[q] = x[(int)((uint32_t)w[q].y >> 16) * st];  // b == a for sqr(x_a) and x_a terms
        }
#pragma unroll
        for (int q = 0; q < kTermRun; ++q) acc = term32(acc, (w[q].x >> 3) & 31, xa[q], xb[q], w[q].z);
        pc += kTermRun;
        continue;
      }
    }
    const int4 w = __ldg(code4 + pc);
    ++pc;
    if ((w.x & 7) == kOpTerm) {
      const uint32_t ab = (uint32_t)w.y;
      acc = term32(acc, (w.x >> 3) & 31, x[(int)(ab & 0xffffu) * st], x[(int)(ab >> 16) * st], w.z);
      continue;
    }
    Instr cur;
    memcpy(&cur, &w, sizeof(Instr));
    const int code = cur.head & 7;
    const int sub = cur.head >> 3;
    switch (code) {
      case kOpGeneric: {
        const float a = pfetch32(t, acc, cur, cur.modes & 3, cur.a);
        const float b = pfetch32(t, acc, cur, (cur.modes >> 2) & 3, cur.b);
        t.slo[cur.dst * t.stride + t.tid] = pt32_generic((uint8_t)sub, a, b, (int)(int16_t)cur.b);
        break;
      }
      case kOpStoreAcc:
        t.slo[cur.dst * t.stride + t.tid] = acc;
        break;
      case kOpLoadAcc:
        acc = pfetch32(t, acc, cur, cur.modes & 3, cur.a);
        break;
      case kOpConstToSlot:
        t.slo[cur.dst * t.stride + t.tid] = cur.c32.clo;
        break;
      case kOpCheck: {
        const double v = (double)pfetch32(t, acc, cur, cur.modes & 3, cur.a);
        const bool ok = (sub == 0) ? (v <= cur.c) : almost_equal(v, cur.c);
        out.feasible = out.feasible && ok;
        // an infeasible point ranks as +inf whatever the rest gives: stop
        if (!ok) return;
        break;
      }
      case kOpObjective:
        out.obj = pfetch32(t, acc, cur, cur.modes & 3, cur.a);
        out.has_obj = true;
        break;
      default:
        break;
    }
  }
}

// ---- region decode (region/decode.hpp:44-71), FMA form as compiled on
// the device, and the sampler (graph/subregion_sampler.cuh:53-120) ----
// The part of slot `s` that child `r` of a parent takes: (r / prefix) %
// width. The branching policy's plans have power-of-two widths, which take
// a shift and a mask instead of a 64-bit division.
__device__ __forceinline__ uint64_t slot_part(uint64_t r, const SlotPlan& s)
{
  if (((s.prefix & (s.prefix - 1)) | (s.width & (s.width - 1))) == 0)
    return (r >> (__ffsll((long long)s.prefix) - 1)) & (s.width - 1);
  return (r / s.prefix) % s.width;
}

// bounds of part `part` of slot `s` over the parent's [plo, phi]
__device__ __forceinline__ void slot_bounds(const SlotPlan& s, double plo, double phi, uint64_t part, double& lo,
                                            double& hi)
{
  if (s.kind == 2 || s.kind == 3) {  // IntegerEnumerate / BinaryEnumerate
    double value = __dadd_rn(s.step, (double)part);  // step = ceil(plo)
    if (value > phi) value = phi;
    lo = value;
    hi = value;
    return;
  }
  lo = __fma_rn(s.step, (double)part, plo);
  hi = (part + 1 == s.width) ? phi : __fma_rn(s.step, (double)(part + 1), plo);
}

__device__ __forceinline__ uint64_t sample_hash(uint64_t vid, uint64_t i, uint64_t region, uint64_t salt)
{
  uint64_t x = vid * 0x9e3779b97f4a7c15ULL;
  x ^= i * 0xbf58476d1ce4e5b9ULL;
  x ^= region * 0x94d049bb133111ebULL;
  x ^= salt * 0xd6e8feb86659fd93ULL;
  x += 0x9e3779b97f4a7c15ULL;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
  x ^= x >> 31;
  return x;
}

__device__ __forceinline__ double sample_value(bool discrete, double lb, double ub, uint64_t vid, uint64_t i,
                                               uint64_t region, uint64_t salt)
{
  const uint64_t x = sample_hash(vid, i, region, salt);
  if (!discrete) {
    const double u = __dmul_rn(__ull2double_rn(x >> 11), 1.0 / 9007199254740992.0);
    return __fma_rn(u, __dsub_rn(ub, lb), lb);
  }
  const double lo = ceil(lb), hi = floor(ub);
  if (hi < lo) return lo;
  const uint64_t count = (uint64_t)__double2ull_rz(__dsub_rn(hi, lo)) + 1;
  const uint64_t idx = x % count;
  return __dadd_rn(lo, __ull2double_rn(idx));
}

// Total order on doubles for selection keys (NaN last), from the raw bits.
// The pool passes stay on the integer pipe: FP64 instructions, even
// compares, issue at a small fraction of the integer rate on this part.
__device__ __forceinline__ uint64_t bits_key(uint64_t u)
{
  if ((u & 0x7fffffffffffffffULL) > 0x7ff0000000000000ULL) return ~0ULL;
  return (u >> 63) ? ~u : (u | 0x8000000000000000ULL);
}

__device__ __forceinline__ uint64_t lb_key(double x) { return bits_key((uint64_t)__double_as_longlong(x)); }

// IEEE `a <= b` on the raw bits of two doubles (false if either is NaN;
// -0 equals +0), on the integer pipe.
__device__ __forceinline__ bool bits_le(uint64_t a, uint64_t b)
{
  const uint64_t am = a & 0x7fffffffffffffffULL, bm = b & 0x7fffffffffffffffULL;
  if (am > 0x7ff0000000000000ULL || bm > 0x7ff0000000000000ULL) return false;
  return bits_key(am == 0 ? 0 : a) <= bits_key(bm == 0 ? 0 : b);
}

// IEEE `a < b` on the raw bits, as bits_le.
__device__ __forceinline__ bool bits_lt(uint64_t a, uint64_t b)
{
  const uint64_t am = a & 0x7fffffffffffffffULL, bm = b & 0x7fffffffffffffffULL;
  if (am > 0x7ff0000000000000ULL || bm > 0x7ff0000000000000ULL) return false;
  return bits_key(am == 0 ? 0 : a) < bits_key(bm == 0 ? 0 : b);
}

__device__ __forceinline__ uint64_t dbits(double x) { return (uint64_t)__double_as_longlong(x); }

}  // namespace cmn
