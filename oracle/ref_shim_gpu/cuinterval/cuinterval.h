// Stand-in for the operator set of the un-vendored neilkichler/cuinterval
// library, written for this repository so that the reference's CUDA graph
// backend (backend/graph/ops.cuh:24-355, kernels.cuh:257-261) compiles and
// runs on the GPU host.
//
// TEST INFRASTRUCTURE ONLY: results of the reference's graph structure with
// these operators are labelled "reference graph structure + the build's
// directed-rounding ops".
//
// Add, Sub, Mul (interval x interval and with a scalar on either side),
// Sqr, Neg, Div, Sqrt, Abs, Min and Max return the tightest enclosure under
// IEEE-754 directed rounding.  The product uses the classic branch-per-sign-
// case table, as interval libraries for GPUs do, written independently of
// the branch-free corner selection of the library under test: two
// implementations of the same unique result.  Exp, Log, Sin, Cos, Tanh and
// Pow are enclosures: the
// CUDA math function at each end, widened outward by kWiden ulps, with the
// interior extrema of Sin/Cos added; they are not tightest.
#pragma once

#include <cmath>

#include <cuinterval/interval.h>

namespace cu
{
namespace detail
{
constexpr int kWiden = 3;

__device__ inline double add_d(double a, double b) { return __dadd_rd(a, b); }
__device__ inline double add_u(double a, double b) { return __dadd_ru(a, b); }
__device__ inline double sub_d(double a, double b) { return __dsub_rd(a, b); }
__device__ inline double sub_u(double a, double b) { return __dsub_ru(a, b); }
__device__ inline double mul_d(double a, double b) { return __dmul_rd(a, b); }
__device__ inline double mul_u(double a, double b) { return __dmul_ru(a, b); }
__device__ inline double div_d(double a, double b) { return __ddiv_rd(a, b); }
__device__ inline double div_u(double a, double b) { return __ddiv_ru(a, b); }
__device__ inline double sqrt_d(double a) { return __dsqrt_rd(a); }
__device__ inline double sqrt_u(double a) { return __dsqrt_ru(a); }
__device__ inline float add_d(float a, float b) { return __fadd_rd(a, b); }
__device__ inline float add_u(float a, float b) { return __fadd_ru(a, b); }
__device__ inline float sub_d(float a, float b) { return __fsub_rd(a, b); }
__device__ inline float sub_u(float a, float b) { return __fsub_ru(a, b); }
__device__ inline float mul_d(float a, float b) { return __fmul_rd(a, b); }
__device__ inline float mul_u(float a, float b) { return __fmul_ru(a, b); }
__device__ inline float div_d(float a, float b) { return __fdiv_rd(a, b); }
__device__ inline float div_u(float a, float b) { return __fdiv_ru(a, b); }
__device__ inline float sqrt_d(float a) { return __fsqrt_rd(a); }
__device__ inline float sqrt_u(float a) { return __fsqrt_ru(a); }

template<typename T>
__device__ inline T inf() { return T(INFINITY); }
template<typename T>
__device__ inline T qnan() { return T(NAN); }

template<typename T>
__device__ inline T lo_of(T a, T b) { return a < b ? a : b; }
template<typename T>
__device__ inline T hi_of(T a, T b) { return a > b ? a : b; }

// endpoint products: 0 * inf is 0 for interval bounds
template<typename T>
__device__ inline T pmul_d(T a, T b) { return (a == T(0) || b == T(0)) ? T(0) : mul_d(a, b); }
template<typename T>
__device__ inline T pmul_u(T a, T b) { return (a == T(0) || b == T(0)) ? T(0) : mul_u(a, b); }

template<typename T>
__device__ inline T down(T x, int k)
{
  for (int i = 0; i < k; ++i) x = std::nextafter(x, -inf<T>());
  return x;
}
template<typename T>
__device__ inline T up(T x, int k)
{
  for (int i = 0; i < k; ++i) x = std::nextafter(x, inf<T>());
  return x;
}
template<typename T>
__device__ inline T clamp(T x, T lo, T hi) { return x < lo ? lo : (x > hi ? hi : x); }
}  // namespace detail

template<typename T>
__device__ inline interval<T> operator+(interval<T> a, interval<T> b)
{
  return {detail::add_d(a.lb, b.lb), detail::add_u(a.ub, b.ub)};
}
template<typename T>
__device__ inline interval<T> operator+(interval<T> a, T b) { return a + interval<T>(b); }
template<typename T>
__device__ inline interval<T> operator+(T a, interval<T> b) { return interval<T>(a) + b; }

template<typename T>
__device__ inline interval<T> operator-(interval<T> a, interval<T> b)
{
  return {detail::sub_d(a.lb, b.ub), detail::sub_u(a.ub, b.lb)};
}
template<typename T>
__device__ inline interval<T> operator-(interval<T> a, T b) { return a - interval<T>(b); }
template<typename T>
__device__ inline interval<T> operator-(T a, interval<T> b) { return interval<T>(a) - b; }

template<typename T>
__device__ inline interval<T> operator-(interval<T> a) { return {-a.ub, -a.lb}; }

// The nine sign cases of the endpoint-product table (Hickey, Ju and van
// Emden, "Interval arithmetic: from principles to implementation", JACM
// 2001): two directed products, four only when both operands contain zero
// in their interior.
template<typename T>
__device__ inline interval<T> operator*(interval<T> a, interval<T> b)
{
  using namespace detail;
  const T z = T(0);
  if (a.lb >= z) {
    if (b.lb >= z) return {pmul_d(a.lb, b.lb), pmul_u(a.ub, b.ub)};
    if (b.ub <= z) return {pmul_d(a.ub, b.lb), pmul_u(a.lb, b.ub)};
    return {pmul_d(a.ub, b.lb), pmul_u(a.ub, b.ub)};
  }
  if (a.ub <= z) {
    if (b.lb >= z) return {pmul_d(a.lb, b.ub), pmul_u(a.ub, b.lb)};
    if (b.ub <= z) return {pmul_d(a.ub, b.ub), pmul_u(a.lb, b.lb)};
    return {pmul_d(a.lb, b.ub), pmul_u(a.lb, b.lb)};
  }
  if (b.lb >= z) return {pmul_d(a.lb, b.ub), pmul_u(a.ub, b.ub)};
  if (b.ub <= z) return {pmul_d(a.ub, b.lb), pmul_u(a.lb, b.lb)};
  return {lo_of(pmul_d(a.lb, b.ub), pmul_d(a.ub, b.lb)), hi_of(pmul_u(a.lb, b.lb), pmul_u(a.ub, b.ub))};
}
template<typename T>
__device__ inline interval<T> operator*(interval<T> a, T b) { return a * interval<T>(b); }
template<typename T>
__device__ inline interval<T> operator*(T a, interval<T> b) { return interval<T>(a) * b; }

template<typename T>
__device__ inline interval<T> operator/(interval<T> a, interval<T> b)
{
  using namespace detail;
  if (b.lb > T(0) || b.ub < T(0)) {
    const T l = lo_of(lo_of(div_d(a.lb, b.lb), div_d(a.lb, b.ub)), lo_of(div_d(a.ub, b.lb), div_d(a.ub, b.ub)));
    const T u = hi_of(hi_of(div_u(a.lb, b.lb), div_u(a.lb, b.ub)), hi_of(div_u(a.ub, b.lb), div_u(a.ub, b.ub)));
    return {l, u};
  }
  if (b.lb == T(0) && b.ub == T(0)) return {qnan<T>(), qnan<T>()};
  if (b.lb == T(0)) {
    if (a.lb >= T(0)) return {div_d(a.lb, b.ub), inf<T>()};
    if (a.ub <= T(0)) return {-inf<T>(), div_u(a.ub, b.ub)};
  } else if (b.ub == T(0)) {
    if (a.lb >= T(0)) return {-inf<T>(), div_u(a.lb, b.lb)};
    if (a.ub <= T(0)) return {div_d(a.ub, b.lb), inf<T>()};
  }
  return {-inf<T>(), inf<T>()};
}
template<typename T>
__device__ inline interval<T> operator/(interval<T> a, T b) { return a / interval<T>(b); }
template<typename T>
__device__ inline interval<T> operator/(T a, interval<T> b) { return interval<T>(a) / b; }

template<typename T>
__device__ inline interval<T> sqr(interval<T> a)
{
  using namespace detail;
  if (a.lb >= T(0)) return {pmul_d(a.lb, a.lb), pmul_u(a.ub, a.ub)};
  if (a.ub <= T(0)) return {pmul_d(a.ub, a.ub), pmul_u(a.lb, a.lb)};
  const T m = hi_of(-a.lb, a.ub);
  return {T(0), pmul_u(m, m)};
}

template<typename T>
__device__ inline interval<T> abs(interval<T> a)
{
  if (a.lb >= T(0)) return a;
  if (a.ub <= T(0)) return -a;
  return {T(0), detail::hi_of(-a.lb, a.ub)};
}

template<typename T>
__device__ inline interval<T> min(interval<T> a, interval<T> b)
{
  return {detail::lo_of(a.lb, b.lb), detail::lo_of(a.ub, b.ub)};
}
template<typename T>
__device__ inline interval<T> max(interval<T> a, interval<T> b)
{
  return {detail::hi_of(a.lb, b.lb), detail::hi_of(a.ub, b.ub)};
}

template<typename T>
__device__ inline interval<T> sqrt(interval<T> a)
{
  if (a.ub < T(0)) return {detail::qnan<T>(), detail::qnan<T>()};
  return {a.lb > T(0) ? detail::sqrt_d(a.lb) : T(0), detail::sqrt_u(a.ub)};
}

template<typename T>
__device__ inline interval<T> exp(interval<T> a)
{
  using namespace detail;
  T l = down(std::exp(a.lb), kWiden), u = up(std::exp(a.ub), kWiden);
  return {l < T(0) ? T(0) : l, u};
}

template<typename T>
__device__ inline interval<T> log(interval<T> a)
{
  using namespace detail;
  if (a.ub < T(0)) return {qnan<T>(), qnan<T>()};
  const T l = a.lb <= T(0) ? -inf<T>() : down(std::log(a.lb), kWiden);
  const T u = a.ub == T(0) ? -inf<T>() : up(std::log(a.ub), kWiden);
  return {l, u};
}

template<typename T>
__device__ inline interval<T> tanh(interval<T> a)
{
  using namespace detail;
  return {clamp(down(std::tanh(a.lb), kWiden), T(-1), T(1)), clamp(up(std::tanh(a.ub), kWiden), T(-1), T(1))};
}

namespace detail
{
// Interval enclosure of cos(x + shift*pi/2) for shift 0 (cos) or -1 (sin):
// the ends, widened, plus +-1 wherever a multiple of pi (shifted) may lie
// inside.
template<typename T>
__device__ inline interval<T> trig(interval<T> a, bool is_sin)
{
  if (!(a.lb <= a.ub)) return {qnan<T>(), qnan<T>()};
  if (a.lb == -inf<T>() || a.ub == inf<T>()) return {T(-1), T(1)};
  const T pl = T(3.141592653589793), ph = up(pl, 1);
  const T f_lo = is_sin ? std::sin(a.lb) : std::cos(a.lb);
  const T f_hi = is_sin ? std::sin(a.ub) : std::cos(a.ub);
  T l = down(lo_of(f_lo, f_hi), kWiden), u = up(hi_of(f_lo, f_hi), kWiden);
  // critical points of cos at j*pi (value (-1)^j); of sin at (j+1/2)*pi
  T tl = lo_of(div_d(a.lb, pl), div_d(a.lb, ph));
  T th = hi_of(div_u(a.ub, pl), div_u(a.ub, ph));
  if (is_sin) {
    tl = sub_d(tl, T(0.5));
    th = sub_u(th, T(0.5));
  }
  const T jl = std::ceil(down(tl, 1)), jh = std::floor(up(th, 1));
  if (jh - jl >= T(2)) return {T(-1), T(1)};
  for (T j = jl; j <= jh; j = j + T(1)) {
    const bool even = std::fmod(std::fabs(j), T(2)) == T(0);
    if (even) u = T(1);
    else l = T(-1);
  }
  return {clamp(l, T(-1), T(1)), clamp(u, T(-1), T(1))};
}
}  // namespace detail

template<typename T>
__device__ inline interval<T> cos(interval<T> a) { return detail::trig(a, false); }
template<typename T>
__device__ inline interval<T> sin(interval<T> a) { return detail::trig(a, true); }

// x^n by binary powering with directed products (the same sequence as the
// repository's oracle), tightest for n in {0, 1, 2}.
template<typename T>
__device__ inline interval<T> pown(interval<T> a, int n)
{
  using namespace detail;
  if (n == 0) return {T(1), T(1)};
  if (n == 1) return a;
  if (n == 2) return sqr(a);
  if (n < 0) return interval<T>(T(1)) / pown(a, -n);
  auto pw_d = [](T x, int k) {
    T r = T(1), b = x;
    while (k > 0) {
      if (k & 1) r = pmul_d(r, b);
      k >>= 1;
      if (k > 0) b = pmul_d(b, b);
    }
    return r;
  };
  auto pw_u = [](T x, int k) {
    T r = T(1), b = x;
    while (k > 0) {
      if (k & 1) r = pmul_u(r, b);
      k >>= 1;
      if (k > 0) b = pmul_u(b, b);
    }
    return r;
  };
  if ((n & 1) == 0) {
    const T mig = a.lb > T(0) ? a.lb : (a.ub < T(0) ? -a.ub : T(0));
    const T mag = hi_of(a.lb < T(0) ? -a.lb : a.lb, a.ub < T(0) ? -a.ub : a.ub);
    return {pw_d(mig, n), pw_u(mag, n)};
  }
  return {a.lb >= T(0) ? pw_d(a.lb, n) : -pw_u(-a.lb, n), a.ub >= T(0) ? pw_u(a.ub, n) : -pw_d(-a.ub, n)};
}

// x^y for x clipped to [0, inf): exp(y * log(x)), an enclosure
template<typename T>
__device__ inline interval<T> pow(interval<T> a, interval<T> b)
{
  if (a.ub < T(0)) return {detail::qnan<T>(), detail::qnan<T>()};
  const interval<T> x = {a.lb < T(0) ? T(0) : a.lb, a.ub};
  return exp(b * log(x));
}
template<typename T>
__device__ inline interval<T> pow(interval<T> a, T b) { return pow(a, interval<T>(b)); }

namespace intrinsic
{
template<typename T>
__device__ inline T min(T a, T b) { return a < b ? a : b; }
template<typename T>
__device__ inline T max(T a, T b) { return a > b ? a : b; }
}  // namespace intrinsic
}  // namespace cu
