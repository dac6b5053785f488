// Stand-in for the interval type of the un-vendored neilkichler/cuinterval
// library, for building the reference's CUDA graph backend on the GPU host.
//
// TEST INFRASTRUCTURE ONLY.  The reference reads and writes the two bounds
// (`lb`, `ub`), value-initialises arrays of intervals, builds point
// intervals from one scalar (`cu::interval<T>(b)`, graph/ops.cuh:143-207)
// and brace-initialises from two bounds.
#pragma once

namespace cu
{
template<typename T>
struct interval
{
  T lb;
  T ub;

  interval() = default;
  __host__ __device__ constexpr interval(T point) : lb(point), ub(point) {}
  __host__ __device__ constexpr interval(T lo, T hi) : lb(lo), ub(hi) {}
};
}  // namespace cu
