// Stand-in for the interval type of the un-vendored neilkichler/cuinterval
// library, for building the reference's CUDA graph backend on the GPU host.
//
// TEST INFRASTRUCTURE ONLY.  The reference reads and writes the two bounds
// (`lb`, `ub`), value-initialises arrays of intervals, builds point
// intervals from one scalar (`cu::interval<T>(b)`, graph/ops.cuh:143-207)
// and brace-initialises from two bounds.  The same definition serves the
// reference's host code compiled by g++ (its GAMS frontend), so every
// translation unit of the harness sees one interval type.
#pragma once

// host and device under nvcc; host code (the GAMS frontend) under g++
#ifdef __CUDACC__
#define CMN_SHIM_HD __host__ __device__
#else
#define CMN_SHIM_HD
#endif

namespace cu
{
template<typename T>
struct interval
{
  T lb;
  T ub;

  interval() = default;
  CMN_SHIM_HD constexpr interval(T point) : lb(point), ub(point) {}
  CMN_SHIM_HD constexpr interval(T lo, T hi) : lb(lo), ub(hi) {}
};
}  // namespace cu
