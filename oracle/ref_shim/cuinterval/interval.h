// Stand-in for the un-vendored neilkichler/cuinterval interval.h: the
// reference's host code only reads and writes the two bounds.
#pragma once

namespace cu
{
template<typename T>
struct interval
{
  T lb;
  T ub;
};
}  // namespace cu
