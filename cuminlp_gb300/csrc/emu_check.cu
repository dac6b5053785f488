// emu_check.cu -- device self-test of the integer-pipe binary64 operations
// (fp64_emu.cuh) against the FP64 instructions they stand in for.
#include <cuda_runtime.h>

#include <cfenv>
#include <cstdint>
#include <cstring>

#include "../../include/cuminlp_gb300.h"
#include "fp64_emu.cuh"

namespace cmn {

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x)
{
  x += 0x9e3779b97f4a7c15ULL;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
  return x ^ (x >> 31);
}

// Operand pairs by family:
//   0: any bit patterns (every class, all exponents)
//   1: normal numbers whose exponents differ by at most 70
//   2: b close to -a (cancellation in a + b, and in a - b for b close to a)
//   3: exponents near the top and the bottom of the normal range
//   4: significands with long runs of ones or zeros (carries, exact results)
__host__ __device__ __forceinline__ void operands(int family, uint64_t i, uint64_t seed, uint64_t& a, uint64_t& b)
{
  const uint64_t r0 = mix64(seed ^ (i * 4 + 0)), r1 = mix64(seed ^ (i * 4 + 1));
  const uint64_t r2 = mix64(seed ^ (i * 4 + 2)), r3 = mix64(seed ^ (i * 4 + 3));
  const uint64_t sa = r2 & (1ULL << 63), sb = (r2 << 1) & (1ULL << 63);
  switch (family) {
    case 0:
      a = r0;
      b = r1;
      break;
    case 1: {
      const uint64_t ea = 1 + (r2 >> 8) % 2046;
      const int64_t dd = (int64_t)((r3 >> 8) % 141) - 70;
      int64_t eb = (int64_t)ea + dd;
      eb = eb < 1 ? 1 : (eb > 2046 ? 2046 : eb);
      a = sa | (ea << 52) | (r0 & emu::kM52);
      b = sb | ((uint64_t)eb << 52) | (r1 & emu::kM52);
      break;
    }
    case 2: {
      const uint64_t ea = 1 + (r2 >> 8) % 2046;
      a = sa | (ea << 52) | (r0 & emu::kM52);
      const int64_t delta = (int64_t)(r1 % 2049) - 1024;  // a few ulps up or down
      const uint64_t flip = (r3 & 1) ? (1ULL << 63) : 0;
      b = (uint64_t)((int64_t)a + delta) ^ flip;
      if (r3 & 2) b = (b & ~emu::kM52) | ((b + (r1 >> 40)) & emu::kM52);
      break;
    }
    case 3: {
      const uint64_t top = (r2 >> 8) & 1;
      const uint64_t ea = top ? 2046 - (r2 >> 16) % 8 : 1 + (r2 >> 16) % 8;
      const uint64_t eb = top ? 1023 + (r3 >> 16) % 1024 : 1 + (r3 >> 16) % 1024;
      a = sa | (ea << 52) | (r0 & emu::kM52);
      b = sb | (eb << 52) | (r1 & emu::kM52);
      break;
    }
    default: {
      const uint64_t ea = 1 + (r2 >> 8) % 2046, eb = 1 + (r3 >> 8) % 2046;
      const int ra = (int)(r0 % 53), rb = (int)(r1 % 53);
      const uint64_t ma = (r0 >> 8) & 1 ? ((1ULL << ra) - 1) << (52 - ra) : ((1ULL << ra) - 1);
      const uint64_t mb = (r1 >> 8) & 1 ? ((1ULL << rb) - 1) << (52 - rb) : ((1ULL << rb) - 1);
      a = sa | (ea << 52) | (ma & emu::kM52);
      b = sb | (((r3 >> 20) & 1 ? ea : eb) << 52) | (mb & emu::kM52);
      break;
    }
  }
}

// the integer path's result of operation `op` (the device check and its host twin)
__host__ __device__ __forceinline__ bool emu_op(int op, uint64_t a, uint64_t b, uint64_t& r)
{
  const bool up = op & 1;
  return op < 2 ? emu::add_dir(a, b, up, r)
       : op < 4 ? emu::add_dir(a, b ^ (1ULL << 63), up, r)
       : op < 6 ? emu::mul_dir(a, b, up, r)
                : emu::mul_round(a, b, emu::kNearest, r);
}

// out[0] mismatches, out[1] results taken on the integer path, out[2]
// results checked
__global__ void emu_check_kernel(uint64_t n, uint64_t seed, int family, unsigned long long* out)
{
  unsigned long long bad = 0, handled = 0, total = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t a, b;
    operands(family, i, seed, a, b);
    const double x = emu::from_bits(a), y = emu::from_bits(b);
    const double hw[7] = {__dadd_rd(x, y), __dadd_ru(x, y), __dsub_rd(x, y), __dsub_ru(x, y),
                          __dmul_rd(x, y), __dmul_ru(x, y), __dmul_rn(x, y)};
    for (int op = 0; op < 7; ++op) {
      uint64_t r;
      const bool ok = emu_op(op, a, b, r);
      ++total;
      if (!ok) continue;
      ++handled;
      if (r != emu::bits(hw[op])) ++bad;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    bad += __shfl_down_sync(0xffffffffu, bad, off);
    handled += __shfl_down_sync(0xffffffffu, handled, off);
    total += __shfl_down_sync(0xffffffffu, total, off);
  }
  if ((threadIdx.x & 31) == 0) {
    if (bad) atomicAdd(out, bad);
    atomicAdd(out + 1, handled);
    atomicAdd(out + 2, total);
  }
}

// The host FPU's result of operation `op` in its rounding mode. The
// operands pass through volatile memory so that the arithmetic happens
// after the mode switch.
static uint64_t host_op(int op, uint64_t a, uint64_t b)
{
  volatile double x, y;
  double xs, ys;
  std::memcpy(&xs, &a, 8);
  std::memcpy(&ys, &b, 8);
  static const int modes[7] = {FE_DOWNWARD, FE_UPWARD, FE_DOWNWARD, FE_UPWARD, FE_DOWNWARD, FE_UPWARD, FE_TONEAREST};
  std::fesetround(modes[op]);
  x = xs;
  y = ys;
  volatile double r;
  if (op < 2) r = x + y;
  else if (op < 4) r = x - y;
  else r = x * y;
  const double out = r;
  std::fesetround(FE_TONEAREST);
  uint64_t u;
  std::memcpy(&u, &out, 8);
  return u;
}

}  // namespace cmn

// Host twin of cmn_fp64_emu_check: the same integer path compiled for the
// host, against the host FPU (IEEE binary64 in each rounding mode).
extern "C" cmn_status cmn_fp64_emu_check_host(uint64_t n, uint64_t seed, int32_t family, uint64_t* out3)
{
  if (!out3 || family < 0 || family > 4) return CMN_INVALID_CONFIGURATION;
  uint64_t bad = 0, handled = 0, total = 0;
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t a, b;
    cmn::operands(family, i, seed, a, b);
    for (int op = 0; op < 7; ++op) {
      uint64_t r;
      ++total;
      if (!cmn::emu_op(op, a, b, r)) continue;
      ++handled;
      if (r != cmn::host_op(op, a, b)) ++bad;
    }
  }
  out3[0] = bad;
  out3[1] = handled;
  out3[2] = total;
  return CMN_OK;
}

extern "C" cmn_status cmn_fp64_emu_op_host(int32_t op, double a, double b, double* out, int32_t* handled)
{
  if (!out || !handled || op < 0 || op > 6) return CMN_INVALID_CONFIGURATION;
  uint64_t ua, ub, r;
  std::memcpy(&ua, &a, 8);
  std::memcpy(&ub, &b, 8);
  const bool ok = cmn::emu_op(op, ua, ub, r);
  *handled = ok ? 1 : 0;
  if (ok) std::memcpy(out, &r, 8);
  return CMN_OK;
}

extern "C" cmn_status cmn_fp64_emu_check(uint64_t n, uint64_t seed, int32_t family, uint64_t* out3)
{
  if (!out3 || family < 0 || family > 4) return CMN_INVALID_CONFIGURATION;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 3 * sizeof(unsigned long long)) != cudaSuccess) return CMN_CUDA_ERROR;
  cudaError_t e = cudaMemset(d, 0, 3 * sizeof(unsigned long long));
  if (e == cudaSuccess) {
    cmn::emu_check_kernel<<<1024, 256>>>(n, seed, family, d);
    e = cudaGetLastError();
  }
  unsigned long long h[3] = {0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return CMN_CUDA_ERROR;
  for (int k = 0; k < 3; ++k) out3[k] = h[k];
  return CMN_OK;
}
