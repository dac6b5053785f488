// noalloc.cu -- the sampler role without any device allocation.
//
// Some callers of this library cannot call cudaMalloc: processes whose
// device memory is handed out by a pool they do not own (the caching
// allocator of a serving framework, or a fixed arena carved out at start-up
// on a shared GPU), and code that must not grow the device footprint once
// it is running.  cmn_sample_noalloc gives them the sampler role -- the same
// kernels and the same results as a sampler built with cmn_role_build --
// with all of its device scratch in one fixed-size array of device memory
// declared in this file.  Every GPU that loads the library holds that array
// (kScratchBytes) until the process exits.
//
// The array's name is a host-side stand-in, not a device address, in host
// code: its address is looked up with cudaGetSymbolAddress, with the
// problem's device current, on every call (a lookup is cheap, and a device
// reset between calls cannot leave a stale address behind), and that
// pointer is what the kernels receive.
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>
#include <cstring>
#include <string>

#include "../../include/cuminlp_gb300.h"
#include "handles.hpp"
#include "kernels.cuh"
#include "launch.hpp"

using namespace cmn;

namespace {

constexpr size_t kScratchBytes = 512 * 1024;  // per device
constexpr int64_t kMaxVars = 8192;
constexpr int kMaxBlocks = 4096;

// slot table and parent record, staged together with one copy
struct StagedSlots {
  SlotPlan slots[64];
  ParentInfo info;
};

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of the scratch array on the current device.
static cmn_status scratch_on_device(unsigned char** out)
{
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess)
    return set_error(CMN_CUDA_ERROR, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
  *out = static_cast<unsigned char*>(p);
  return CMN_OK;
}

// Restores the caller's current device on every return path.
struct DeviceGuard {
  int prev = -1;
  ~DeviceGuard()
  {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

#define NA_CK(call)                                                                                            \
  do {                                                                                                         \
    cudaError_t e_ = (call);                                                                                   \
    if (e_ != cudaSuccess) return set_error(CMN_CUDA_ERROR, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

extern "C" cmn_status cmn_sample_noalloc(const cmn_problem* p, const uint8_t* slot_kinds, int64_t slot_count,
                                         uint64_t n_regions, uint64_t sample_points, const double* box,
                                         const uint64_t* var_ids, const uint64_t* widths, uint64_t salt,
                                         cmn_candidate* out, double* point, void* stream)
{
  if (!p || !out || !point || !box) return set_error(CMN_INVALID_CONFIGURATION, "null argument");
  const int64_t n = p->host.n_vars();
  if (n > kMaxVars)
    return set_error(CMN_INVALID_CONFIGURATION, "cmn_sample_noalloc handles at most " + std::to_string(kMaxVars) +
                                                    " variables; this problem has " + std::to_string(n));
  if (sample_points < 1) return set_error(CMN_INVALID_CONFIGURATION, "sample_points must be at least 1");
  if (slot_count < 0 || slot_count > 64) return set_error(CMN_SHAPE_MISMATCH, "slot_count must be within [0, 64]");
  if (slot_count > 0 && (!slot_kinds || !var_ids || !widths))
    return set_error(CMN_SHAPE_MISMATCH, "missing slot kinds, var_ids or widths");
  if (n_regions < 1 || n_regions > (1ULL << 32))
    return set_error(CMN_INVALID_CONFIGURATION, "n_regions must be within [1, 2^32]");

  StagedSlots staged;
  std::memset(&staged, 0, sizeof staged);
  uint64_t running = 1;
  for (int64_t j = 0; j < slot_count; ++j) {
    if (slot_kinds[j] > CMN_SLOT_BINARY_ENUMERATE) return set_error(CMN_INVALID_CONFIGURATION, "unknown slot kind");
    if (var_ids[j] >= (uint64_t)n) return set_error(CMN_SHAPE_MISMATCH, "var_id out of range");
    if (widths[j] < 1) return set_error(CMN_SHAPE_MISMATCH, "slot width must be at least 1");
    staged.slots[j] = SlotPlan{widths[j], running, widths[j], (uint32_t)var_ids[j], slot_kinds[j],
                               slot_step(slot_kinds[j], box[2 * var_ids[j]], box[2 * var_ids[j] + 1], widths[j])};
    running = running > UINT64_MAX / widths[j] ? UINT64_MAX : running * widths[j];
  }
  if (running != n_regions) return set_error(CMN_SHAPE_MISMATCH, "the product of widths does not equal n_regions");
  staged.info = ParentInfo{(uint32_t)slot_count, 0, n_regions};

  DeviceGuard guard;
  NA_CK(cudaGetDevice(&guard.prev));
  NA_CK(cudaSetDevice(p->device));
  NA_CK(ensure_kernel_attributes());
  unsigned char* base = nullptr;
  cmn_status st = scratch_on_device(&base);
  if (st != CMN_OK) return st;

  const int threads = kEvalThreads;
  const int lg_min = sample_lg_min((int)n, p->prog.n_slots, p->d_sched != nullptr, threads);
  const size_t smem = sample_smem_bytes((int)n, p->prog.n_slots, threads, lg_min);
  if (smem > (size_t)max_dynamic_smem())
    return set_error(CMN_INVALID_CONFIGURATION,
                     "the sampler's point columns (" + std::to_string(smem) + " B per block) do not fit in shared "
                     "memory; a program with shared slots keeps one column of n_vars + slots doubles per thread");
  int occ = sample_kernel_occupancy(smem, threads);
  if (occ < 1) occ = 1;
  const uint64_t need = (n_regions + threads - 1) / threads;
  uint64_t grid64 = (uint64_t)sm_count() * occ;
  if (grid64 > need) grid64 = need;
  if (grid64 > (uint64_t)kMaxBlocks) grid64 = kMaxBlocks;
  const int grid = (int)(grid64 < 1 ? 1 : grid64);

  // scratch layout: box | slots+info | block candidates | result | point
  const size_t off_box = 0;
  const size_t off_slots = align256(off_box + 16 * (size_t)n);
  const size_t off_blocks = align256(off_slots + sizeof(StagedSlots));
  const size_t off_result = align256(off_blocks + sizeof(Cand) * (size_t)grid);
  const size_t off_point = align256(off_result + sizeof(Cand));
  const size_t total = off_point + 8 * (size_t)n;
  if (total > kScratchBytes) return set_error(CMN_INVALID_CONFIGURATION, "scratch array too small for this call");

  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  double* d_box = reinterpret_cast<double*>(base + off_box);
  StagedSlots* d_slots = reinterpret_cast<StagedSlots*>(base + off_slots);
  Cand* d_blocks = reinterpret_cast<Cand*>(base + off_blocks);
  Cand* d_result = reinterpret_cast<Cand*>(base + off_result);
  double* d_point = reinterpret_cast<double*>(base + off_point);

  NA_CK(cudaMemcpyAsync(d_box, box, 16 * (size_t)n, cudaMemcpyHostToDevice, s));
  NA_CK(cudaMemcpyAsync(d_slots, &staged, sizeof staged, cudaMemcpyHostToDevice, s));

  // the interleaved box is read as planes of stride 2: lo at [2v], hi at [2v+1]
  SampleArgs a = {};
  a.prog = p->d_prog64;
  a.prog_len = (int)p->prog.code64.size();
  a.n_vars = (int)n;
  a.n_slots = p->prog.n_slots;
  a.log2C = -1;
  a.plo = d_box;
  a.phi = d_box + 1;
  a.pstride = 2;
  a.pinfo = &d_slots->info;
  a.slots = d_slots->slots;
  a.max_slots = 64;
  a.var_kinds = p->d_kinds;
  a.root_lb = p->d_root_lb;
  a.root_ub = p->d_root_ub;
  a.n_children = n_regions;
  a.S = sample_points;
  a.salt = salt;
  a.exact = 0;
  a.block_best = d_blocks;  // every block writes its own entry
  // lane groups and shared point columns, as the sampler role uses them
  a.sched = p->d_sched;
  a.g_max = p->prog.group_max;
  a.capacity = (uint64_t)grid * threads;
  a.lg_min = lg_min;
  NA_CK(launch_sample(a, grid, threads, s));
  NA_CK(launch_reduce_cand(d_blocks, grid, d_result, s));
  NA_CK(launch_witness(d_result, d_box, d_box + 1, 2, &d_slots->info, d_slots->slots, 64, p->d_kinds, (int)n,
                       sample_points, salt, nullptr, 0, nullptr, d_point, s));
  Cand result;
  NA_CK(cudaMemcpyAsync(&result, d_result, sizeof(Cand), cudaMemcpyDeviceToHost, s));
  NA_CK(cudaMemcpyAsync(point, d_point, 8 * (size_t)n, cudaMemcpyDeviceToHost, s));
  NA_CK(cudaStreamSynchronize(s));
  out->found = result.value < DBL_MAX ? 1 : 0;
  out->reserved = 0;
  out->value = result.value;
  out->point = point;
  out->index = out->found ? (int64_t)result.e : -1;
  return CMN_OK;
}
