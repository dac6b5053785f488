// launch.hpp -- host-side launch wrappers of the device kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "kernels.cuh"

namespace cmn {

constexpr int kEvalThreads = 128;
// resident blocks per SM the single-instance bound kernels are compiled
// for (registers): 5 measured ahead of 4 and 6 on the n=32 and n=4
// workloads, with a little spilling
#ifndef CMN_EVAL_MIN_BLOCKS
#define CMN_EVAL_MIN_BLOCKS 5
#endif

// interval kernels: program slots plus `max_slots` split variables per thread
size_t eval_smem_bytes(int n_slots, int max_slots, bool fp32, int threads);
// sampler: one point column (variables + slots, FP64) per 2^lg_min threads
size_t sample_smem_bytes(int n_vars, int n_slots, int threads, int lg_min);
// Point columns of a block stay within this many bytes: lanes share a
// column (2^lg_min of them) until they do, so the sampler's residency does
// not fall with the number of variables.  Programs with shared slots have
// no lane schedule and keep one column per thread.
constexpr size_t kSampleColumnBytes = 32 * 1024;
int sample_lg_min(int n_vars, int n_slots, bool has_sched, int threads);
size_t sample_screen_smem_bytes(int n_vars, int n_slots, int threads, int lg_min);
// the lazy form's FP32 sample screen: one point column (FP32) per 2^lg_min lanes
int sample_screen_lg_min(int n_vars, int n_slots, bool has_sched, int threads);

// mode 0: role / raw boxes; 1: solver FP64; 2: solver FP32 screen (fp32
// must be true); 3: solver FP64 certify over EvalArgs::list; 4: aggregate
// bounder (FP64, per-child fold into EvalArgs::agg_keys); 5: solver lazy
// form, FP32 children bounded by the parents' certified bounds (fp32 true);
// 6: the lazy form's FP64 verdict of the staged parents (mode 0's outputs,
// each term's coefficient and chain add fused into __fma_rd / __fma_ru)
cudaError_t launch_eval(const EvalArgs& a, int mode, bool fp32, int grid, int threads, cudaStream_t s);
cudaError_t launch_sample(const SampleArgs& a, int grid, int threads, cudaStream_t s);
// the lazy form's incremental FP32 children: the common chain sums per
// (segment, parent), then every child (EvalArgs::inc_* set, prog = FP32)
cudaError_t launch_inc(const EvalArgs& a, int grid, int threads, cudaStream_t s);
// shared memory of the incremental child pass per block
size_t inc_child_smem_bytes(int max_slots, int threads);
// the lazy form's FP32 sample screen (SampleArgs::cbest out, prog = the
// FP32 point program)
cudaError_t launch_sample_screen(const SampleArgs& a, int grid, int threads, cudaStream_t s);
cudaError_t launch_reduce_cand(const Cand* block_best, int n, Cand* out, cudaStream_t s);
cudaError_t launch_witness(const Cand* cand, const double* plo, const double* phi, uint64_t pstride,
                           const ParentInfo* pinfo, const SlotPlan* slots, int max_slots, const int32_t* kinds,
                           int n_vars, uint64_t S, uint64_t salt, const uint64_t* salt_base_dev, int exact,
                           const uint32_t* write_flag, double* out, cudaStream_t s);

// Largest dynamic shared memory a block may use on this device.
int max_dynamic_smem();
// Resident blocks per SM of the sampler at this shared-memory size.
int sample_kernel_occupancy(size_t smem, int threads);
int sample_screen_occupancy(size_t smem, int threads);
int sm_count();

}  // namespace cmn
