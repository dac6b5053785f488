// handles.hpp -- definitions shared by the C ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "../../include/cuminlp_gb300.h"
#include "program.hpp"

// A compiled problem resident on one device.
struct cmn_problem {
  cmn::HostProblem host;
  cmn::Program prog;
  int device = 0;
  cmn::Instr* d_prog64 = nullptr;
  cmn::Instr* d_prog32 = nullptr;
  cmn::Instr* d_prog32p = nullptr;  // FP32 point program (the lazy form's sample screen)
  int32_t* d_kinds = nullptr;
  double* d_root_lb = nullptr;
  double* d_root_ub = nullptr;
  int32_t* d_sched = nullptr;  // lane schedules (Program::sched), null when none
  int32_t* d_inc_seg = nullptr;  // incremental child tables (Program::inc_*), null when none
  int32_t* d_inc_off = nullptr;
  int32_t* d_inc_pcs = nullptr;
  // cmn_autotune's choice per precision (0 FP64, 1 FP32): blocks per SM
  // and lanes per box cap; 0 = not tuned
  int tuned_bps[2] = {0, 0};
  int tuned_lanes[2] = {0, 0};

  ~cmn_problem();
};

namespace cmn {

// Records `msg` as this thread's cmn_last_error() and returns `st`.
cmn_status set_error(cmn_status st, const std::string& msg);

// Sets the kernels' dynamic shared-memory allowance once per device.
cudaError_t ensure_kernel_attributes();

}  // namespace cmn
