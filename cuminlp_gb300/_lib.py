"""Loads libcuminlp_gb300.so and declares the C ABI's signatures.

There is no fallback: if the library is missing or fails to load, every
entry point raises.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

from . import _abi as A

LIB_PATH = Path(__file__).resolve().parent / "libcuminlp_gb300.so"
_lib = None

P = C.c_void_p
PP = C.POINTER(C.c_void_p)
U64 = C.c_uint64
I64 = C.c_int64
I32 = C.c_int32
D = C.c_double

SIGNATURES = {
    "cmn_last_error": (C.c_char_p, []),
    "cmn_version": (C.c_char_p, []),
    "cmn_problem_create": (I32, [C.POINTER(A.ProblemDesc), PP]),
    "cmn_problem_destroy": (None, [P]),
    "cmn_problem_get_info": (I32, [P, C.POINTER(A.ProblemInfo)]),
    "cmn_problem_program": (I32, [P, I32, P, I64, C.POINTER(I64)]),
    "cmn_program_compile": (I32, [C.POINTER(A.ProblemDesc), I32, P, I64, C.POINTER(I64)]),
    "cmn_autotune": (I32, [P, I32, U64, C.POINTER(A.TuneResult)]),
    "cmn_cost_model_get": (I32, [P, C.POINTER(A.CostModel)]),
    "cmn_bisection_choose": (I32, [P, P, I64, I32, U64, U64, I32, P, P, P, P, C.POINTER(I64), C.POINTER(I32)]),
    "cmn_slot_bounds": (None, [I32, D, D, U64, U64, C.POINTER(D), C.POINTER(D)]),
    "cmn_role_build": (I32, [P, I32, P, I64, U64, U64, U64, PP, C.POINTER(A.OverBudget)]),
    "cmn_role_destroy": (None, [P]),
    "cmn_role_n_regions": (U64, [P]),
    "cmn_role_n_elements": (U64, [P]),
    "cmn_bound": (I32, [P, P, P, P, C.POINTER(C.POINTER(C.c_uint8)), C.POINTER(C.POINTER(D)), C.POINTER(U64)]),
    "cmn_sample": (I32, [P, P, P, P, U64, C.POINTER(A.Candidate)]),
    "cmn_bound_children": (I32, [P, P, P, P, U64, C.POINTER(C.POINTER(A.AggregateBound))]),
    "cmn_enumerate": (I32, [P, P, P, P, C.POINTER(A.Candidate)]),
    "cmn_sample_noalloc": (I32, [P, P, I64, U64, U64, P, P, P, U64, C.POINTER(A.Candidate), P, P]),
    "cmn_eval_boxes": (I32, [P, I32, P, P, U64, U64, P, P, P, I32, P]),
    "cmn_solve_options_default": (None, [C.POINTER(A.SolveOptions)]),
    "cmn_solver_create": (I32, [P, C.POINTER(A.SolveOptions), PP]),
    "cmn_solver_destroy": (None, [P]),
    "cmn_solver_step": (I32, [P, U64]),
    "cmn_query_bounds": (I32, [P, C.POINTER(D), C.POINTER(D)]),
    "cmn_query_incumbent": (I32, [P, P, C.POINTER(I32)]),
    "cmn_query_gap": (I32, [P, C.POINTER(D)]),
    "cmn_solver_outcome": (I32, [P, C.POINTER(A.Outcome)]),
    "cmn_solver_stream": (P, [P]),
    "cmn_solver_frontier": (I32, [P, P, P, P, U64, C.POINTER(U64)]),
    "cmn_solver_phase_ms": (I32, [P, C.POINTER(D)]),
    "cmn_solver_lazy_ms": (I32, [P, C.POINTER(D)]),
    "cmn_solver_kernels_per_iteration": (U64, [P]),
    "cmn_measure_fma_peak": (I32, [I32, C.POINTER(D)]),
    "cmn_fp64_emu_check": (I32, [U64, U64, I32, C.POINTER(U64)]),
    "cmn_fp64_emu_check_host": (I32, [U64, U64, I32, C.POINTER(U64)]),
    "cmn_fp64_emu_op_host": (I32, [I32, D, D, C.POINTER(D), C.POINTER(I32)]),
    "cmn_solve": (I32, [P, C.POINTER(A.SolveOptions), C.POINTER(A.Outcome), P]),
    "cmn_batch_create": (I32, [C.POINTER(A.BatchConfig), PP]),
    "cmn_batch_destroy": (None, [P]),
    "cmn_batch_add": (I32, [P, P, C.POINTER(A.SolveOptions), C.POINTER(U64)]),
    "cmn_batch_step": (I32, [P, U64, C.POINTER(U64)]),
    "cmn_batch_poll": (I32, [P, U64, C.POINTER(I32)]),
    "cmn_batch_outcome": (I32, [P, U64, C.POINTER(A.Outcome), P]),
    "cmn_batch_frontier": (I32, [P, U64, P, P, P, U64, C.POINTER(U64)]),
    "cmn_batch_release": (I32, [P, U64]),
    "cmn_batch_stream": (P, [P]),
    "cmn_batch_kernels_per_iteration": (U64, [P]),
    "cmn_batch_solve": (I32, [C.POINTER(A.BatchConfig), P, P, U64, P, P, U64]),
    "cmn_batch_launch": (I32, [P, U64]),
    "cmn_batch_sync": (I32, [P, C.POINTER(U64)]),
    "cmn_batch_query": (I32, [P, C.POINTER(I32)]),
    "cmn_batch_slot_bytes": (U64, [P]),
    "cmn_batch_phase_ms": (I32, [P, C.POINTER(D)]),
    "cmn_batch_totals": (I32, [P, C.POINTER(A.Counters), C.POINTER(U64)]),
    "cmn_server_create": (I32, [C.POINTER(A.ServerConfig), PP]),
    "cmn_server_destroy": (None, [P]),
    "cmn_server_submit": (I32, [P, P, C.POINTER(A.SolveOptions), C.POINTER(U64)]),
    "cmn_server_poll": (I32, [P, U64, C.POINTER(I32), C.POINTER(A.Outcome), P]),
    "cmn_server_wait": (I32, [P, U64, U64, C.POINTER(A.Outcome), P]),
    "cmn_server_stats_get": (I32, [P, C.POINTER(A.ServerStats)]),
}


class CmnError(RuntimeError):
    def __init__(self, status: int, message: str):
        self.status = status
        self.status_name = A.STATUS_NAMES[status] if 0 <= status < len(A.STATUS_NAMES) else str(status)
        super().__init__(f"{self.status_name}: {message}")


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
        handle = C.CDLL(str(LIB_PATH), mode=os.RTLD_NOW | C.RTLD_GLOBAL)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def check(status: int) -> None:
    if status != 0:
        msg = lib().cmn_last_error()
        raise CmnError(status, msg.decode() if msg else "")
