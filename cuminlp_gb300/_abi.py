"""ctypes mirror of the C ABI structs in include/cuminlp_gb300.h.

Shared by the product bindings (``_lib``) and by the test-side oracle
bindings, which take the same problem description.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

# cmn_op (model/dag.hpp:12-33 order)
OP_VAR, OP_CONST, OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_SQR, OP_NEG = range(8)
OP_EXP, OP_LOG, OP_SQRT, OP_SIN, OP_COS, OP_TANH, OP_POWN, OP_POW = range(8, 16)
OP_ABS, OP_MIN, OP_MAX = 16, 17, 18
OP_NAMES = ["Var", "Const", "Add", "Sub", "Mul", "Div", "Sqr", "Neg", "Exp", "Log", "Sqrt", "Sin",
            "Cos", "Tanh", "PowN", "Pow", "Abs", "Min", "Max"]

VAR_CONTINUOUS, VAR_INTEGER, VAR_BINARY = 0, 1, 2
CMP_LE, CMP_EQ = 0, 1
SLOT_CONTINUOUS, SLOT_INTEGER_PARTITION, SLOT_INTEGER_ENUMERATE, SLOT_BINARY_ENUMERATE = 0, 1, 2, 3
ROLE_BOUNDER, ROLE_SAMPLER, ROLE_ENUMERATOR = 0, 1, 2
PRECISION_FP64, PRECISION_FP32_SCREEN, PRECISION_FP32_LAZY = 0, 1, 2


def precision_code(v) -> int:
    """cmn_precision from a name ("fp64", "fp32" for the screen with FP64
    certification of every survivor, "lazy" for the FP32 bound with FP64
    certification at selection) or a code."""
    if not isinstance(v, str):
        return int(v)
    v = v.lower()
    if "lazy" in v:
        return PRECISION_FP32_LAZY
    return PRECISION_FP32_SCREEN if v.startswith("fp32") else PRECISION_FP64

STATUS_NAMES = ["OK", "INVALID_DAG", "INVALID_PROBLEM", "SHAPE_MISMATCH", "INVALID_CONFIGURATION",
                "OVER_BUDGET", "CUDA_ERROR", "TIMEOUT", "INTERNAL"]
STOP_NAMES = ["converged", "exhausted", "iteration-limit", "host-memory", "allocation-failure",
              "device-memory", "running"]

NODE_DTYPE = np.dtype({
    "names": ["op", "n_in", "in0", "in1", "var_index", "constant", "int_exp", "reserved"],
    "formats": [np.int32, np.int32, np.int64, np.int64, np.int64, np.float64, np.int32, np.int32],
    "offsets": [0, 4, 8, 16, 24, 32, 40, 44],
    "itemsize": 48,
})
CONSTRAINT_DTYPE = np.dtype({
    "names": ["root", "cmp", "reserved", "rhs"],
    "formats": [np.int64, np.int32, np.int32, np.float64],
    "offsets": [0, 8, 12, 16],
    "itemsize": 24,
})


class ProblemDesc(C.Structure):
    _fields_ = [
        ("nodes", C.c_void_p), ("n_nodes", C.c_int64),
        ("var_lb", C.c_void_p), ("var_ub", C.c_void_p), ("var_kinds", C.c_void_p), ("n_vars", C.c_int64),
        ("objective_root", C.c_int64),
        ("constraints", C.c_void_p), ("n_constraints", C.c_int64),
    ]


class ProblemInfo(C.Structure):
    _fields_ = [
        ("n_vars", C.c_int64), ("n_constraints", C.c_int64), ("n_nodes", C.c_int64),
        ("buffer_node_count", C.c_int64), ("program_length", C.c_int64), ("program_slots", C.c_int64),
        ("flops_per_box", C.c_double), ("point_flops_per_box", C.c_double), ("bytes_per_box", C.c_double),
        ("program_segments", C.c_int64), ("lanes_per_box_max", C.c_int64),
    ]


class CostModel(C.Structure):
    _fields_ = [("sampler_bytes_per_sample", C.c_uint64), ("bound_bytes_per_region", C.c_uint64),
                ("exact_bytes_per_region", C.c_uint64), ("fixed_bytes", C.c_uint64)]


class OverBudget(C.Structure):
    _fields_ = [("needed_bytes", C.c_uint64), ("budget_bytes", C.c_uint64), ("n_regions", C.c_uint64),
                ("elements_per_region", C.c_uint64), ("bytes_per_element", C.c_uint64)]


class Candidate(C.Structure):
    _fields_ = [("found", C.c_int32), ("reserved", C.c_int32), ("value", C.c_double),
                ("point", C.POINTER(C.c_double)), ("index", C.c_int64)]


class AggregateBound(C.Structure):
    _fields_ = [("lb", C.c_double), ("hull_ub", C.c_double), ("feasible", C.c_int32), ("reserved", C.c_int32)]


class SolveOptions(C.Structure):
    _fields_ = [
        ("iter_limit", C.c_uint64), ("batch_iter_limit", C.c_uint64), ("tolerance", C.c_double),
        ("precision", C.c_int32), ("bisection_budget", C.c_int32), ("frontier_cap", C.c_uint64),
        ("batch_parents", C.c_uint64), ("sample_points", C.c_uint64), ("sample_all", C.c_int32),
        ("relative_width", C.c_int32), ("max_cycle_size", C.c_uint64), ("enumerate_cap", C.c_uint64),
        ("has_known_primal", C.c_int32), ("autotune", C.c_int32), ("known_primal_bound", C.c_double),
        ("time_limit_ms", C.c_uint64),
    ]


class TuneResult(C.Structure):
    _fields_ = [("blocks_per_sm", C.c_int32), ("lanes_cap", C.c_int32), ("ms_best", C.c_double),
                ("ms_default", C.c_double), ("candidates", C.c_int32), ("reserved", C.c_int32)]


class BatchConfig(C.Structure):
    _fields_ = [("slots", C.c_uint64), ("max_vars", C.c_int32), ("max_program_slots", C.c_int32),
                ("device", C.c_int32), ("max_segments", C.c_int32), ("shared", SolveOptions)]


SERVER_MAX_CLASSES = 8


class ServerConfig(C.Structure):
    _fields_ = [("shared", SolveOptions), ("device", C.c_int32), ("n_classes", C.c_int32),
                ("class_max_vars", C.c_int32 * SERVER_MAX_CLASSES),
                ("class_max_program_slots", C.c_int32 * SERVER_MAX_CLASSES),
                ("class_slots", C.c_uint64 * SERVER_MAX_CLASSES), ("pool_budget_bytes", C.c_uint64),
                ("iterations_per_round", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("submitted", "admitted", "completed", "queued", "running", "converged",
                                          "boxes", "rounds", "pool_bytes_in_use", "pool_bytes_peak",
                                          "pool_budget_bytes")] + \
               [(n, C.c_double) for n in ("latency_p50_ms", "latency_p99_ms", "latency_mean_ms", "latency_max_ms",
                                          "queue_p50_ms", "queue_p99_ms", "wall_ms", "boxes_per_s")]


COUNTER_NAMES = ["iterations", "expansions", "fathomed", "fathomed_points", "bounded", "sampled", "enqueued",
                 "witness_rejected", "pruned_duplicate", "pruned_infeasible", "pruned_dominated",
                 "dropped_viable", "dropped_dominated", "screened_fp32", "certified_fp64", "peak_frontier",
                 "certify_pruned"]


class Counters(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in COUNTER_NAMES]


class Outcome(C.Structure):
    _fields_ = [
        ("lower_bound", C.c_double), ("upper_bound", C.c_double), ("stop_reason", C.c_int32),
        ("proven_optimal", C.c_int32), ("infeasible", C.c_int32), ("found_incumbent", C.c_int32),
        ("frontier_size", C.c_uint64), ("viable", C.c_uint64), ("dropped_lb_min", C.c_double),
        ("elapsed_ms", C.c_double), ("counters", Counters),
    ]


def outcome_dict(o: Outcome) -> dict:
    d = {f: getattr(o, f) for f, _ in Outcome._fields_ if f != "counters"}
    d["stop_reason"] = STOP_NAMES[o.stop_reason] if 0 <= o.stop_reason < len(STOP_NAMES) else str(o.stop_reason)
    d["counters"] = {n: int(getattr(o.counters, n)) for n in COUNTER_NAMES}
    return d


def ptr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data
