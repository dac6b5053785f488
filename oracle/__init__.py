"""ctypes bindings of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
baseline.  Only tests/, the smoke check and bench.py's CPU arm import this
package; the product package never does.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from cuminlp_gb300 import _abi as A

LIB_PATH = Path(__file__).resolve().parent / "liboracle.so"
_lib = None

P = C.c_void_p
D = C.c_double
F = C.c_float
U64 = C.c_uint64
I64 = C.c_int64
I32 = C.c_int32

_SIG = {
    "orc_problem_create": (P, [C.POINTER(A.ProblemDesc)]),
    "orc_problem_destroy": (None, [P]),
    "orc_last_error": (C.c_char_p, []),
    "orc_buffer_node_count": (I64, [P]),
    "orc_add_rd": (D, [D, D]), "orc_add_ru": (D, [D, D]),
    "orc_mul_rd": (D, [D, D]), "orc_mul_ru": (D, [D, D]),
    "orc_div_rd": (D, [D, D]), "orc_div_ru": (D, [D, D]),
    "orc_addf_rd": (F, [F, F]), "orc_addf_ru": (F, [F, F]),
    "orc_mulf_rd": (F, [F, F]), "orc_mulf_ru": (F, [F, F]),
    "orc_d2f_rd": (F, [D]), "orc_d2f_ru": (F, [D]),
    "orc_interval_op_f64": (None, [I32, D, D, D, D, I32, C.POINTER(D), C.POINTER(D)]),
    "orc_interval_op_f32": (None, [I32, F, F, F, F, I32, C.POINTER(F), C.POINTER(F)]),
    "orc_eval_nodes_f64": (I32, [P, P, P, P]),
    "orc_eval_nodes_f32": (I32, [P, P, P, P]),
    "orc_eval_boxes": (I32, [P, I32, P, P, I64, I64, P, P, P, I32]),
    "orc_eval_point": (I32, [P, P, C.POINTER(D), C.POINTER(C.c_uint8)]),
    "orc_slot_bounds": (None, [I32, D, D, U64, U64, C.POINTER(D), C.POINTER(D)]),
    "orc_sample_hash": (U64, [U64, U64, U64, U64]),
    "orc_sample_continuous": (D, [D, D, U64, U64, U64, U64]),
    "orc_sample_discrete": (D, [D, D, U64, U64, U64, U64]),
    "orc_sample_continuous_f32": (F, [F, F, U64, U64, U64, U64]),
    "orc_sample_discrete_f32": (F, [F, F, U64, U64, U64, U64]),
    "orc_bound": (I32, [P, P, P, P, P, I64, U64, P, P, I32]),
    "orc_bound_hw": (I32, [P, P, P, P, P, I64, U64, P, P, I32]),
    "orc_set_program32": (I32, [P, P, I64]),
    "orc_set_program64": (I32, [P, P, I64]),
    "orc_program_eval64": (I32, [P, P, C.POINTER(D), C.POINTER(D)]),
    "orc_program_eval32": (I32, [P, P, C.POINTER(D), C.POINTER(D)]),
    "orc_finalise": (I32, [D, D, D, I32, I32, I32, D, U64, P, P, I64, C.POINTER(A.Outcome)]),
    "orc_bound_inc32": (I32, [P, P, P, P, P, I64, U64, P, P, P]),
    "orc_aggregate_bound": (I32, [P, P, P, P, P, I64, U64, U64, P, P, P, I32]),
    "orc_sample": (I32, [P, P, P, P, P, I64, U64, U64, U64, C.POINTER(I32), C.POINTER(D), C.POINTER(I64), P, I32]),
    "orc_enumerate": (I32, [P, P, P, P, P, I64, U64, C.POINTER(I32), C.POINTER(D), C.POINTER(I64), P, I32]),
    "orc_bisection_choose": (I64, [P, P, I64, I64, I64, I64, I32, P, P, P, P]),
    "orc_solve_reference": (I32, [P, C.POINTER(A.SolveOptions), C.POINTER(A.Outcome), P, I32]),
    "orc_solve_batched": (I32, [P, C.POINTER(A.SolveOptions), C.POINTER(A.Outcome), P, I32]),
    "orc_batched_frontier": (I64, [P, C.POINTER(A.SolveOptions), U64, P, P, P, I64, C.POINTER(A.Outcome), P, I32]),
}


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from cuminlp_gb300 import build
            build.build_oracle()
        h = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIG.items():
            f = getattr(h, name)
            f.restype = res
            f.argtypes = args
        _lib = h
    return _lib


def threads_default() -> int:
    return max(1, os.cpu_count() or 1)


def options(**kw) -> A.SolveOptions:
    """Solve options with the library defaults (no GPU needed)."""
    o = A.SolveOptions()
    o.iter_limit = 1000000
    o.tolerance = 1e-6
    o.precision = A.PRECISION_FP64
    o.bisection_budget = 4
    o.frontier_cap = 1 << 20
    o.batch_parents = 1 << 16
    o.sample_points = 1
    for k, v in kw.items():
        if k == "precision" and isinstance(v, str):
            v = A.precision_code(v)
        if k == "known_primal_bound" and v is not None:
            o.has_known_primal = 1
        if v is None:
            continue
        setattr(o, k, v)
    return o


class OracleProblem:
    def __init__(self, problem):
        desc, self._keep = problem.desc()
        h = lib().orc_problem_create(C.byref(desc))
        if not h:
            raise ValueError(lib().orc_last_error().decode())
        self.h = h
        self.problem = problem
        self.n_vars = problem.n_vars
        self.n_nodes = len(problem.graph.nodes)

    def __del__(self):
        try:
            if self.h:
                lib().orc_problem_destroy(self.h)
        except Exception:
            pass

    @property
    def buffer_node_count(self) -> int:
        return int(lib().orc_buffer_node_count(self.h))

    def eval_nodes(self, box, fp32: bool = False):
        box = np.ascontiguousarray(box, dtype=np.float64)
        dt = np.float32 if fp32 else np.float64
        lo = np.empty(self.n_nodes, dtype=dt)
        hi = np.empty(self.n_nodes, dtype=dt)
        fn = lib().orc_eval_nodes_f32 if fp32 else lib().orc_eval_nodes_f64
        if fn(self.h, A.ptr(box), A.ptr(lo), A.ptr(hi)):
            raise ValueError(lib().orc_last_error().decode())
        return lo, hi

    def eval_boxes(self, lo, hi, precision=A.PRECISION_FP64, threads=None):
        lo = np.ascontiguousarray(lo, dtype=np.float64)
        hi = np.ascontiguousarray(hi, dtype=np.float64)
        nb = lo.shape[1]
        lb = np.empty(nb)
        ub = np.empty(nb)
        fe = np.empty(nb, dtype=np.uint8)
        if lib().orc_eval_boxes(self.h, precision, A.ptr(lo), A.ptr(hi), nb, nb, A.ptr(lb), A.ptr(ub), A.ptr(fe),
                                threads or threads_default()):
            raise ValueError(lib().orc_last_error().decode())
        return lb, ub, fe

    def eval_point(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        obj = C.c_double()
        f = C.c_uint8()
        lib().orc_eval_point(self.h, A.ptr(x), C.byref(obj), C.byref(f))
        return obj.value, bool(f.value)

    @staticmethod
    def _slots(kinds, var_ids, widths):
        k = np.ascontiguousarray(kinds, dtype=np.uint8)
        v = np.ascontiguousarray(var_ids, dtype=np.uint64)
        w = np.ascontiguousarray(widths, dtype=np.uint64)
        return k, v, w

    def set_program32(self, code: np.ndarray) -> bool:
        """The library's compiled FP32 program (DeviceProblem.program(1)):
        the lazy form then bounds children incrementally, as the device
        does.  True when the program has the sum-chain shape for that."""
        code = np.ascontiguousarray(code, dtype=np.uint8)
        return bool(lib().orc_set_program32(self.h, A.ptr(code), code.size // 16))

    def set_program64(self, code: np.ndarray) -> bool:
        """The library's compiled FP64 program (DeviceProblem.program(0)):
        the lazy form's verdict of each expanded box runs it with fused
        terms, as the device does."""
        code = np.ascontiguousarray(code, dtype=np.uint8)
        return bool(lib().orc_set_program64(self.h, A.ptr(code), code.size // 16))

    def program_eval64(self, box):
        """One box through the FP64 program (after set_program64) with every
        operation rounded on its own, as the plain form runs it: (feasible,
        lb, ub), feasible -1 for an operator without an interval form."""
        box = np.ascontiguousarray(box, dtype=np.float64)
        lb, ub = C.c_double(), C.c_double()
        f = lib().orc_program_eval64(self.h, A.ptr(box), C.byref(lb), C.byref(ub))
        if f == -2:
            raise ValueError(lib().orc_last_error().decode())
        return f, lb.value, ub.value

    def program_eval32(self, box):
        """The same through the FP32 program (after set_program32): (not
        proven infeasible, lb, ub) as the FP32 screen evaluates it."""
        box = np.ascontiguousarray(box, dtype=np.float64)
        lb, ub = C.c_double(), C.c_double()
        f = lib().orc_program_eval32(self.h, A.ptr(box), C.byref(lb), C.byref(ub))
        if f == -2:
            raise ValueError(lib().orc_last_error().decode())
        return f, lb.value, ub.value

    def bound_inc32(self, box, kinds, var_ids, widths, n_regions):
        """The lazy form's incremental FP32 bounds of one parent's regions
        (after set_program32): feasible (not proven violated), lb, ub."""
        box = np.ascontiguousarray(box, dtype=np.float64)
        k, v, w = self._slots(kinds, var_ids, widths)
        fe = np.empty(n_regions, dtype=np.uint8)
        lb = np.empty(n_regions)
        ub = np.empty(n_regions)
        if lib().orc_bound_inc32(self.h, A.ptr(box), A.ptr(k), A.ptr(v), A.ptr(w), len(k), n_regions, A.ptr(fe),
                                 A.ptr(lb), A.ptr(ub)):
            raise ValueError(lib().orc_last_error().decode())
        return fe, lb, ub

    def bound(self, box, kinds, var_ids, widths, n_regions, threads=None, hardware_rounding=False):
        """orc_bound; hardware_rounding=True runs orc_bound_hw (the host's
        directed-rounding mode instead of error-free transformations, same
        results)."""
        box = np.ascontiguousarray(box, dtype=np.float64)
        k, v, w = self._slots(kinds, var_ids, widths)
        fe = np.empty(n_regions, dtype=np.uint8)
        lb = np.empty(n_regions)
        fn = lib().orc_bound_hw if hardware_rounding else lib().orc_bound
        if fn(self.h, A.ptr(box), A.ptr(k), A.ptr(v), A.ptr(w), len(k), n_regions, A.ptr(fe), A.ptr(lb),
              threads or threads_default()):
            raise ValueError(lib().orc_last_error().decode())
        return fe, lb

    def aggregate_bound(self, box, kinds, var_ids, widths, n_regions, k, threads=None):
        """(lb, hull_ub, feasible) per child: k children of n_regions / k regions."""
        box = np.ascontiguousarray(box, dtype=np.float64)
        kk, v, w = self._slots(kinds, var_ids, widths)
        lb = np.empty(k)
        ub = np.empty(k)
        fe = np.empty(k, dtype=np.int32)
        if lib().orc_aggregate_bound(self.h, A.ptr(box), A.ptr(kk), A.ptr(v), A.ptr(w), len(kk), n_regions, k,
                                     A.ptr(lb), A.ptr(ub), A.ptr(fe), threads or threads_default()):
            raise ValueError(lib().orc_last_error().decode())
        return lb, ub, fe

    def sample(self, box, kinds, var_ids, widths, n_regions, sample_points, salt, threads=None):
        box = np.ascontiguousarray(box, dtype=np.float64)
        k, v, w = self._slots(kinds, var_ids, widths)
        found = C.c_int32()
        val = C.c_double()
        idx = C.c_int64()
        pt = np.empty(self.n_vars)
        if lib().orc_sample(self.h, A.ptr(box), A.ptr(k), A.ptr(v), A.ptr(w), len(k), n_regions, sample_points, salt,
                            C.byref(found), C.byref(val), C.byref(idx), A.ptr(pt), threads or threads_default()):
            raise ValueError(lib().orc_last_error().decode())
        return bool(found.value), val.value, pt, idx.value

    def enumerate(self, box, kinds, var_ids, widths, n_regions, threads=None):
        box = np.ascontiguousarray(box, dtype=np.float64)
        k, v, w = self._slots(kinds, var_ids, widths)
        found = C.c_int32()
        val = C.c_double()
        idx = C.c_int64()
        pt = np.empty(self.n_vars)
        if lib().orc_enumerate(self.h, A.ptr(box), A.ptr(k), A.ptr(v), A.ptr(w), len(k), n_regions, C.byref(found),
                               C.byref(val), C.byref(idx), A.ptr(pt), threads or threads_default()):
            raise ValueError(lib().orc_last_error().decode())
        return bool(found.value), val.value, pt, idx.value

    def solve_reference(self, threads=None, **kw):
        o = options(**kw)
        out = A.Outcome()
        pt = np.empty(self.n_vars)
        if lib().orc_solve_reference(self.h, C.byref(o), C.byref(out), A.ptr(pt), threads or threads_default()):
            raise ValueError(lib().orc_last_error().decode())
        d = A.outcome_dict(out)
        d["best_point"] = pt
        return d

    def solve_batched(self, threads=None, **kw):
        o = options(**kw)
        out = A.Outcome()
        pt = np.empty(self.n_vars)
        if lib().orc_solve_batched(self.h, C.byref(o), C.byref(out), A.ptr(pt), threads or threads_default()):
            raise ValueError(lib().orc_last_error().decode())
        d = A.outcome_dict(out)
        d["best_point"] = pt
        return d

    def batched_frontier(self, iterations, room=1 << 16, threads=None, **kw):
        o = options(**kw)
        out = A.Outcome()
        pt = np.empty(self.n_vars)
        box = np.empty((room, 2 * self.n_vars))
        lb = np.empty(room)
        depth = np.empty(room, dtype=np.uint32)
        n = lib().orc_batched_frontier(self.h, C.byref(o), iterations, A.ptr(box), A.ptr(lb), A.ptr(depth), room,
                                       C.byref(out), A.ptr(pt), threads or threads_default())
        if n < 0:
            raise ValueError(lib().orc_last_error().decode())
        m = min(n, room)
        d = A.outcome_dict(out)
        d["best_point"] = pt
        return box[:m], lb[:m], depth[:m], d


def finalise(glb, gub, converged, pending_empty, frontier_min, viable, drops=(), tolerance=1e-6,
             found=None):
    """The epilogue's answers (proven_optimal, infeasible, lower_bound) for
    a run that dropped the (lb, gub at the time) pairs in `drops`; `found`
    defaults to gub below the no-incumbent sentinel (DBL_MAX)."""
    if found is None:
        found = gub < np.finfo(np.float64).max
    lbs = np.ascontiguousarray([d[0] for d in drops] or [0.0], dtype=np.float64)
    gubs = np.ascontiguousarray([d[1] for d in drops] or [0.0], dtype=np.float64)
    out = A.Outcome()
    lib().orc_finalise(glb, gub, tolerance, int(found), int(converged), int(pending_empty), frontier_min, viable,
                       A.ptr(lbs), A.ptr(gubs), len(drops), C.byref(out))
    return bool(out.proven_optimal), bool(out.infeasible), out.lower_bound


def bisection_choose(box, var_kinds, B, max_cycle=0, enumerate_cap=0, relative=False):
    box = np.ascontiguousarray(box, dtype=np.float64)
    vk = np.ascontiguousarray(var_kinds, dtype=np.int32)
    n = len(vk)
    kinds = np.empty(max(n, 1), dtype=np.uint8)
    vids = np.empty(max(n, 1), dtype=np.uint64)
    widths = np.empty(max(n, 1), dtype=np.uint64)
    dom = np.empty(max(n, 1), dtype=np.uint64)
    c = lib().orc_bisection_choose(A.ptr(box), A.ptr(vk), n, B, max_cycle, enumerate_cap, int(relative),
                                   A.ptr(kinds), A.ptr(vids), A.ptr(widths), A.ptr(dom))
    return kinds[:c].copy(), vids[:c].copy(), widths[:c].copy(), dom[:c].copy()


def slot_bounds(kind, plo, phi, part, fan_out):
    lo, hi = C.c_double(), C.c_double()
    lib().orc_slot_bounds(kind, plo, phi, part, fan_out, C.byref(lo), C.byref(hi))
    return lo.value, hi.value


def interval_op(op, a, b=(0.0, 0.0), int_exp=0, fp32=False):
    if fp32:
        lo, hi = C.c_float(), C.c_float()
        lib().orc_interval_op_f32(op, a[0], a[1], b[0], b[1], int_exp, C.byref(lo), C.byref(hi))
    else:
        lo, hi = C.c_double(), C.c_double()
        lib().orc_interval_op_f64(op, a[0], a[1], b[0], b[1], int_exp, C.byref(lo), C.byref(hi))
    return lo.value, hi.value
