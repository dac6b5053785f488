"""Python face of the C ABI: region roles, batched evaluation and the
device-resident solver.

Role objects mirror the reference's plugin boundary
(backend/backend.hpp:81-219): ``Bounder.bound(box, var_ids, widths)``
returns per-region ``feasible`` and ``obj_lb`` views valid until the next
call; ``Sampler.sample(..., salt)`` and ``Enumerator.enumerate(...)``
return a candidate (found, value, point, index).  ``solve()`` mirrors
``SearchDriver::solve`` (search/driver.hpp:137-537) and returns the
``SolveOutcome`` fields.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi as A
from ._lib import check, lib
from .problem import Problem


K_MAX_SLOTS = 64  # config::kMaxSlots


# -- the library's host builds of the branching policy and the decode ------
@dataclass
class SlotAssignment:
    kinds: list = field(default_factory=list)
    var_ids: list = field(default_factory=list)
    widths: list = field(default_factory=list)
    domains: list = field(default_factory=list)

    def size(self) -> int:
        return len(self.kinds)

    def key(self) -> tuple:
        return (tuple(self.kinds), tuple(self.var_ids), tuple(self.widths))


def bisection_choose(box, var_kinds, budget_bits: int, max_cycle: int = 0, enumerate_cap: int = 0,
                     relative: bool = False) -> SlotAssignment:
    """BisectionBudgetCompositionPolicy::choose on the host (cmn_bisection_choose)."""
    box = np.ascontiguousarray(box, dtype=np.float64)
    vk = np.ascontiguousarray(var_kinds, dtype=np.int32)
    kinds = np.zeros(K_MAX_SLOTS, dtype=np.uint8)
    vids = np.zeros(K_MAX_SLOTS, dtype=np.uint64)
    widths = np.zeros(K_MAX_SLOTS, dtype=np.uint64)
    doms = np.zeros(K_MAX_SLOTS, dtype=np.uint64)
    cnt = C.c_int64()
    check(lib().cmn_bisection_choose(A.ptr(box), A.ptr(vk), len(vk), int(budget_bits), int(max_cycle),
                                     int(enumerate_cap), int(relative), A.ptr(kinds), A.ptr(vids), A.ptr(widths),
                                     A.ptr(doms), C.byref(cnt), None))
    c = cnt.value
    return SlotAssignment([int(x) for x in kinds[:c]], [int(x) for x in vids[:c]], [int(x) for x in widths[:c]],
                          [int(x) for x in doms[:c]])


def slot_bounds(kind: int, plo: float, phi: float, part: int, fan_out: int):
    lo, hi = C.c_double(), C.c_double()
    lib().cmn_slot_bounds(int(kind), float(plo), float(phi), int(part), int(fan_out), C.byref(lo), C.byref(hi))
    return lo.value, hi.value


def materialise(parent: list, sidx: int, a: SlotAssignment) -> list:
    """region::materialise: the child `sidx` of `parent` under `a` (slot 0
    least significant)."""
    out = list(parent)
    idx = sidx
    for kind, vid, w in zip(a.kinds, a.var_ids, a.widths):
        part = idx % w
        idx //= w
        out[vid] = slot_bounds(kind, parent[vid][0], parent[vid][1], part, w)
    return out


def compile_program(problem: Problem, precision: int = 0) -> np.ndarray:
    """The compiled program of `problem` built on the host
    (cmn_program_compile), without a CUDA device: the bytes
    DeviceProblem.program(precision) returns."""
    desc, _keep = problem.desc()  # _keep holds the arrays desc points into
    n = C.c_int64()
    check(lib().cmn_program_compile(C.byref(desc), precision, None, 0, C.byref(n)))
    buf = np.zeros(16 * n.value, dtype=np.uint8)
    check(lib().cmn_program_compile(C.byref(desc), precision, A.ptr(buf), n.value, C.byref(n)))
    return buf


class DeviceProblem:
    """A Problem compiled and resident on the current CUDA device."""

    def __init__(self, problem: Problem, **desc_options):
        """`desc_options` go to Problem.desc (a node as the objective, no
        constraints, reused arrays)."""
        self.problem = problem
        desc, self._keep = problem.desc(**desc_options)
        h = C.c_void_p()
        check(lib().cmn_problem_create(C.byref(desc), C.byref(h)))
        self.handle = h
        self.n_vars = problem.n_vars

    def program(self, precision: int = 0) -> np.ndarray:
        """The compiled program (cmn_problem_program): 16 bytes per
        instruction, FP64 (0) or the FP32 screen's (1)."""
        n = C.c_int64()
        check(lib().cmn_problem_program(self.handle, precision, None, 0, C.byref(n)))
        buf = np.zeros(16 * n.value, dtype=np.uint8)
        check(lib().cmn_problem_program(self.handle, precision, A.ptr(buf), n.value, C.byref(n)))
        return buf

    def autotune(self, precision: int = 0, n_boxes: int = 1 << 16) -> dict:
        """cmn_autotune: times the evaluator's launch shapes on this problem
        and records the fastest for solvers created with autotune=1."""
        r = A.TuneResult()
        check(lib().cmn_autotune(self.handle, precision, n_boxes, C.byref(r)))
        return {f: getattr(r, f) for f, _ in A.TuneResult._fields_ if f != "reserved"}

    def info(self) -> dict:
        inf = A.ProblemInfo()
        check(lib().cmn_problem_get_info(self.handle, C.byref(inf)))
        return {f: getattr(inf, f) for f, _ in A.ProblemInfo._fields_}

    def cost_model(self) -> dict:
        cm = A.CostModel()
        check(lib().cmn_cost_model_get(self.handle, C.byref(cm)))
        return {f: int(getattr(cm, f)) for f, _ in A.CostModel._fields_}

    def close(self):
        if getattr(self, "handle", None):
            lib().cmn_problem_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OverBudgetError(RuntimeError):
    def __init__(self, message, facts: dict):
        super().__init__(message)
        self.facts = facts


@dataclass
class CandidateResult:
    found: bool
    value: float
    point: np.ndarray
    index: int


class _Role:
    kind = -1

    def __init__(self, dp: DeviceProblem, slot_kinds, n_regions: int, budget_bytes: int = 0,
                 sample_points: int = 1):
        self.dp = dp
        self.slot_kinds = np.ascontiguousarray(slot_kinds, dtype=np.uint8)
        h = C.c_void_p()
        facts = A.OverBudget()
        st = lib().cmn_role_build(dp.handle, self.kind, A.ptr(self.slot_kinds) if len(self.slot_kinds) else None,
                                  len(self.slot_kinds), int(n_regions), int(budget_bytes), int(sample_points),
                                  C.byref(h), C.byref(facts))
        if st == 5:  # OVER_BUDGET
            msg = lib().cmn_last_error().decode()
            raise OverBudgetError(msg, {f: int(getattr(facts, f)) for f, _ in A.OverBudget._fields_})
        check(st)
        self.handle = h

    @property
    def n_regions(self) -> int:
        return int(lib().cmn_role_n_regions(self.handle))

    @property
    def n_elements(self) -> int:
        return int(lib().cmn_role_n_elements(self.handle))

    def _args(self, box, var_ids, widths):
        box = np.ascontiguousarray(box, dtype=np.float64)
        vids = np.ascontiguousarray(var_ids, dtype=np.uint64)
        w = np.ascontiguousarray(widths, dtype=np.uint64)
        self._keep = (box, vids, w)
        return A.ptr(box), A.ptr(vids) if len(vids) else None, A.ptr(w) if len(w) else None

    def _candidate(self, cand: A.Candidate) -> CandidateResult:
        n = self.dp.n_vars
        pt = np.ctypeslib.as_array(cand.point, shape=(n,)).copy()
        return CandidateResult(bool(cand.found), float(cand.value), pt, int(cand.index))

    def close(self):
        if getattr(self, "handle", None):
            lib().cmn_role_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _view(ptr, ctype, n: int, owner, dtype):
    """numpy view of role-owned memory that keeps the role alive."""
    buf = (ctype * n).from_address(C.cast(ptr, C.c_void_p).value)
    buf.owner = owner
    return np.frombuffer(buf, dtype=dtype)


class Bounder(_Role):
    kind = A.ROLE_BOUNDER

    def bound(self, box, var_ids, widths):
        """(feasible, obj_lb) per region: views of role-owned storage, valid
        until the next call on this role (backend/backend.hpp:66-67)."""
        fp = C.POINTER(C.c_uint8)()
        lp = C.POINTER(C.c_double)()
        n = C.c_uint64()
        check(lib().cmn_bound(self.handle, *self._args(box, var_ids, widths), C.byref(fp), C.byref(lp), C.byref(n)))
        nr = n.value
        return _view(fp, C.c_uint8, nr, self, np.uint8), _view(lp, C.c_double, nr, self, np.float64)

    def bound_children(self, box, var_ids, widths, k: int):
        """(lb, hull_ub, feasible) of the k children of this region: region r
        belongs to child r // (n_regions // k) (AggregateBounder::bound_children)."""
        out = C.POINTER(A.AggregateBound)()
        check(lib().cmn_bound_children(self.handle, *self._args(box, var_ids, widths), int(k), C.byref(out)))
        arr = (A.AggregateBound * int(k)).from_address(C.cast(out, C.c_void_p).value)
        lb = np.array([arr[i].lb for i in range(k)])
        ub = np.array([arr[i].hull_ub for i in range(k)])
        fe = np.array([arr[i].feasible for i in range(k)], dtype=np.int32)
        return lb, ub, fe


class Sampler(_Role):
    kind = A.ROLE_SAMPLER

    def sample(self, box, var_ids, widths, salt: int) -> CandidateResult:
        cand = A.Candidate()
        check(lib().cmn_sample(self.handle, *self._args(box, var_ids, widths), int(salt), C.byref(cand)))
        return self._candidate(cand)


class Enumerator(_Role):
    kind = A.ROLE_ENUMERATOR

    def enumerate(self, box, var_ids, widths) -> CandidateResult:
        cand = A.Candidate()
        check(lib().cmn_enumerate(self.handle, *self._args(box, var_ids, widths), C.byref(cand)))
        return self._candidate(cand)


def eval_boxes(dp: DeviceProblem, lo: np.ndarray, hi: np.ndarray, precision: int = A.PRECISION_FP64):
    """Fused evaluation of host boxes given as (n_vars, n_boxes) planes."""
    lo = np.ascontiguousarray(lo, dtype=np.float64)
    hi = np.ascontiguousarray(hi, dtype=np.float64)
    nb = lo.shape[1]
    lb = np.empty(nb)
    ub = np.empty(nb)
    fe = np.empty(nb, dtype=np.uint8)
    check(lib().cmn_eval_boxes(dp.handle, precision, A.ptr(lo), A.ptr(hi), nb, nb, A.ptr(lb), A.ptr(ub), A.ptr(fe),
                               0, None))
    return lb, ub, fe


def eval_boxes_device(dp: DeviceProblem, lo_ptr: int, hi_ptr: int, n_boxes: int, stride: int, lb_ptr: int,
                      ub_ptr: int, feas_ptr: int, precision: int = A.PRECISION_FP64, stream: int = 0):
    """Asynchronous fused evaluation of device-resident planes."""
    check(lib().cmn_eval_boxes(dp.handle, precision, lo_ptr, hi_ptr, n_boxes, stride, lb_ptr, ub_ptr, feas_ptr, 1,
                               stream or None))


def default_options(**kw) -> A.SolveOptions:
    o = A.SolveOptions()
    lib().cmn_solve_options_default(C.byref(o))
    for k, v in kw.items():
        if k == "precision" and isinstance(v, str):
            v = A.precision_code(v)
        if k == "known_primal_bound" and v is not None:
            o.has_known_primal = 1
        if v is None:
            continue
        if not hasattr(o, k):
            raise TypeError(f"unknown solve option {k}")
        setattr(o, k, v)
    return o


class Solver:
    """Incremental handle over the batched device solver."""

    def __init__(self, dp: DeviceProblem, **options):
        self.dp = dp
        self.options = default_options(**options)
        h = C.c_void_p()
        check(lib().cmn_solver_create(dp.handle, C.byref(self.options), C.byref(h)))
        self.handle = h

    def step(self, max_iterations: int = 0) -> None:
        check(lib().cmn_solver_step(self.handle, int(max_iterations)))

    def bounds(self):
        lb, ub = C.c_double(), C.c_double()
        check(lib().cmn_query_bounds(self.handle, C.byref(lb), C.byref(ub)))
        return lb.value, ub.value

    def gap(self) -> float:
        g = C.c_double()
        check(lib().cmn_query_gap(self.handle, C.byref(g)))
        return g.value

    def incumbent(self):
        pt = np.empty(self.dp.n_vars)
        f = C.c_int32()
        check(lib().cmn_query_incumbent(self.handle, A.ptr(pt), C.byref(f)))
        return bool(f.value), pt

    def outcome(self) -> dict:
        o = A.Outcome()
        check(lib().cmn_solver_outcome(self.handle, C.byref(o)))
        d = A.outcome_dict(o)
        found, pt = self.incumbent()
        d["best_point"] = pt if found else np.array([])
        return d

    def frontier(self, room: int = 1 << 20):
        """(boxes [count, 2n] interleaved, lower bounds, depths) in pool order."""
        n = self.dp.n_vars
        cnt = C.c_uint64()
        check(lib().cmn_solver_frontier(self.handle, None, None, None, 0, C.byref(cnt)))
        m = min(cnt.value, room)
        boxes = np.empty((m, 2 * n))
        lb = np.empty(m)
        depth = np.empty(m, dtype=np.uint32)
        if m:
            check(lib().cmn_solver_frontier(self.handle, A.ptr(boxes), A.ptr(lb), A.ptr(depth), m, C.byref(cnt)))
        return boxes, lb, depth

    def phase_ms(self) -> list[float]:
        """[select+branch, bound, sample, prune+rebuild, whole] device ms of the
        last iteration, from events recorded inside its graph."""
        ms = (C.c_double * 5)()
        check(lib().cmn_solver_phase_ms(self.handle, ms))
        return list(ms)

    def lazy_ms(self) -> list[float]:
        """Lazy form: [FP64 verdict of the staged parents, FP32 child bounds]
        device ms of the last iteration; the two run at once."""
        ms = (C.c_double * 2)()
        check(lib().cmn_solver_lazy_ms(self.handle, ms))
        return list(ms)

    @property
    def stream(self) -> int:
        return lib().cmn_solver_stream(self.handle) or 0

    def close(self):
        if getattr(self, "handle", None):
            lib().cmn_solver_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve(problem: Problem | DeviceProblem, **options) -> dict:
    dp = problem if isinstance(problem, DeviceProblem) else DeviceProblem(problem)
    s = Solver(dp, **options)
    try:
        s.step(0)
        return s.outcome()
    finally:
        s.close()


# the options a batch fixes for all of its instances
SHARED_OPTIONS = ("precision", "bisection_budget", "batch_parents", "frontier_cap", "sample_points", "sample_all",
                  "relative_width", "max_cycle_size", "enumerate_cap")


def batch_options(**kw) -> A.SolveOptions:
    """Options for a batch: per-instance pools are small (frontier_cap +
    batch_parents * 2^bisection_budget <= 8192), so the defaults differ
    from the single-instance solver's."""
    kw.setdefault("batch_parents", 256)
    kw.setdefault("frontier_cap", 4096)
    return default_options(**kw)


class Batch:
    """Many problems of uneven sizes resident in slots and advanced together
    (cmn_batch_*)."""

    def __init__(self, slots: int, max_vars: int, max_program_slots: int = -1, device: int = 0, **shared):
        self.options = batch_options(**shared)
        cfg = A.BatchConfig()
        cfg.slots = slots
        cfg.max_vars = max_vars
        cfg.max_program_slots = max_program_slots
        cfg.device = device
        cfg.shared = self.options
        h = C.c_void_p()
        check(lib().cmn_batch_create(C.byref(cfg), C.byref(h)))
        self.handle = h
        self.slots: dict[int, DeviceProblem] = {}

    def instance_options(self, **kw) -> A.SolveOptions:
        o = A.SolveOptions()
        C.memmove(C.byref(o), C.byref(self.options), C.sizeof(o))
        for k, v in kw.items():
            if k in SHARED_OPTIONS:
                raise TypeError(f"{k} is fixed by the batch")
            if k == "known_primal_bound" and v is not None:
                o.has_known_primal = 1
            if v is None:
                continue
            if not hasattr(o, k):
                raise TypeError(f"unknown solve option {k}")
            setattr(o, k, v)
        return o

    def add(self, dp: DeviceProblem, **options) -> int:
        o = self.instance_options(**options)
        slot = C.c_uint64()
        check(lib().cmn_batch_add(self.handle, dp.handle, C.byref(o), C.byref(slot)))
        self.slots[slot.value] = dp
        return slot.value

    def step(self, max_iterations: int = 0) -> int:
        running = C.c_uint64()
        check(lib().cmn_batch_step(self.handle, int(max_iterations), C.byref(running)))
        return running.value

    def launch(self, iterations: int) -> None:
        """Enqueues iterations without waiting (see sync)."""
        check(lib().cmn_batch_launch(self.handle, int(iterations)))

    def sync(self) -> int:
        running = C.c_uint64()
        check(lib().cmn_batch_sync(self.handle, C.byref(running)))
        return running.value

    def phase_ms(self) -> list[float]:
        """[select+branch, bound, sample, finish, whole] of the last iteration."""
        ms = (C.c_double * 5)()
        check(lib().cmn_batch_phase_ms(self.handle, ms))
        return list(ms)

    def totals(self) -> tuple[dict, int]:
        """(counters summed over the occupied slots, slots still searching)."""
        c = A.Counters()
        running = C.c_uint64()
        check(lib().cmn_batch_totals(self.handle, C.byref(c), C.byref(running)))
        return {n: int(getattr(c, n)) for n in A.COUNTER_NAMES}, running.value

    def done(self, slot: int) -> bool:
        d = C.c_int32()
        check(lib().cmn_batch_poll(self.handle, slot, C.byref(d)))
        return bool(d.value)

    def outcome(self, slot: int) -> dict:
        o = A.Outcome()
        pt = np.empty(self.slots[slot].n_vars)
        check(lib().cmn_batch_outcome(self.handle, slot, C.byref(o), A.ptr(pt)))
        d = A.outcome_dict(o)
        d["best_point"] = pt if o.found_incumbent else np.array([])
        return d

    def frontier(self, slot: int, room: int = 1 << 16):
        """(boxes [count, 2n] interleaved, lower bounds, depths) of `slot`."""
        n = self.slots[slot].n_vars
        cnt = C.c_uint64()
        check(lib().cmn_batch_frontier(self.handle, slot, None, None, None, 0, C.byref(cnt)))
        m = min(cnt.value, room)
        boxes = np.empty((m, 2 * n))
        lb = np.empty(m)
        depth = np.empty(m, dtype=np.uint32)
        if m:
            check(lib().cmn_batch_frontier(self.handle, slot, A.ptr(boxes), A.ptr(lb), A.ptr(depth), m,
                                           C.byref(cnt)))
        return boxes, lb, depth

    def release(self, slot: int) -> None:
        check(lib().cmn_batch_release(self.handle, slot))
        self.slots.pop(slot, None)

    @property
    def kernels_per_iteration(self) -> int:
        return int(lib().cmn_batch_kernels_per_iteration(self.handle))

    @property
    def stream(self) -> int:
        return lib().cmn_batch_stream(self.handle) or 0

    def close(self):
        if getattr(self, "handle", None):
            lib().cmn_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_solve(problems, slots: int | None = None, per_instance: list[dict] | None = None, **shared) -> list[dict]:
    """Solves every problem through cmn_batch_solve with up to `slots`
    resident at once; returns one outcome dict per problem."""
    dps = [p if isinstance(p, DeviceProblem) else DeviceProblem(p) for p in problems]
    count = len(dps)
    base = batch_options(**{k: v for k, v in shared.items() if k in SHARED_OPTIONS})
    rest = {k: v for k, v in shared.items() if k not in SHARED_OPTIONS}
    cfg = A.BatchConfig()
    cfg.slots = slots or max(1, count)
    cfg.max_vars = max(dp.n_vars for dp in dps) if dps else 1
    cfg.max_program_slots = max(int(dp.info()["program_slots"]) for dp in dps) if dps else 0
    cfg.device = 0
    cfg.shared = base
    opts = (A.SolveOptions * max(1, count))()
    for i in range(count):
        C.memmove(C.byref(opts[i]), C.byref(base), C.sizeof(base))
        kw = dict(rest)
        if per_instance is not None:
            kw.update(per_instance[i])
        for k, v in kw.items():
            if k == "known_primal_bound" and v is not None:
                opts[i].has_known_primal = 1
            if v is not None:
                setattr(opts[i], k, v)
    handles = (C.c_void_p * max(1, count))(*[dp.handle.value for dp in dps])
    outs = (A.Outcome * max(1, count))()
    stride = cfg.max_vars
    pts = np.full(max(1, count) * stride, np.nan)
    check(lib().cmn_batch_solve(C.byref(cfg), handles, opts, count, outs, A.ptr(pts), stride))
    res = []
    for i, dp in enumerate(dps):
        d = A.outcome_dict(outs[i])
        d["best_point"] = pts[i * stride:i * stride + dp.n_vars].copy() if outs[i].found_incumbent else np.array([])
        res.append(d)
    return res


class Server:
    """Continuous-batching request loop (cmn_server_*): one batch per size
    class, requests admitted into free slots within a box-pool memory cap."""

    def __init__(self, classes, pool_budget_bytes: int = 0, iterations_per_round: int = 4, device: int = 0,
                 **shared):
        """`classes`: [(max_vars, slots)] or [(max_vars, slots, max_program_slots)], ascending in max_vars."""
        self.options = batch_options(**shared)
        cfg = A.ServerConfig()
        cfg.shared = self.options
        cfg.device = device
        cfg.n_classes = len(classes)
        for i, c in enumerate(classes):
            cfg.class_max_vars[i] = c[0]
            cfg.class_slots[i] = c[1]
            cfg.class_max_program_slots[i] = c[2] if len(c) > 2 else 0
        cfg.pool_budget_bytes = pool_budget_bytes
        cfg.iterations_per_round = iterations_per_round
        h = C.c_void_p()
        check(lib().cmn_server_create(C.byref(cfg), C.byref(h)))
        self.handle = h
        self._n = {}
        self._keep = {}

    def submit(self, dp: DeviceProblem, **options) -> int:
        o = A.SolveOptions()
        C.memmove(C.byref(o), C.byref(self.options), C.sizeof(o))
        for k, v in options.items():
            if k in SHARED_OPTIONS:
                raise TypeError(f"{k} is fixed by the server")
            if k == "known_primal_bound" and v is not None:
                o.has_known_primal = 1
            if v is not None:
                setattr(o, k, v)
        rid = C.c_uint64()
        check(lib().cmn_server_submit(self.handle, dp.handle, C.byref(o), C.byref(rid)))
        self._n[rid.value] = dp.n_vars
        self._keep[rid.value] = dp
        return rid.value

    def _result(self, rid, o, pt):
        d = A.outcome_dict(o)
        d["best_point"] = pt if o.found_incumbent else np.array([])
        self._keep.pop(rid, None)
        return d

    def poll(self, rid: int):
        """The outcome dict once the request finished, else None."""
        o = A.Outcome()
        pt = np.empty(self._n[rid])
        done = C.c_int32()
        check(lib().cmn_server_poll(self.handle, rid, C.byref(done), C.byref(o), A.ptr(pt)))
        return self._result(rid, o, pt) if done.value else None

    def wait(self, rid: int, timeout_ms: int = 0) -> dict:
        o = A.Outcome()
        pt = np.empty(self._n[rid])
        check(lib().cmn_server_wait(self.handle, rid, timeout_ms, C.byref(o), A.ptr(pt)))
        return self._result(rid, o, pt)

    def stats(self) -> dict:
        s = A.ServerStats()
        check(lib().cmn_server_stats_get(self.handle, C.byref(s)))
        return {f: getattr(s, f) for f, _ in A.ServerStats._fields_}

    def close(self):
        if getattr(self, "handle", None):
            lib().cmn_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
