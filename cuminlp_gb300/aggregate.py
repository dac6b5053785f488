"""The aggregate search: branch-and-bound in which each expanded box gets k
children, each bounded by the min/max over its N / k refined subregions
(one device launch) rather than enumerated.

Restates the reference's host-side aggregate loop (aggregate/driver.hpp
AggregateDriver::solve :137-420, frontier.hpp AggregateFrontier,
selection.hpp selection keys, policy.hpp WidestBranchPolicy, history.hpp
IntervalHistory, epilogue.hpp finalise_bounds) over this library's roles:
`Bounder.bound_children` (the fused aggregate fold, cmn_bound_children) and
`Sampler.sample` (cmn_sample).  The host policy is cmn_bisection_choose and
the host decode cmn_slot_bounds, so the refine and the children are the
ones the device decodes.  Pop order, tie-breaking (the frontier's two
binary heaps follow the C++ library's push/pop/make_heap), history slot
reuse and counters follow the reference, so with the same roles the
trajectory is the reference's.
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi as A
from ._lib import check, lib
from .problem import Problem

DBL_MAX = float(np.finfo(np.float64).max)
DBL_LOWEST = -DBL_MAX
K_MAX_SLOTS = 64  # config::kMaxSlots


# -- host policy and decode (the library's) --------------------------------
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


# -- the reference's host point evaluation (model/eval.hpp) -----------------
def _c_div(a: float, b: float) -> float:
    if b != 0.0:
        return a / b
    if a != a or a == 0.0:
        return math.nan
    return math.copysign(math.inf, a) * math.copysign(1.0, b)


def _c_call(f, x):
    try:
        return f(x)
    except OverflowError:
        return math.inf
    except ValueError:
        if f is math.log and x == 0.0:
            return -math.inf
        return math.nan


def _c_pow(x: float, e: float) -> float:
    try:
        return math.pow(x, e)
    except OverflowError:
        return math.copysign(math.inf, x) if (e == int(e) and int(e) % 2 == 1) else math.inf
    except ValueError:
        if x == 0.0 and e < 0:
            odd = e == int(e) and int(e) % 2 == 1
            return math.copysign(math.inf, x) if odd else math.inf
        return math.nan


def _fmin(a, b):
    if a != a:
        return b
    if b != b:
        return a
    return a if a <= b else b


def _fmax(a, b):
    if a != a:
        return b
    if b != b:
        return a
    return a if a >= b else b


def evaluate_nodes(problem: Problem, point, last: int) -> list:
    vals = [0.0] * (last + 1)
    for i in range(last + 1):
        nd = problem.graph.nodes[i]
        op = nd.op
        a = vals[nd.inputs[0]] if nd.inputs else 0.0
        b = vals[nd.inputs[1]] if len(nd.inputs) > 1 else 0.0
        if op == A.OP_VAR:
            v = float(point[nd.var_index])
        elif op == A.OP_CONST:
            v = nd.constant
        elif op == A.OP_ADD:
            v = a + b
        elif op == A.OP_SUB:
            v = a - b
        elif op == A.OP_MUL:
            v = a * b
        elif op == A.OP_DIV:
            v = _c_div(a, b)
        elif op == A.OP_MIN:
            v = _fmin(a, b)
        elif op == A.OP_MAX:
            v = _fmax(a, b)
        elif op == A.OP_NEG:
            v = -a
        elif op == A.OP_SQR:
            v = a * a
        elif op == A.OP_EXP:
            v = _c_call(math.exp, a)
        elif op == A.OP_LOG:
            v = _c_call(math.log, a)
        elif op == A.OP_SQRT:
            v = _c_call(math.sqrt, a)
        elif op == A.OP_SIN:
            v = _c_call(math.sin, a)
        elif op == A.OP_COS:
            v = _c_call(math.cos, a)
        elif op == A.OP_TANH:
            v = math.tanh(a)
        elif op == A.OP_ABS:
            v = math.fabs(a)
        elif op == A.OP_POWN:
            v = _c_pow(a, float(nd.int_exp))
        elif op == A.OP_POW:
            v = _c_pow(a, b)
        else:
            raise ValueError("evaluate: unhandled op")
        vals[i] = v
    return vals


def satisfies(lhs: float, cmp: int, rhs: float, abs_tol: float = 1e-8, rel_tol: float = 1e-6) -> bool:
    if cmp == A.CMP_LE:
        return lhs <= rhs
    diff = math.fabs(lhs - rhs)
    if diff <= abs_tol:
        return True
    return diff <= rel_tol * _fmax(math.fabs(lhs), math.fabs(rhs))


def witness_is_admissible(point, var_kinds, box_bounds) -> bool:
    """search::witness_is_admissible (epilogue.hpp:35-59)."""
    for x, k, (lb, ub) in zip(point, var_kinds, box_bounds):
        if not (x >= lb) or not (x <= ub):
            return False
        if k != A.VAR_CONTINUOUS and math.fabs(x - round(x)) > 1e-6:
            return False
    return True


# -- WidestBranchPolicy (policy.hpp) ----------------------------------------
@dataclass
class Partition:
    branch: SlotAssignment
    refine: SlotAssignment
    launch: SlotAssignment
    k: int
    m: int
    nested: bool = False

    def is_leaf(self) -> bool:
        return self.branch.size() == 0


def _partition_kind(var_kind: int) -> int:
    return A.SLOT_CONTINUOUS if var_kind == A.VAR_CONTINUOUS else A.SLOT_INTEGER_PARTITION


class WidestBranchPolicy:
    """k-way split of the widest live variable (branch), plus a
    BisectionBudget refine of log2(N / k) bits over the rest."""

    def __init__(self, branch_fan_out: int, total_fan_out: int, max_cycle: int = 0, enumerate_cap: int = 0,
                 relative: bool = False):
        def pow2(v):
            return v != 0 and (v & (v - 1)) == 0
        if branch_fan_out < 2 or not pow2(branch_fan_out):
            raise ValueError("branch fan-out k must be a power of two and at least 2")
        if total_fan_out <= branch_fan_out or not pow2(total_fan_out):
            raise ValueError("total fan-out N must be a power of two strictly greater than k")
        self.k, self.n = branch_fan_out, total_fan_out
        self.m = total_fan_out // branch_fan_out
        self.bits = self.m.bit_length() - 1
        self.max_cycle, self.enumerate_cap, self.relative = max_cycle, enumerate_cap, relative

    @staticmethod
    def _widest_live(box):
        best, best_key = None, 0.0
        for i, (lb, ub) in enumerate(box):
            if not (ub > lb):
                continue
            key = ub - lb
            if best is None or key > best_key:
                best, best_key = i, key
        return best

    def branch(self, box, var_kinds) -> SlotAssignment:
        vid = self._widest_live(box)
        if vid is None:
            return SlotAssignment()
        return SlotAssignment([_partition_kind(var_kinds[vid])], [vid], [self.k], [self.k])

    def partition(self, box, var_kinds) -> Partition:
        br = self.branch(box, var_kinds)
        out = Partition(br, SlotAssignment(), SlotAssignment(), self.k, self.m)
        if br.size() == 0:
            return out
        bvid = br.var_ids[0]
        if sum(1 for lb, ub in box if ub > lb) == 1:
            out.nested = True
            out.launch = SlotAssignment([br.kinds[0]], [bvid], [self.n], [self.n])
            return out
        masked = [tuple(b) for b in box]
        masked[bvid] = (masked[bvid][0], masked[bvid][0])
        flat = np.array([x for b in masked for x in b], dtype=np.float64)
        refine = bisection_choose(flat, var_kinds, self.bits, self.max_cycle, self.enumerate_cap, self.relative)
        # pad with width-1 slots for the remaining live variables
        cap = K_MAX_SLOTS - 1
        for vid, (lb, ub) in enumerate(box):
            if refine.size() >= cap:
                break
            if vid == bvid or not (ub > lb) or vid in refine.var_ids:
                continue
            refine.kinds.append(_partition_kind(var_kinds[vid]))
            refine.var_ids.append(vid)
            refine.widths.append(1)
            refine.domains.append(1)
        out.refine = refine
        out.launch = SlotAssignment(refine.kinds + br.kinds, refine.var_ids + br.var_ids,
                                    refine.widths + br.widths, refine.domains + br.domains)
        return out


# -- frontier: two heaps over one node store (frontier.hpp) ----------------
def _push_hole(h, hole, top, value, less):
    parent = (hole - 1) // 2
    while hole > top and less(h[parent], value):
        h[hole] = h[parent]
        hole = parent
        parent = (hole - 1) // 2
    h[hole] = value


def _adjust(h, hole, length, value, less):
    top = hole
    second = hole
    while second < (length - 1) // 2:
        second = 2 * (second + 1)
        if less(h[second], h[second - 1]):
            second -= 1
        h[hole] = h[second]
        hole = second
    if (length & 1) == 0 and second == (length - 2) // 2:
        second = 2 * (second + 1)
        h[hole] = h[second - 1]
        hole = second - 1
    _push_hole(h, hole, top, value, less)


def push_heap(h, value, less):
    h.append(value)
    _push_hole(h, len(h) - 1, 0, value, less)


def pop_heap(h, less):
    if len(h) > 1:
        value = h[-1]
        h[-1] = h[0]
        _adjust(h, 0, len(h) - 1, value, less)
    return h.pop()


def make_heap(h, less):
    n = len(h)
    if n < 2:
        return
    parent = (n - 2) // 2
    while True:
        _adjust(h, parent, n, h[parent], less)
        if parent == 0:
            return
        parent -= 1


def selection_key(rule: str, lb: float, hull_ub: float, f_best: float) -> float:
    """selection.hpp selection_key."""
    if rule == "least-lower-bound":
        return lb
    if not (f_best < DBL_MAX):
        return lb
    width = hull_ub - lb
    if not (width > 0.0):
        return -math.inf if lb < f_best else math.inf
    return -((f_best - lb) / width)


@dataclass
class AggregateNode:
    sidx: int
    pidx: int
    depth: int
    lb: float
    hull_ub: float
    branch_key: tuple = ()


def _is_better(a, b) -> bool:
    # refs are (key, depth, pidx, slot, gen)
    if a[0] < b[0]:
        return True
    if b[0] < a[0]:
        return False
    if a[1] != b[1]:
        return a[1] > b[1]
    return a[2] > b[2]


def _heap_less(a, b) -> bool:
    return _is_better(b, a)


class AggregateFrontier:
    def __init__(self, rule: str = "least-lower-bound"):
        if rule not in ("least-lower-bound", "reject-index", "reject-index-stale"):
            raise ValueError(f"unknown selection rule {rule}")
        self.rule = rule
        self.slots: list = []  # [node, gen, alive]
        self.free: list = []
        self.by_key: list = []
        self.by_lb: list = []
        self.live = 0

    def empty(self) -> bool:
        return self.live == 0

    def _ref(self, slot, key):
        node, gen, _ = self.slots[slot]
        return (key, node.depth, node.pidx, slot, gen)

    def _current(self, ref) -> bool:
        node, gen, alive = self.slots[ref[3]]
        return alive and gen == ref[4]

    def enqueue(self, node: AggregateNode, f_best: float):
        if self.free:
            slot = self.free.pop()
            self.slots[slot] = [node, self.slots[slot][1] + 1, True]
        else:
            slot = len(self.slots)
            self.slots.append([node, 0, True])
        self.live += 1
        push_heap(self.by_key, self._ref(slot, selection_key(self.rule, node.lb, node.hull_ub, f_best)), _heap_less)
        push_heap(self.by_lb, self._ref(slot, node.lb), _heap_less)

    def pop(self) -> AggregateNode:
        while self.by_key:
            ref = pop_heap(self.by_key, _heap_less)
            if not self._current(ref):
                continue
            node = self.slots[ref[3]][0]
            self.slots[ref[3]][2] = False
            self.live -= 1
            self.free.append(ref[3])
            self._collect_garbage()
            return node
        raise RuntimeError("pop() on an empty frontier")

    def min_lb(self) -> float:
        while self.by_lb and not self._current(self.by_lb[0]):
            pop_heap(self.by_lb, _heap_less)
        return self.slots[self.by_lb[0][3]][0].lb if self.by_lb else DBL_MAX

    def on_incumbent(self, f_best: float):
        if self.rule != "reject-index":
            return
        self.by_key, self.by_lb = [], []
        for slot, (node, gen, alive) in enumerate(self.slots):
            if alive:
                self.by_key.append(self._ref(slot, selection_key(self.rule, node.lb, node.hull_ub, f_best)))
                self.by_lb.append(self._ref(slot, node.lb))
        make_heap(self.by_key, _heap_less)
        make_heap(self.by_lb, _heap_less)

    def count_viable(self, gub: float) -> int:
        return sum(1 for node, gen, alive in self.slots if alive and not (node.lb > gub))

    def _collect_garbage(self):
        if len(self.by_key) + len(self.by_lb) <= 2 * self.live + 64:
            return
        for name in ("by_key", "by_lb"):
            kept = [r for r in getattr(self, name) if self._current(r)]
            make_heap(kept, _heap_less)
            setattr(self, name, kept)


class IntervalHistory:
    """search::IntervalHistory: refcounted parent boxes; slot 0 is the root
    sentinel and freed slots are reused last-in first-out."""

    def __init__(self):
        self.intervals: list = []
        self.refs: list = []
        self.free: list = []
        self.freed = 0
        self.peak_live = 0

    def enqueue(self, box) -> int:
        if self.free:
            idx = self.free.pop()
            self.intervals[idx] = box
            self.refs[idx] = 1
        else:
            idx = len(self.intervals)
            self.intervals.append(box)
            self.refs.append(1)
        self.peak_live = max(self.peak_live, len(self.intervals) - len(self.free))
        return idx

    def add_ref(self, idx: int):
        if idx != 0:
            self.refs[idx] += 1

    def release(self, idx: int):
        if idx == 0:
            return
        self.refs[idx] -= 1
        if self.refs[idx] > 0:
            return
        self.intervals[idx] = None
        self.free.append(idx)
        self.freed += 1


# -- roles on the device -----------------------------------------------------
class DeviceAggregateRoles:
    """The bounder and sampler for each launch composition
    (AggregateRoleCache), built on first use."""

    def __init__(self, dp, bound_regions: int, k: int, sample_regions: int, sample_points: int = 1):
        from .solver import Bounder, Sampler
        self._Bounder, self._Sampler = Bounder, Sampler
        self.dp = dp
        self.n, self.k, self.ns, self.s = bound_regions, k, sample_regions, sample_points
        self.bounders: dict = {}
        self.samplers: dict = {}

    def n_samples(self) -> int:
        return self.ns * self.s

    def bound_children(self, box, launch: SlotAssignment):
        key = tuple(launch.kinds)
        if key not in self.bounders:
            self.bounders[key] = self._Bounder(self.dp, launch.kinds, self.n)
        flat = np.array([x for b in box for x in b], dtype=np.float64)
        return self.bounders[key].bound_children(flat, launch.var_ids, launch.widths, self.k)

    def sample(self, box, launch: SlotAssignment, salt: int):
        key = tuple(launch.kinds)
        if key not in self.samplers:
            self.samplers[key] = self._Sampler(self.dp, launch.kinds, self.ns, sample_points=self.s)
        flat = np.array([x for b in box for x in b], dtype=np.float64)
        c = self.samplers[key].sample(flat, launch.var_ids, launch.widths, salt)
        return c.found, c.value, c.point


# -- the driver ----------------------------------------------------------------
def _gap_closed(gub: float, bound: float, tol: float) -> bool:
    return gub - bound <= tol * max(1.0, abs(gub))


class AggregateDriver:
    """AggregateDriver::solve (aggregate/driver.hpp:137-420)."""

    def __init__(self, policy: WidestBranchPolicy, sampler_policy: WidestBranchPolicy, roles,
                 rule: str = "least-lower-bound", iter_limit: int = 100000, tolerance: float = 1e-6,
                 known_primal_bound: float | None = None):
        self.policy, self.sampler_policy, self.roles = policy, sampler_policy, roles
        self.rule, self.iter_limit, self.tol = rule, iter_limit, tolerance
        self.known = known_primal_bound

    def solve(self, problem: Problem) -> dict:
        gub = self.known if self.known is not None else DBL_MAX
        best_point: list = []
        kinds = list(problem.var_kinds)
        root = [tuple(b) for b in problem.box_bounds]
        frontier = AggregateFrontier(self.rule)
        history = IntervalHistory()
        history.enqueue([])  # slot 0: the root sentinel
        frontier.enqueue(AggregateNode(0, 0, 0, DBL_LOWEST, DBL_MAX), gub)
        it = 0
        converged = stopped_early = engaged = False
        stop = "iteration-limit"
        c = dict(bounded=0, sampled=0, enqueued=0, fathomed=0, pruned_infeasible=0, pruned_dominated=0,
                 witness_rejected=0)
        glb = DBL_LOWEST
        while it < self.iter_limit and not frontier.empty():
            flb = frontier.min_lb()
            glb = flb
            if _gap_closed(gub, flb, self.tol):
                converged = stopped_early = True
                stop = "converged"
                break
            it += 1
            cur = frontier.pop()
            if cur.pidx == 0:
                box = list(root)
            else:
                parent = history.intervals[cur.pidx]
                branch = self.policy.branch(parent, kinds)
                if branch.key() != cur.branch_key:
                    raise RuntimeError("the branch policy is not a pure function of (box, var_kinds)")
                box = materialise(parent, cur.sidx, branch)
            history.release(cur.pidx)
            part = self.policy.partition(box, kinds)
            if part.is_leaf():
                c["fathomed"] += 1
                gub, best_point, frontier = self._fold_point(problem, box, gub, best_point, c, frontier)
                continue
            spart = self.sampler_policy.partition(box, kinds)
            box_idx = history.enqueue(box)
            if not spart.is_leaf():
                found, value, point = self.roles.sample(box, spart.launch, it)
                c["sampled"] += self.roles.n_samples()
                if found and value < gub:
                    if witness_is_admissible(point, kinds, problem.box_bounds):
                        gub = float(value)
                        best_point = [float(x) for x in point]
                        frontier.on_incumbent(gub)
                        engaged = True
                    else:
                        c["witness_rejected"] += 1
            lbs, ubs, fes = self.roles.bound_children(box, part.launch)
            c["bounded"] += len(lbs)
            bkey = part.branch.key()
            for ch in range(len(lbs)):
                if not fes[ch]:
                    c["pruned_infeasible"] += 1
                    continue
                lb = max(float(lbs[ch]), cur.lb)
                if lb > float(ubs[ch]):
                    c["pruned_infeasible"] += 1
                    continue
                if lb > gub:
                    c["pruned_dominated"] += 1
                    continue
                frontier.enqueue(AggregateNode(ch, box_idx, cur.depth + 1, lb, float(ubs[ch]), bkey), gub)
                history.add_ref(box_idx)
                c["enqueued"] += 1
            history.release(box_idx)
        if not stopped_early:
            stop = "exhausted" if frontier.empty() else "iteration-limit"
        found = gub < DBL_MAX
        viable = frontier.count_viable(gub)
        fmin = DBL_MAX if frontier.empty() else frontier.min_lb()
        # finalise_bounds (search/epilogue.hpp:89-127); nothing is ever dropped
        proven = found and (converged or frontier.empty() or viable == 0) and _gap_closed(gub, math.inf, self.tol)
        infeasible = False
        if proven:
            glb = gub
        elif frontier.empty():
            infeasible = True
        else:
            glb = min(fmin, math.inf)
            if found:
                glb = min(glb, gub)
        counters = dict(iterations=it, fathomed=c["fathomed"], fathomed_points=c["fathomed"],
                        bounded=c["bounded"], sampled=c["sampled"], enqueued=c["enqueued"],
                        witness_rejected=c["witness_rejected"], pruned_duplicate=0,
                        pruned_infeasible=c["pruned_infeasible"], pruned_dominated=c["pruned_dominated"],
                        pending=frontier.live, viable=viable, history_freed=history.freed,
                        history_peak_live=history.peak_live)
        return dict(lower_bound=glb, upper_bound=gub, best_point=best_point, stop_reason=stop,
                    proven_optimal=bool(proven), infeasible=bool(infeasible), counters=counters,
                    selection_rule_engaged=bool(engaged or self.rule != "reject-index"))

    def _fold_point(self, problem, box, gub, best_point, c, frontier):
        point = [b[0] for b in box]
        vals = evaluate_nodes(problem, point, len(problem.graph.nodes) - 1) if problem.graph.nodes else []
        for con in problem.constraints:
            if not satisfies(vals[con.root_id], con.cmp, con.rhs):
                return gub, best_point, frontier
        value = vals[problem.objective_root]
        if not (value < gub):
            return gub, best_point, frontier
        if not witness_is_admissible(point, problem.var_kinds, problem.box_bounds):
            c["witness_rejected"] += 1
            return gub, best_point, frontier
        frontier.on_incumbent(value)
        return value, point, frontier


def solve_aggregate(problem: Problem, branch_fan_out: int = 2, total_fan_out: int = 1 << 12,
                    sample_fan_out: int = 1 << 8, sample_points: int = 1, rule: str = "least-lower-bound",
                    iter_limit: int = 100000, tolerance: float = 1e-6, known_primal_bound: float | None = None,
                    roles=None) -> dict:
    """Runs the aggregate search with the device roles (or `roles`)."""
    from .solver import DeviceProblem
    policy = WidestBranchPolicy(branch_fan_out, total_fan_out)
    spolicy = WidestBranchPolicy(branch_fan_out, sample_fan_out)
    if roles is None:
        roles = DeviceAggregateRoles(DeviceProblem(problem), total_fan_out, branch_fan_out, sample_fan_out,
                                     sample_points)
    return AggregateDriver(policy, spolicy, roles, rule, iter_limit, tolerance, known_primal_bound).solve(problem)
