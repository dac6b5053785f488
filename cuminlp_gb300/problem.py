"""Problem / Expr builder: the host-side mirror of the reference's model API.

Mirrors ``model::Expr`` and ``model::Problem`` (model/problem.hpp:35-358):
the same operator overloads, the same node-emission order, the same
constant folding (``a * a`` on one node emits ``Sqr``; unary ops on a
``Const`` fold), and the same ``validate()`` rules.  ``Problem.desc()``
flattens the DAG into the C ABI's ``cmn_problem_desc``.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi as A


class InvalidDAG(ValueError):
    """model::InvalidDAG (errors.hpp)."""


class InvalidProblem(ValueError):
    """model::InvalidProblem (errors.hpp)."""


@dataclass
class Node:
    id: int
    op: int
    inputs: tuple
    constant: float = 0.0
    var_index: int = 0
    int_exp: int = 0
    op_count: int = 1


class ExprDAG:
    """model::ExprDAG (model/dag.hpp:70-93)."""

    def __init__(self):
        self.nodes: list[Node] = []

    def emit(self, op: int, inputs=(), constant=0.0, var_index=0, int_exp=0) -> int:
        nid = len(self.nodes)
        op_count = 1 + sum(self.nodes[i].op_count for i in inputs)
        self.nodes.append(Node(nid, op, tuple(inputs), float(constant), int(var_index), int(int_exp), op_count))
        return nid


class Expr:
    """model::Expr (model/problem.hpp:35-164)."""

    __slots__ = ("graph", "id")

    def __init__(self, graph: ExprDAG, nid: int):
        self.graph = graph
        self.id = nid

    # -- helpers
    def _is_const(self) -> bool:
        return self.graph.nodes[self.id].op == A.OP_CONST

    def _const_value(self) -> float:
        return self.graph.nodes[self.id].constant

    def constant(self, c: float) -> "Expr":
        return Expr(self.graph, self.graph.emit(A.OP_CONST, (), constant=c))

    def _lift(self, other) -> "Expr":
        return other if isinstance(other, Expr) else self.constant(float(other))

    # -- binary operators: a T operand becomes a Const node first
    def __add__(self, other):
        b = self._lift(other)
        return Expr(self.graph, self.graph.emit(A.OP_ADD, (self.id, b.id)))

    def __radd__(self, other):
        a = self.constant(float(other))
        return Expr(self.graph, self.graph.emit(A.OP_ADD, (a.id, self.id)))

    def __sub__(self, other):
        b = self._lift(other)
        return Expr(self.graph, self.graph.emit(A.OP_SUB, (self.id, b.id)))

    def __rsub__(self, other):
        a = self.constant(float(other))
        return Expr(self.graph, self.graph.emit(A.OP_SUB, (a.id, self.id)))

    def __mul__(self, other):
        b = self._lift(other)
        return _mul(self, b)

    def __rmul__(self, other):
        a = self.constant(float(other))
        return _mul(a, self)

    def __truediv__(self, other):
        b = self._lift(other)
        return Expr(self.graph, self.graph.emit(A.OP_DIV, (self.id, b.id)))

    def __rtruediv__(self, other):
        a = self.constant(float(other))
        return Expr(self.graph, self.graph.emit(A.OP_DIV, (a.id, self.id)))

    def __neg__(self):
        if self._is_const():
            return self.constant(-self._const_value())
        return Expr(self.graph, self.graph.emit(A.OP_NEG, (self.id,)))


def _mul(a: Expr, b: Expr) -> Expr:
    if a.id == b.id:
        if a._is_const():
            return a.constant(a._const_value() * a._const_value())
        return Expr(a.graph, a.graph.emit(A.OP_SQR, (a.id,)))
    return Expr(a.graph, a.graph.emit(A.OP_MUL, (a.id, b.id)))


def sqr(a: Expr) -> Expr:
    return a * a


def _unary(op: int, fold):
    def f(a: Expr) -> Expr:
        if a._is_const():
            return a.constant(fold(a._const_value()))
        return Expr(a.graph, a.graph.emit(op, (a.id,)))
    return f


sqrt = _unary(A.OP_SQRT, math.sqrt)
exp = _unary(A.OP_EXP, math.exp)
log = _unary(A.OP_LOG, math.log)


def pow(a: Expr, n) -> Expr:  # noqa: A001 - mirrors the reference's free function
    if isinstance(n, Expr):
        if a._is_const() and n._is_const():
            return a.constant(math.pow(a._const_value(), n._const_value()))
        return Expr(a.graph, a.graph.emit(A.OP_POW, (a.id, n.id)))
    if a._is_const():
        return a.constant(float(a._const_value() ** int(n)))
    return Expr(a.graph, a.graph.emit(A.OP_POWN, (a.id,), int_exp=int(n)))


@dataclass
class Constraint:
    root_id: int
    cmp: int
    rhs: float


@dataclass
class Problem:
    """model::Problem<double> (model/problem.hpp:195-358)."""

    graph: ExprDAG = field(default_factory=ExprDAG)
    box_bounds: list = field(default_factory=list)
    var_kinds: list = field(default_factory=list)
    objective_root: int = -1
    constraints: list = field(default_factory=list)

    def var(self, lb: float = -np.finfo(np.float64).max, ub: float = np.finfo(np.float64).max,
            kind: int = A.VAR_CONTINUOUS) -> Expr:
        idx = len(self.box_bounds)
        self.box_bounds.append((float(lb), float(ub)))
        self.var_kinds.append(int(kind))
        return Expr(self.graph, self.graph.emit(A.OP_VAR, (), var_index=idx))

    def int_var(self, lb: float, ub: float) -> Expr:
        return self.var(lb, ub, A.VAR_INTEGER)

    def bin_var(self) -> Expr:
        return self.var(0.0, 1.0, A.VAR_BINARY)

    def fixed(self, value: float) -> Expr:
        return Expr(self.graph, self.graph.emit(A.OP_CONST, (), constant=value))

    def set_objective(self, e: Expr) -> None:
        self.objective_root = e.id

    def add_constraint(self, lhs: Expr, cmp: int, rhs: float) -> None:
        self.constraints.append(Constraint(lhs.id, int(cmp), float(rhs)))

    # -- validate (model/problem.hpp:282-355)
    def validate(self) -> None:
        nodes = self.graph.nodes
        for nd in nodes:
            for i in nd.inputs:
                if i >= nd.id:
                    raise InvalidDAG("DAG node operand id is not strictly less than the node's own id")
            if nd.op_count != 1 + sum(nodes[i].op_count for i in nd.inputs):
                raise InvalidDAG("DAG node op_count does not match the size of its subtree")
        if sum(1 for nd in nodes if nd.op == A.OP_VAR) != len(self.box_bounds) or \
                len(self.box_bounds) != len(self.var_kinds):
            raise InvalidDAG("box_bounds/var_kinds are out of sync with the number of Op::Var nodes")
        if 0 <= self.objective_root < len(nodes) and nodes[self.objective_root].op == A.OP_CONST:
            raise InvalidDAG("objective root is a bare Const")
        for c in self.constraints:
            if nodes[c.root_id].op == A.OP_CONST:
                raise InvalidDAG("constraint root is a bare Const")
        if not self.var_kinds:
            raise InvalidProblem("Problem has zero variables")
        if self.objective_root < 0:
            raise InvalidProblem("Problem's objective was never set (set_objective was never called)")
        for (lb, ub), k in zip(self.box_bounds, self.var_kinds):
            if not lb <= ub:
                raise InvalidProblem("variable's lower bound exceeds its upper bound")
            if k in (A.VAR_INTEGER, A.VAR_BINARY) and (math.floor(lb) < lb or math.floor(ub) < ub):
                raise InvalidProblem("Integer/Binary variable has non-integer-valued bounds")
            if k == A.VAR_BINARY and (lb != 0.0 or ub != 1.0):
                raise InvalidProblem("Binary variable's bounds are not exactly [0,1]")
        for c in self.constraints:
            if not math.isfinite(c.rhs):
                raise InvalidProblem("constraint rhs must be finite")

    # -- flattening for the C ABI
    def arrays(self):
        nodes = np.zeros(len(self.graph.nodes), dtype=A.NODE_DTYPE)
        for nd in self.graph.nodes:
            r = nodes[nd.id]
            r["op"] = nd.op
            r["n_in"] = len(nd.inputs)
            r["in0"] = nd.inputs[0] if len(nd.inputs) > 0 else -1
            r["in1"] = nd.inputs[1] if len(nd.inputs) > 1 else -1
            r["var_index"] = nd.var_index
            r["constant"] = nd.constant
            r["int_exp"] = nd.int_exp
        lb = np.array([b[0] for b in self.box_bounds], dtype=np.float64)
        ub = np.array([b[1] for b in self.box_bounds], dtype=np.float64)
        kinds = np.array(self.var_kinds, dtype=np.int32)
        cons = np.zeros(len(self.constraints), dtype=A.CONSTRAINT_DTYPE)
        for i, c in enumerate(self.constraints):
            cons[i]["root"] = c.root_id
            cons[i]["cmp"] = c.cmp
            cons[i]["rhs"] = c.rhs
        return nodes, lb, ub, kinds, cons

    def desc(self, arrays=None, objective_root: int | None = None, constraints: bool = True):
        """Returns (ProblemDesc, keepalive) for the C ABI.  `arrays` reuses
        an earlier arrays() result; `objective_root` and `constraints=False`
        describe the same DAG rooted at another node, unconstrained (that
        objective's enclosure is the node's enclosure)."""
        nodes, lb, ub, kinds, cons = self.arrays() if arrays is None else arrays
        if not constraints:
            cons = cons[:0]
        d = A.ProblemDesc()
        d.nodes = nodes.ctypes.data
        d.n_nodes = len(nodes)
        d.var_lb = lb.ctypes.data
        d.var_ub = ub.ctypes.data
        d.var_kinds = kinds.ctypes.data
        d.n_vars = len(lb)
        d.objective_root = self.objective_root if objective_root is None else int(objective_root)
        d.constraints = cons.ctypes.data if len(cons) else None
        d.n_constraints = len(cons)
        return d, (nodes, lb, ub, kinds, cons)

    @property
    def n_vars(self) -> int:
        return len(self.box_bounds)

    def root_box(self) -> np.ndarray:
        """Interleaved (lb, ub) pairs: the layout of cu::interval<double>[n]."""
        return np.array(self.box_bounds, dtype=np.float64).reshape(-1)
