"""Shared helpers of the GPU parity tests."""

from __future__ import annotations

import copy

import numpy as np

from cuminlp_gb300 import _abi as A
from cuminlp_gb300.problem import Problem


def random_boxes(problem: Problem, n: int, rng: np.random.Generator, scale: float = 0.2):
    """n boxes inside the root box as (n_vars, n) lo/hi planes: random
    centres, widths up to `scale` of the root width, some degenerate."""
    root = np.array(problem.box_bounds)
    c = rng.uniform(root[:, 0:1], root[:, 1:2], (len(root), n))
    w = rng.uniform(0, 1, (len(root), n)) * (root[:, 1:2] - root[:, 0:1]) * scale
    w[:, : n // 16] = 0.0  # degenerate boxes
    lo = np.maximum(c - w, root[:, 0:1])
    hi = np.minimum(c + w, root[:, 1:2])
    kinds = np.array(problem.var_kinds)
    ints = kinds != A.VAR_CONTINUOUS
    lo[ints] = np.ceil(lo[ints])
    hi[ints] = np.maximum(np.floor(hi[ints]), lo[ints])
    return np.ascontiguousarray(lo), np.ascontiguousarray(hi)


def with_objective(problem: Problem, node_id: int) -> Problem:
    """The same DAG with `node_id` as the objective and no constraints: its
    objective enclosure is that node's enclosure."""
    q = copy.deepcopy(problem)
    q.objective_root = node_id
    q.constraints = []
    return q


def ops_problem() -> Problem:
    """A DAG exercising every operator with an interval form, constants on
    either side, const-const nodes, and LE/EQ constraints."""
    p = Problem()
    x = p.var(-3.0, 2.0)
    y = p.var(0.5, 4.0)
    z = p.var(-1.0, 1.0)
    k = p.int_var(0.0, 5.0)
    from cuminlp_gb300.problem import pow, sqr, sqrt
    e1 = (x - y) * (z + 2.0) / y
    e2 = sqrt(y) + sqr(x - z) - 3.0 * k
    e3 = pow(x, 3) + pow(z, 4) - pow(y, -1) + pow(x, 2)
    g = p.graph
    from cuminlp_gb300.problem import Expr
    amin = Expr(g, g.emit(A.OP_MIN, (x.id, z.id)))
    amax = Expr(g, g.emit(A.OP_MAX, (e1.id, z.id)))
    aabs = Expr(g, g.emit(A.OP_ABS, ((x * z).id,)))
    cc = p.fixed(2.0) * p.fixed(-1.5)  # const op const
    obj = e1 + e2 - e3 + amin * amax + aabs + cc + (-x)
    p.set_objective(obj)
    p.add_constraint(x * y - z, A.CMP_LE, 1.0)
    p.add_constraint(x + k, A.CMP_EQ, 2.0)
    p.add_constraint(2.0 - y * y, A.CMP_LE, 0.0)
    return p
