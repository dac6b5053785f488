"""CPU: the oracle against the reference's own known answers that pin this
path and run without Catch2 or a GPU.

- The cost model's count of buffer-bearing nodes
  (backend/graph/cost.hpp:38-68): graph_replay_test.cu:463-480.

- The epilogue (search/epilogue.hpp:89-127, finalise_bounds, with
  DropAccounting, search/budget.hpp:190-209): every case of
  host_budget_test.cpp:398-500, at the driver's tolerance of 1e-6, with
  the test's rule that a run found an incumbent when gub is below the
  no-incumbent sentinel (DBL_MAX).
- Point evaluation and the constraint predicates
  (model/eval.hpp:186-200, backend/graph/kernels.cuh:283-340): the cases of
  dag_test.cpp:440-527 -- LE exact, EQ within 1e-8 absolute or 1e-6
  relative, NaN infeasible in both."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import _abi as A
from cuminlp_gb300.problem import Problem

NO_INCUMBENT = np.finfo(np.float64).max


# (glb, gub, converged, pending_empty, frontier_min, viable, drops) ->
# (proven_optimal, infeasible, reported lower bound)
EPILOGUE_CASES = {
    # "with nothing dropped the epilogue behaves exactly as before"
    "emptied_with_incumbent_is_proven": ((1.0, 5.0, False, True, 0.0, 0, []), (True, False, 5.0)),
    "emptied_without_incumbent_is_infeasible": ((1.0, NO_INCUMBENT, False, True, 0.0, 0, []), (False, True, 1.0)),
    "stranded_frontier_clamped_to_incumbent": ((1.0, 5.0, False, False, 9.0, 0, []), (True, False, 5.0)),
    "unfinished_run_reports_frontier_min": ((1.0, 5.0, False, False, 2.0, 3, []), (False, False, 2.0)),
    # "a dominated-only drop still permits proven optimality"
    "dominated_drop_still_proven": ((1.0, 5.0, False, True, 0.0, 0, [(40.0, 5.0)]), (True, False, 5.0)),
    # "a viable drop caps the reported lower bound"
    "viable_floor_beats_emptied_frontier": ((1.0, 5.0, False, True, 0.0, 0, [(2.0, 5.0)]), (False, False, 2.0)),
    "viable_floor_beats_higher_frontier": ((1.0, 5.0, False, False, 4.0, 1, [(2.0, 5.0)]), (False, False, 2.0)),
    "lower_frontier_min_still_wins": ((1.0, 5.0, False, False, 1.5, 1, [(2.0, 5.0)]), (False, False, 1.5)),
    # "a viable drop within tolerance is still proven optimal"
    "viable_drop_within_tolerance": ((1.0, 5.0, True, False, 5.0, 1, [(5.0 - 1e-9, 5.0)]), (True, False, 5.0)),
    # "an emptied frontier with viable drops is not infeasible"
    "viable_drops_block_infeasibility": ((1.0, NO_INCUMBENT, False, True, 0.0, 0, [(-3.0, NO_INCUMBENT)]),
                                         (False, False, -3.0)),
}


@pytest.mark.parametrize("name", list(EPILOGUE_CASES))
def test_epilogue_known_answers(name):
    (glb, gub, converged, pending_empty, frontier_min, viable, drops), (proven, infeasible, lb) = EPILOGUE_CASES[name]
    got = O.finalise(glb, gub, converged, pending_empty, frontier_min, viable, drops)
    assert got[0] == proven and got[1] == infeasible
    assert got[2] == pytest.approx(lb, rel=0, abs=1e-12)


def test_buffer_node_count_counts_only_reachable_nodes():
    # graph_replay_test.cu:463-480 over backend/graph/cost.hpp:38-68: the
    # cost model counts the non-Const nodes a root reaches; an expression no
    # root refers to adds nothing
    p = Problem()
    x = p.var(0.0, 10.0)
    p.set_objective(x * x)
    p.add_constraint(x, A.CMP_LE, 5.0)
    reachable = O.OracleProblem(p).buffer_node_count
    dead = p.var(0.0, 1.0) * p.var(0.0, 1.0)
    assert dead is not None
    assert O.OracleProblem(p).buffer_node_count == reachable == 2  # x and x*x
    assert reachable < len(p.graph.nodes)


def test_point_evaluation_every_root():
    # dag_test.cpp:440-460: shared = x*x + y; objective shared + y,
    # constraint shared - x <= 4; at (2, 3) the objective is 10 and the
    # constraint reads 5, so the point is infeasible
    p = Problem()
    x, y = p.var(-5.0, 5.0), p.var(-5.0, 5.0)
    shared = x * x + y
    p.set_objective(shared + y)
    p.add_constraint(shared - x, A.CMP_LE, 4.0)
    obj, feas = O.OracleProblem(p).eval_point([2.0, 3.0])
    assert obj == 10.0 and not feas


def one_constraint(cmp: int, rhs: float) -> O.OracleProblem:
    p = Problem()
    x = p.var(-10.0, 1e7)
    p.set_objective(x * x)
    p.add_constraint(x, cmp, rhs)
    return O.OracleProblem(p)


@pytest.mark.parametrize("cmp,rhs,x,ok", [
    (A.CMP_LE, 1.0, 1.0, True),            # LE is exact
    (A.CMP_LE, 1.0, 0.5, True),
    (A.CMP_LE, 1.0, 1.0 + 1e-12, False),
    (A.CMP_EQ, 1.0, 1.0, True),            # EQ: 1e-8 absolute or 1e-6 relative
    (A.CMP_EQ, 1.0, 1.0 + 1e-10, True),
    (A.CMP_EQ, 1.0, 1.0 + 1e-3, False),
    (A.CMP_EQ, 1e6, 1e6 + 1e-4, True),     # the relative arm
    (A.CMP_LE, 1.0, float("nan"), False),  # NaN fails every comparison
    (A.CMP_EQ, 1.0, float("nan"), False),
])
def test_constraint_predicates(cmp, rhs, x, ok):
    # dag_test.cpp:475-498, satisfies() mirroring the device's predicates
    _, feas = one_constraint(cmp, rhs).eval_point([x])
    assert feas == ok


def test_first_violated_constraint_and_no_constraints():
    # dag_test.cpp:500-527: the EQ constraint binds at (3, 4); a model
    # without constraints is satisfied everywhere
    p = Problem()
    x, y = p.var(0.0, 10.0), p.var(0.0, 10.0)
    p.set_objective(x + y)
    p.add_constraint(x + y, A.CMP_LE, 100.0)
    p.add_constraint(x - y, A.CMP_EQ, 0.0)
    op = O.OracleProblem(p)
    assert op.eval_point([3.0, 3.0])[1]
    assert not op.eval_point([3.0, 4.0])[1]
    q = Problem()
    z = q.var(0.0, 1.0)
    q.set_objective(z * z)
    assert O.OracleProblem(q).eval_point([0.5]) == (0.25, True)
