"""CPU: the compiled program keeps every node's roundings in their order.

The library compiles a problem's DAG into a straight-line program (sum
chains folded into TERM instructions, shared intermediates in liveness-
allocated slots) and the plain FP64 form evaluates that program.  Here the
program comes from cmn_program_compile (no GPU) and runs through the
oracle's restatement of the interpreter with every operation rounded on its
own; its enclosures and feasibility verdicts must equal the oracle's
node-by-node evaluation of the DAG -- the reference's per-node kernel chain
(backend/graph/kernels.cuh:177-419) -- bit for bit.  A mistake planted in
the program is caught the same way."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import _abi as A
from cuminlp_gb300 import generators as G
from cuminlp_gb300.problem import Problem
from cuminlp_gb300.solver import compile_program
from tests.gpu_common import ops_problem, random_boxes, with_objective
from tests.test_oracle_pins import fixture_problems

OP_TERM, T_HASC = 1, 4  # instruction opcode (head bits 0-2) and term sub-code bit (head bits 3-7)


def mismatches(p: Problem, code: np.ndarray, n_boxes: int, seed: int, scale: float = 0.2) -> int:
    """Boxes on which the program and node-by-node evaluation differ in the
    objective's enclosure or the feasibility verdict (+0 and -0 equal)."""
    op = O.OracleProblem(p)
    assert op.set_program64(code)
    lo, hi = random_boxes(p, n_boxes, np.random.default_rng(seed), scale)
    lb, ub, fe = op.eval_boxes(lo, hi, A.PRECISION_FP64, threads=2)
    bad = 0
    for k in range(n_boxes):
        f, plb, pub = op.program_eval64(np.stack([lo[:, k], hi[:, k]], 1).reshape(-1))
        assert f >= 0, "an operator without an interval form"
        same = f == fe[k] and (plb == lb[k] or (np.isnan(plb) and np.isnan(lb[k]))) and (
            pub == ub[k] or (np.isnan(pub) and np.isnan(ub[k])))
        bad += not same
    return bad


def cases():
    yield "qcqp_n4", G.qcqp_n4()
    yield "miqcqp_n32", G.miqcqp_n32()
    yield "miqcqp_n64", G.miqcqp_n64()
    yield "uneven_qcqp_0", G.uneven_qcqp(0)
    yield "every_operator", ops_problem()
    for name, p in fixture_problems().items():
        yield name, p


@pytest.mark.parametrize("name,p", list(cases()), ids=[n for n, _ in cases()])
def test_program_matches_node_by_node(name, p):
    n_boxes = 200 if p.n_vars > 8 else 1000
    assert mismatches(p, compile_program(p, 0), n_boxes, seed=7, scale=0.5 if name == "every_operator" else 0.2) == 0


@pytest.mark.parametrize("n_vars", [32, 64])
def test_every_constraint_chain_matches_node_by_node(n_vars):
    # each constraint root as the objective: the chain's enclosure itself,
    # not only the verdict it feeds
    p = G.BY_N[n_vars]()
    for c in p.constraints[:8]:
        q = with_objective(p, c.root_id)
        assert mismatches(q, compile_program(q, 0), 64, seed=c.root_id) == 0


def test_every_node_of_the_operator_problem_matches():
    p = ops_problem()
    for node in p.graph.nodes:
        if node.op in (A.OP_CONST, A.OP_VAR):
            continue
        q = with_objective(p, node.id)
        assert mismatches(q, compile_program(q, 0), 200, seed=node.id, scale=0.5) == 0, node.op


def test_a_planted_program_error_is_caught():
    p = G.miqcqp_n32()
    base = compile_program(p, 0)
    rows = base.reshape(-1, 16)
    terms = [i for i in range(len(rows)) if (rows[i, 0] & 7) == OP_TERM and (rows[i, 0] >> 3) & T_HASC]
    assert terms

    def planted(sel, change):
        code = base.copy()
        r = code.reshape(-1, 16)
        for i in sel:
            c = r[i, 8:16].view(np.float64)[0]
            r[i, 8:16] = np.frombuffer(np.float64(change(c)).tobytes(), dtype=np.uint8)
        return code

    assert mismatches(p, planted(terms[:1], lambda c: 2.0 * c), 200, seed=7) > 0
    assert mismatches(p, planted(terms, lambda c: np.nextafter(c, np.inf)), 200, seed=7) > 0
