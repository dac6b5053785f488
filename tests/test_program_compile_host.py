"""CPU: the compiled programs keep every node's roundings in their order.

The library compiles a problem's DAG into a straight-line program (sum
chains folded into TERM instructions, shared intermediates in liveness-
allocated slots): an FP64 one, which the plain form evaluates, and an FP32
one with outward-rounded constant pairs, which the FP32 screen evaluates.
Here both come from cmn_program_compile (no GPU) and run through the
oracle's restatement of the interpreter with every operation rounded on its
own; their enclosures and verdicts must equal the oracle's node-by-node
evaluation of the DAG in the same precision -- the reference's per-node
kernel chain (backend/graph/kernels.cuh:177-419) -- bit for bit.  A mistake
planted in the program is caught the same way."""

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


def mismatches(p: Problem, code: np.ndarray, n_boxes: int, seed: int, scale: float = 0.2, fp32: bool = False) -> int:
    """Boxes on which the program and node-by-node evaluation differ in the
    objective's enclosure or the verdict (+0 and -0 equal): FP64, the
    reference predicate; FP32, not proven violated."""
    op = O.OracleProblem(p)
    if fp32:
        op.set_program32(code)  # False only says the program is not a set of sum chains
    else:
        assert op.set_program64(code)
    run = op.program_eval32 if fp32 else op.program_eval64
    lo, hi = random_boxes(p, n_boxes, np.random.default_rng(seed), scale)
    lb, ub, fe = op.eval_boxes(lo, hi, A.PRECISION_FP32_SCREEN if fp32 else A.PRECISION_FP64, threads=2)
    bad = 0
    for k in range(n_boxes):
        f, plb, pub = run(np.stack([lo[:, k], hi[:, k]], 1).reshape(-1))
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


@pytest.mark.parametrize("fp32", [False, True], ids=["fp64", "fp32"])
@pytest.mark.parametrize("name,p", list(cases()), ids=[n for n, _ in cases()])
def test_program_matches_node_by_node(name, p, fp32):
    n_boxes = 200 if p.n_vars > 8 else 1000
    scale = 0.5 if name == "every_operator" else 0.2
    assert mismatches(p, compile_program(p, int(fp32)), n_boxes, seed=7, scale=scale, fp32=fp32) == 0


@pytest.mark.parametrize("fp32", [False, True], ids=["fp64", "fp32"])
@pytest.mark.parametrize("n_vars", [32, 64])
def test_every_constraint_chain_matches_node_by_node(n_vars, fp32):
    # each constraint root as the objective: the chain's enclosure itself,
    # not only the verdict it feeds
    p = G.BY_N[n_vars]()
    for c in p.constraints[:8]:
        q = with_objective(p, c.root_id)
        assert mismatches(q, compile_program(q, int(fp32)), 64, seed=c.root_id, fp32=fp32) == 0


@pytest.mark.parametrize("fp32", [False, True], ids=["fp64", "fp32"])
def test_every_node_of_the_operator_problem_matches(fp32):
    p = ops_problem()
    for node in p.graph.nodes:
        if node.op in (A.OP_CONST, A.OP_VAR):
            continue
        q = with_objective(p, node.id)
        assert mismatches(q, compile_program(q, int(fp32)), 200, seed=node.id, scale=0.5, fp32=fp32) == 0, node.op


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


def test_a_planted_fp32_program_error_is_caught():
    p = G.miqcqp_n32()
    code = compile_program(p, 1)
    r = code.reshape(-1, 16)
    first = next(i for i in range(len(r)) if (r[i, 0] & 7) == OP_TERM and (r[i, 0] >> 3) & T_HASC)
    r[first, 8:16] = np.frombuffer((2.0 * r[first, 8:16].view(np.float32)).astype(np.float32).tobytes(), np.uint8)
    assert mismatches(p, code, 200, seed=7, fp32=True) > 0


def random_problem(seed: int) -> Problem:
    """A random DAG over a few variables: every operator with an interval
    form, shared subexpressions (each new node may reuse any earlier one),
    sum chains of coefficient products, and LE / EQ constraints on random
    nodes -- the shapes that exercise the compiler's slot liveness and
    chain folding beyond the generated QCQPs."""
    from cuminlp_gb300.problem import Expr, pow, sqr, sqrt
    rng = np.random.default_rng(seed)
    p = Problem()
    pool = []
    for _ in range(int(rng.integers(2, 7))):
        if rng.random() < 0.2:
            pool.append(p.int_var(-2.0, 3.0))
        else:
            lo = float(rng.uniform(-5.0, 1.0))
            pool.append(p.var(lo, lo + float(rng.uniform(0.5, 6.0))))
    n_vars = len(pool)
    g = p.graph
    for _ in range(int(rng.integers(10, 60))):
        a, b = pool[int(rng.integers(len(pool)))], pool[int(rng.integers(len(pool)))]
        c = float(np.round(rng.normal() * 3.0, 3)) or 1.5
        kind = int(rng.integers(0, 14))
        e = (a + b if kind == 0 else a - b if kind == 1 else a * b if kind == 2 else a / b if kind == 3
             else sqr(a) if kind == 4 else -a if kind == 5 else sqrt(a) if kind == 6
             else pow(a, int(rng.integers(-3, 5))) if kind == 7
             else Expr(g, g.emit(A.OP_ABS, (a.id,))) if kind == 8
             else Expr(g, g.emit(A.OP_MIN, (a.id, b.id))) if kind == 9
             else Expr(g, g.emit(A.OP_MAX, (a.id, b.id))) if kind == 10
             else c * a if kind == 11 else a + c if kind == 12 else None)
        if e is None:  # a sum chain over the variables, from an earlier node
            e = pool[int(rng.integers(len(pool)))]
            for _ in range(int(rng.integers(1, 5))):
                xi, xj = pool[int(rng.integers(n_vars))], pool[int(rng.integers(n_vars))]
                e = e + float(np.round(rng.normal() * 3.0, 3) or 0.5) * (xi * xj)
        pool.append(e)
    p.set_objective(pool[-1])
    for _ in range(int(rng.integers(0, 4))):
        root = pool[int(rng.integers(n_vars, len(pool)))]
        p.add_constraint(root, A.CMP_LE if rng.random() < 0.7 else A.CMP_EQ, float(rng.normal() * 5.0))
    return p


@pytest.mark.parametrize("fp32", [False, True], ids=["fp64", "fp32"])
def test_random_dags_match_node_by_node(fp32):
    for seed in range(60):
        p = random_problem(seed)
        assert mismatches(p, compile_program(p, int(fp32)), 100, seed=seed, scale=0.4, fp32=fp32) == 0, seed
