"""The Python Problem/Expr builder emits the reference's node sequence
(model/problem.hpp:35-164) and applies its validate() rules."""

import pytest

from cuminlp_gb300 import _abi as A
from cuminlp_gb300 import generators as G
from cuminlp_gb300.problem import InvalidDAG, InvalidProblem, Problem, log, pow, sqrt


def ops(p):
    return [A.OP_NAMES[n.op] for n in p.graph.nodes]


def test_same_node_product_is_sqr_and_scalars_become_consts():
    p = Problem()
    x = p.var(-1, 1)
    y = p.var(0, 5)
    e = x * x + 2.0 * y
    p.set_objective(e)
    assert ops(p) == ["Var", "Var", "Sqr", "Const", "Mul", "Add"]
    assert p.graph.nodes[4].inputs == (3, 1)


def test_unary_on_const_folds():
    p = Problem()
    c = p.fixed(4.0)
    assert p.graph.nodes[sqrt(c).id].constant == 2.0
    assert p.graph.nodes[pow(c, 2).id].constant == 16.0
    assert p.graph.nodes[(-c).id].op == A.OP_CONST
    x = p.var(1, 2)
    assert p.graph.nodes[log(x).id].op == A.OP_LOG
    assert p.graph.nodes[pow(x, 3).id].int_exp == 3


def test_op_count_and_validate():
    p = Problem()
    x = p.var(0, 1)
    e = (x + 1.0) * (x - 1.0)
    p.set_objective(e)
    assert p.graph.nodes[e.id].op_count == 7
    p.validate()
    q = Problem()
    q.var(0, 1)
    with pytest.raises(InvalidProblem):
        q.validate()
    r = Problem()
    r.var(0, 1)
    r.set_objective(r.fixed(1.0))
    with pytest.raises(InvalidDAG):
        r.validate()


def test_generators_are_deterministic_and_shaped():
    a, b = G.miqcqp_n32(), G.miqcqp_n32()
    assert [(n.op, n.inputs, n.constant) for n in a.graph.nodes] == [(n.op, n.inputs, n.constant) for n in b.graph.nodes]
    assert a.n_vars == 32 and sum(k == A.VAR_INTEGER for k in a.var_kinds) == 4
    assert len(a.constraints) == 16
    assert a.box_bounds[0] == (0.0, 7.0) and a.box_bounds[10] == (-5.0, 5.0)
    c1 = G.qcqp_n4()
    assert c1.n_vars == 4 and len(c1.constraints) == 1 and c1.constraints[0].rhs == 5.0
    c3 = G.miqcqp_n64()
    assert c3.n_vars == 64 and len(c3.constraints) == 32
    for i in range(5):
        p = G.uneven_qcqp(i)
        assert 4 <= p.n_vars <= 48 and len(p.constraints) <= 24
        p.validate()


def test_normal_draws_have_unit_variance():
    rng = G.SplitMix64(123)
    xs = [rng.normal() for _ in range(20000)]
    m = sum(xs) / len(xs)
    v = sum((x - m) ** 2 for x in xs) / len(xs)
    assert abs(m) < 0.03 and abs(v - 1.0) < 0.05
