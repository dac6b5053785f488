"""Region roles through the C ABI (the reference's plugin boundary,
backend/backend.hpp:81-219) against the oracle and the reference's own
known answers (graph_replay_test.cu, backend_contract.hpp)."""

from __future__ import annotations

import functools
import math

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import _abi as A
from cuminlp_gb300 import generators as G
from cuminlp_gb300._lib import CmnError
from cuminlp_gb300.problem import Problem
from cuminlp_gb300.solver import Bounder, DeviceProblem, Enumerator, OverBudgetError, Sampler
from tests.conftest import bits_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cuminlp_gb300 import build
    build.build_library()


def square_problem(rhs=5.0):
    p = Problem()
    x = p.var(0.0, 10.0)
    p.set_objective(x * x)
    p.add_constraint(x, A.CMP_LE, rhs)
    return p


def test_bound_known_answer():
    # graph_replay_test.cu:77-84 at fan-out 4
    p = square_problem()
    b = Bounder(DeviceProblem(p), [A.SLOT_CONTINUOUS], 4)
    fe, lb = b.bound(p.root_box(), [0], [4])
    assert lb.tolist() == [0.0, 6.25, 25.0, 56.25]
    assert fe.tolist() == [1, 1, 1, 0]


def test_sampler_candidates_and_nan_witness():
    # graph_replay_test.cu:221-264
    dp = DeviceProblem(square_problem())
    s = Sampler(dp, [A.SLOT_CONTINUOUS], 4, sample_points=16)
    c = s.sample([0.0, 5.0], [0], [4], salt=1)
    assert c.found and not math.isnan(c.point[0]) and c.value < np.finfo(np.float64).max
    dpi = DeviceProblem(square_problem(-100.0))
    si = Sampler(dpi, [A.SLOT_CONTINUOUS], 4, sample_points=16)
    c = si.sample([0.0, 10.0], [0], [4], salt=1)
    assert not c.found and math.isnan(c.point[0])


def test_sampler_determinism_and_salt():
    # graph_replay_test.cu:266-356
    dp = DeviceProblem(square_problem())
    s = Sampler(dp, [A.SLOT_CONTINUOUS], 4, sample_points=32)
    a = s.sample([0.0, 5.0], [0], [4], salt=7)
    b = s.sample([0.0, 5.0], [0], [4], salt=7)
    c = s.sample([0.0, 5.0], [0], [4], salt=8)
    assert a.value == b.value and np.array_equal(a.point, b.point)
    assert a.value != c.value
    bd = Bounder(dp, [A.SLOT_CONTINUOUS], 4)
    l1 = bd.bound([0.0, 10.0], [0], [4])[1].copy()
    l2 = bd.bound([0.0, 10.0], [0], [4])[1].copy()
    assert np.array_equal(l1, l2)


@pytest.mark.parametrize("n_vars,B", [(4, 8), (32, 10), (64, 6)])
def test_roles_match_oracle(n_vars, B):
    p = G.BY_N[n_vars]()
    dp = DeviceProblem(p)
    op = O.OracleProblem(p)
    box = p.root_box()
    kinds, vids, widths, dom = O.bisection_choose(box, p.var_kinds, B)
    N = int(np.prod(widths))
    fe, lb = Bounder(dp, kinds, N).bound(box, vids, widths)
    ofe, olb = op.bound(box, kinds, vids, widths, N)
    assert bits_equal(lb, olb) and np.array_equal(fe, ofe)
    for S, salt in ((1, 3), (4, 12345)):
        c = Sampler(dp, kinds, N, sample_points=S).sample(box, vids, widths, salt)
        found, val, pt, idx = op.sample(box, kinds, vids, widths, N, S, salt)
        assert c.found == found
        if found:
            assert c.value == val and c.index == idx and np.array_equal(c.point, pt)


def test_contract_model_roles():
    # backend_contract.hpp:103-288 with backend_contract_test.cu:32-104
    from tests.test_oracle_pins import contract_model
    p = contract_model()
    dp = DeviceProblem(p)
    op = O.OracleProblem(p)
    box = p.root_box()
    ek = [A.SLOT_BINARY_ENUMERATE] * 2 + [A.SLOT_INTEGER_ENUMERATE] * 2
    en = Enumerator(dp, ek, 64)
    c = en.enumerate(box, [0, 1, 2, 3], [2, 2, 4, 4])
    found, val, pt, idx = op.enumerate(box, ek, [0, 1, 2, 3], [2, 2, 4, 4], 64)
    assert c.found and found and c.value == val and np.array_equal(c.point, pt) and c.index == idx
    assert c.value == sum((x - 1.0) ** 2 for x in c.point) and c.point[0] + c.point[1] <= 1.0
    fe, lb = Bounder(dp, ek, 64).bound(box, [0, 1, 2, 3], [2, 2, 4, 4])
    assert lb[fe == 1].min() <= c.value + 1e-9
    s = Sampler(dp, [A.SLOT_CONTINUOUS] * 2, 4, sample_points=4)
    d = s.sample(box, [4, 5], [2, 2], 7)
    assert d.found and abs(d.value - sum((x - 1.0) ** 2 for x in d.point)) < 1e-12
    assert all(x == round(x) for x in d.point[:4])
    cm = dp.cost_model()
    assert cm["bound_bytes_per_region"] > 0


def test_over_budget_and_shape_errors():
    p = square_problem()
    dp = DeviceProblem(p)
    with pytest.raises(OverBudgetError) as ei:
        Bounder(dp, [A.SLOT_CONTINUOUS], 4, budget_bytes=1)
    f = ei.value.facts
    assert f["budget_bytes"] == 1 and f["needed_bytes"] > 1 and f["n_regions"] == 4
    b = Bounder(dp, [A.SLOT_CONTINUOUS], 4)
    with pytest.raises(CmnError) as e2:
        b.bound(p.root_box(), [0], [3])
    assert e2.value.status_name == "SHAPE_MISMATCH"
    with pytest.raises(CmnError) as e3:
        Enumerator(dp, [A.SLOT_CONTINUOUS], 4)
    assert e3.value.status_name == "INVALID_CONFIGURATION"
    with pytest.raises(CmnError):
        Sampler(dp, [A.SLOT_CONTINUOUS], 4, sample_points=0)


@functools.lru_cache(maxsize=1)
def wide_qcqp():
    """n = 512: sparse Q and constraints, so the DAG stays small while the
    sampler's point (512 doubles) far exceeds one thread's share of shared
    memory; lanes share point columns (sample_lg_min)."""
    return G.qcqp(G.QCQPSpec(n=512, m=4, n_int=32, int_lb=0, int_ub=3, cont_lb=-1.0, cont_ub=1.0,
                             q_density=0.002, a_density=0.002, rhs=(1.0, 10.0)), G.seed_for(11, 0))


def test_sampler_n512_matches_oracle():
    p = wide_qcqp()
    assert p.n_vars == 512
    dp = DeviceProblem(p)
    op = O.OracleProblem(p)
    box = p.root_box()
    kinds, vids, widths, _ = O.bisection_choose(box, p.var_kinds, 10)
    N = int(np.prod(widths))
    s = Sampler(dp, kinds, N, sample_points=2)
    found_any = False
    for salt in (1, 2, 3):
        c = s.sample(box, vids, widths, salt)
        found, val, pt, idx = op.sample(box, kinds, vids, widths, N, 2, salt)
        assert c.found == found
        if found:
            found_any = True
            assert c.value == val and c.index == idx
            assert np.array_equal(c.point, pt)
    assert found_any
