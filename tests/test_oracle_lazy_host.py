"""CPU: the lazy form as the oracle restates it, on programs the library
compiles on the host (cmn_program_compile), with no GPU.

The GPU tests hold the device's lazy form to this restatement bit for bit;
these tests hold the restatement itself to the properties the form rests
on: the incremental FP32 child bounds enclose the FP64 ones (never above,
never a false infeasibility), and a search to the 1e-6 gap certifies the
plain FP64 form's bounds within the solver's tolerance while it spends
FP64 on fewer boxes (search/driver.hpp:319-350 for the gap test the
tolerance comes from)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import _abi as A
from cuminlp_gb300 import generators as G
from cuminlp_gb300 import report
from cuminlp_gb300._lib import CmnError
from cuminlp_gb300.problem import Problem
from cuminlp_gb300.solver import compile_program
from tests.test_oracle_pins import fixture_problems


def lazy_oracle(p: Problem) -> O.OracleProblem:
    op = O.OracleProblem(p)
    op.set_program32(compile_program(p, 1))  # False when the program is not a set of sum chains
    assert op.set_program64(compile_program(p, 0))
    return op


def test_program_compile_is_deterministic_and_validates():
    p = G.miqcqp_n32()
    a, b = compile_program(p, 0), compile_program(p, 0)
    assert np.array_equal(a, b) and len(a) % 16 == 0 and len(a) > 0
    assert len(compile_program(p, 1)) == len(a)  # one FP32 instruction per FP64 one
    with pytest.raises(CmnError) as e:
        compile_program(p, 2)
    assert e.value.status_name == "INVALID_CONFIGURATION"
    bad = Problem()
    x = bad.var(0.0, 1.0)
    bad.set_objective(x * x)
    bad.objective_root = 99  # no such node
    with pytest.raises(CmnError):
        compile_program(bad, 0)


@pytest.mark.parametrize("n_vars,seed", [(4, 1), (32, 2), (64, 3)])
def test_incremental_fp32_bounds_enclose_fp64(n_vars, seed):
    p = G.BY_N[n_vars]()
    op = O.OracleProblem(p)
    assert op.set_program32(compile_program(p, 1))  # every generated QCQP is a set of sum chains
    rng = np.random.default_rng(seed)
    root = np.array(p.box_bounds)
    ints = np.array(p.var_kinds) != A.VAR_CONTINUOUS
    for _ in range(8):
        c = rng.uniform(root[:, 0], root[:, 1])
        w = (root[:, 1] - root[:, 0]) * rng.uniform(0.01, 0.3)
        lo, hi = np.maximum(c - w, root[:, 0]), np.minimum(c + w, root[:, 1])
        lo[ints], hi[ints] = np.ceil(lo[ints]), np.maximum(np.floor(hi[ints]), np.ceil(lo[ints]))
        box = np.stack([lo, hi], 1).reshape(-1)
        kinds, vids, widths, _ = O.bisection_choose(box, p.var_kinds, 8)
        n = int(np.prod(widths))
        fe32, lb32, _ = op.bound_inc32(box, kinds, vids, widths, n)
        fe64, lb64 = op.bound(box, kinds, vids, widths, n)
        assert np.all(lb32 <= lb64)
        assert not np.any(fe64.astype(bool) & ~fe32.astype(bool))


def test_incremental_fp32_bounds_enclose_fp64_on_random_shapes():
    # the same soundness over random QCQP shapes: sizes, densities, integer
    # shares and constraint counts the three workloads do not cover
    rng = np.random.default_rng(2024)
    checked = 0
    for seed in range(30):
        n = int(rng.integers(2, 21))
        spec = G.QCQPSpec(n=n, m=int(rng.integers(0, 7)), n_int=int(rng.integers(0, n // 2 + 1)), int_lb=-3,
                          int_ub=4, cont_lb=-6.0, cont_ub=6.0, q_density=float(rng.uniform(0.1, 1.0)),
                          a_density=float(rng.uniform(0.1, 1.0)), rhs=(1.0, 10.0))
        p = G.qcqp(spec, G.seed_for(20, seed))
        op = O.OracleProblem(p)
        if not op.set_program32(compile_program(p, 1)):
            continue
        root = np.array(p.box_bounds)
        ints = np.array(p.var_kinds) != A.VAR_CONTINUOUS
        for _ in range(3):
            c = rng.uniform(root[:, 0], root[:, 1])
            w = (root[:, 1] - root[:, 0]) * rng.uniform(0.01, 0.5)
            lo, hi = np.maximum(c - w, root[:, 0]), np.minimum(c + w, root[:, 1])
            lo[ints], hi[ints] = np.ceil(lo[ints]), np.maximum(np.floor(hi[ints]), np.ceil(lo[ints]))
            box = np.stack([lo, hi], 1).reshape(-1)
            kinds, vids, widths, _ = O.bisection_choose(box, p.var_kinds, int(rng.integers(1, 7)))
            k = int(np.prod(widths))
            fe32, lb32, _ = op.bound_inc32(box, kinds, vids, widths, k)
            fe64, lb64 = op.bound(box, kinds, vids, widths, k)
            assert np.all(lb32 <= lb64), seed
            assert not np.any(fe64.astype(bool) & ~fe32.astype(bool)), seed
            checked += 1
    assert checked >= 60


def lazy_cases():
    fx = fixture_problems()
    for name in ("square_le5", "infeasible", "int_eq", "miqcqp_n6"):
        yield name, fx[name]
    for i in (1, 2):
        yield f"qcqp_n4_{i}", G.qcqp_n4(i)


@pytest.mark.parametrize("name,p", list(lazy_cases()), ids=[n for n, _ in lazy_cases()])
def test_lazy_form_certifies_the_plain_bounds(name, p):
    opts = dict(iter_limit=200000, bisection_budget=3, batch_parents=256, threads=4)
    plain = O.OracleProblem(p).solve_batched(precision="fp64", **opts)
    lazy = lazy_oracle(p).solve_batched(precision="lazy", **opts)
    assert plain["stop_reason"] == lazy["stop_reason"] != "iteration-limit", name
    assert plain["proven_optimal"] == lazy["proven_optimal"] and plain["infeasible"] == lazy["infeasible"]
    if plain["stop_reason"] == "converged":
        tol = 1e-6 * max(1.0, abs(plain["upper_bound"]))
        assert abs(plain["upper_bound"] - lazy["upper_bound"]) <= tol
        assert abs(plain["lower_bound"] - lazy["lower_bound"]) <= tol
        assert lazy["lower_bound"] <= lazy["upper_bound"]
    # FP64 only where it decides something: fewer FP64 box evaluations
    assert lazy["counters"]["certified_fp64"] < plain["counters"]["certified_fp64"]
    assert report.balances(lazy)
