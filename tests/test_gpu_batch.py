"""The multi-instance batch against the oracle's batched restatement, run
per instance: identical frontiers, bounds, incumbents and counters for every
instance of a mixed batch of uneven sizes; each result the same alone and in
the mix; slot refill; the FP32 screen reproducing the FP64 search."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import generators as G
from cuminlp_gb300._lib import CmnError
from cuminlp_gb300.solver import Batch, DeviceProblem, Solver, batch_solve
from tests.conftest import bits_equal
from tests.test_oracle_pins import contract_model, fixture_problems

pytestmark = pytest.mark.gpu

COUNTERS = ["iterations", "expansions", "fathomed", "fathomed_points", "bounded", "sampled", "enqueued",
            "witness_rejected", "pruned_duplicate", "pruned_infeasible", "pruned_dominated", "dropped_viable",
            "dropped_dominated", "screened_fp32", "certified_fp64", "peak_frontier", "certify_pruned"]
FIELDS = ("lower_bound", "upper_bound", "stop_reason", "proven_optimal", "infeasible", "found_incumbent",
          "frontier_size", "viable", "dropped_lb_min")


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cuminlp_gb300 import build
    build.build_library()


def mixed_problems():
    fx = fixture_problems()
    ps = {
        "square_le5": fx["square_le5"], "infeasible": fx["infeasible"], "aggregate": fx["aggregate_fixture"],
        "contract": contract_model(), "int_eq": fx["int_eq"], "miqcqp_n6": fx["miqcqp_n6"],
        "qcqp_n4": G.qcqp_n4(), "qcqp_n4_1": G.qcqp_n4(1),
    }
    for i in range(6):
        ps[f"uneven_{i}"] = G.uneven_qcqp(i)
    return ps


def same_outcome(a: dict, b: dict, name: str = ""):
    for k in FIELDS:
        if isinstance(a[k], float):
            assert bits_equal(np.float64(a[k]), np.float64(b[k])), (name, k, a[k], b[k])
        else:
            assert a[k] == b[k], (name, k, a[k], b[k])
    for k in COUNTERS:
        assert a["counters"][k] == b["counters"][k], (name, k, a["counters"][k], b["counters"][k])
    if a["found_incumbent"]:
        assert bits_equal(a["best_point"], b["best_point"]), name


def same_frontier(fa, fb, name=""):
    assert len(fa[1]) == len(fb[1]), name
    assert bits_equal(fa[1], fb[1]), name
    assert np.array_equal(fa[2], fb[2]), name
    assert bits_equal(fa[0], fb[0]), name


SHARED = dict(bisection_budget=4, batch_parents=16, frontier_cap=256, sample_points=2)


def run_batch(named, shared, per_instance):
    n_max = max(p.n_vars for p in named.values())
    dps = {k: DeviceProblem(p) for k, p in named.items()}
    b = Batch(len(named), n_max, max(dp.info()["program_slots"] for dp in dps.values()), **shared)
    slots = {k: b.add(dp, **per_instance) for k, dp in dps.items()}
    assert b.step(0) == 0
    out = {}
    for k, s in slots.items():
        assert b.done(s)
        out[k] = (b.outcome(s), b.frontier(s))
    b.close()
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_matches_oracle_per_instance(precision):
    named = mixed_problems()
    shared = dict(SHARED, precision=precision)
    got = run_batch(named, shared, dict(batch_iter_limit=20))
    for k, p in named.items():
        obox, olb, odepth, o = O.OracleProblem(p).batched_frontier(0, room=1 << 16, batch_iter_limit=20, **shared)
        g, fg = got[k]
        same_frontier(fg, (obox, olb, odepth), k)
        same_outcome(g, o, k)


def lazy_oracle(p, dp):
    # the lazy form bounds children from the compiled FP32 program's sum
    # chains and certifies each expanded box with the FP64 program's fused
    # terms; the oracle restates both from the same programs
    op = O.OracleProblem(p)
    op.set_program32(dp.program(1))
    op.set_program64(dp.program(0))
    return op


def test_batch_lazy_matches_oracle_per_instance():
    named = mixed_problems()
    shared = dict(SHARED, precision="lazy")
    got = run_batch(named, shared, dict(batch_iter_limit=20))
    for k, p in named.items():
        op = lazy_oracle(p, DeviceProblem(p))
        obox, olb, odepth, o = op.batched_frontier(0, room=1 << 16, batch_iter_limit=20, **shared)
        g, fg = got[k]
        same_frontier(fg, (obox, olb, odepth), k)
        same_outcome(g, o, k)


def test_batch_lazy_matches_single_instance_solver():
    named = mixed_problems()
    keep = {k: named[k] for k in ("aggregate", "contract", "miqcqp_n6", "qcqp_n4_1", "uneven_0", "uneven_3")}
    shared = dict(SHARED, precision="lazy", sample_all=1)
    got = run_batch(keep, shared, dict(batch_iter_limit=30))
    for k, p in keep.items():
        s = Solver(DeviceProblem(p), batch_iter_limit=30, **shared)
        s.step(0)
        same_outcome(s.outcome(), got[k][0], k)
        same_frontier(s.frontier(), got[k][1], k)
        s.close()


def test_batch_alone_equals_mixed():
    named = mixed_problems()
    per = dict(batch_iter_limit=25)
    mixed = run_batch(named, SHARED, per)
    for k, p in named.items():
        alone = run_batch({k: p}, SHARED, per)[k]
        same_outcome(alone[0], mixed[k][0], k)
        same_frontier(alone[1], mixed[k][1], k)


def test_batch_matches_single_instance_solver():
    named = mixed_problems()
    keep = {k: named[k] for k in ("aggregate", "miqcqp_n6", "qcqp_n4_1", "uneven_0", "uneven_3")}
    got = run_batch(keep, SHARED, dict(batch_iter_limit=30))
    for k, p in keep.items():
        s = Solver(DeviceProblem(p), batch_iter_limit=30, **SHARED)
        s.step(0)
        same_outcome(s.outcome(), got[k][0], k)
        same_frontier(s.frontier(), got[k][1], k)
        s.close()


def test_batch_fp32_screen_identical_to_fp64():
    named = mixed_problems()
    a = run_batch(named, dict(SHARED, precision="fp64"), dict(batch_iter_limit=30))
    b = run_batch(named, dict(SHARED, precision="fp32"), dict(batch_iter_limit=30))
    screened = 0
    for k in named:
        ga, gb = a[k][0], b[k][0]
        for f in ("lower_bound", "upper_bound", "stop_reason", "frontier_size", "viable"):
            assert ga[f] == gb[f], (k, f)
        same_frontier(a[k][1], b[k][1], k)
        if ga["found_incumbent"]:
            assert np.array_equal(ga["best_point"], gb["best_point"]), k
        assert gb["counters"]["certified_fp64"] <= ga["counters"]["certified_fp64"]
        screened += ga["counters"]["certified_fp64"] - gb["counters"]["certified_fp64"]
    assert screened > 0


def test_batch_solve_refills_slots():
    named = mixed_problems()
    keys = list(named)
    iter_limits = [200 + 37 * i for i in range(len(keys))]
    per = [dict(iter_limit=il) for il in iter_limits]
    res = batch_solve([named[k] for k in keys], slots=3, per_instance=per, **SHARED)
    for k, il, r in zip(keys, iter_limits, res):
        o = O.OracleProblem(named[k]).solve_batched(iter_limit=il, **SHARED)
        same_outcome(r, o, k)


def test_batch_runs_to_convergence_like_the_oracle():
    named = {k: v for k, v in mixed_problems().items() if k in ("square_le5", "qcqp_n4", "qcqp_n4_1", "int_eq")}
    res = batch_solve(list(named.values()), iter_limit=100000, **SHARED)
    for (k, p), r in zip(named.items(), res):
        o = O.OracleProblem(p).solve_batched(iter_limit=100000, **SHARED)
        same_outcome(r, o, k)


def test_batch_slot_errors():
    p = DeviceProblem(G.qcqp_n4())
    b = Batch(2, 4, **SHARED)
    b.add(p)
    b.add(p)
    with pytest.raises(CmnError) as e:
        b.add(p)
    assert e.value.status_name == "OVER_BUDGET"
    big = DeviceProblem(G.miqcqp_n32())
    b.release(0)
    with pytest.raises(CmnError) as e:
        b.add(big)
    assert e.value.status_name == "INVALID_CONFIGURATION"
    b.close()
    with pytest.raises(CmnError):
        Batch(1, 4, bisection_budget=4, batch_parents=512, frontier_cap=1024)
