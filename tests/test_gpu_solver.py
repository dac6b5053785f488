"""The device-resident batched solver against its CPU restatement in the
oracle: identical frontiers (boxes, bounds, depths) after fixed numbers of
iterations, identical incumbents, bounds and counters; and the FP32 screen
with FP64 certification reproducing the plain FP64 search exactly."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import _abi as A
from cuminlp_gb300 import generators as G
from cuminlp_gb300 import report
from cuminlp_gb300.solver import DeviceProblem, Solver
from tests.conftest import bits_equal
from tests.test_oracle_pins import contract_model, fixture_problems

pytestmark = pytest.mark.gpu

COUNTERS = ["iterations", "expansions", "fathomed", "fathomed_points", "bounded", "sampled", "enqueued",
            "witness_rejected", "pruned_duplicate", "pruned_infeasible", "pruned_dominated", "dropped_viable",
            "dropped_dominated", "screened_fp32", "certified_fp64", "peak_frontier", "certify_pruned"]


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cuminlp_gb300 import build
    build.build_library()


def problems():
    fx = fixture_problems()
    return {
        "square_le5": fx["square_le5"], "infeasible": fx["infeasible"], "aggregate": fx["aggregate_fixture"],
        "contract": contract_model(), "int_eq": fx["int_eq"], "miqcqp_n6": fx["miqcqp_n6"],
        "qcqp_n4": G.qcqp_n4(), "qcqp_n4_1": G.qcqp_n4(1),
    }


def compare(p, iterations, room=1 << 20, **opts):
    dp = DeviceProblem(p)
    s = Solver(dp, batch_iter_limit=iterations, **opts)
    s.step(0)
    g = s.outcome()
    gbox, glb, gdepth = s.frontier()
    op = O.OracleProblem(p)
    if opts.get("precision") == "lazy":
        # the lazy form bounds children incrementally over the compiled
        # program when it is a set of sum chains, and certifies each expanded
        # box with the FP64 program's fused terms; the oracle restates both
        # from the same programs
        op.set_program32(dp.program(1))
        op.set_program64(dp.program(0))
    obox, olb, odepth, o = op.batched_frontier(iterations, room=room, **opts)
    assert len(glb) == len(olb)
    assert bits_equal(glb, olb)
    assert np.array_equal(gdepth, odepth)
    assert bits_equal(gbox, obox)
    for k in ("lower_bound", "upper_bound", "stop_reason", "proven_optimal", "infeasible", "frontier_size",
              "viable"):
        if isinstance(g[k], float):
            assert bits_equal(np.float64(g[k]), np.float64(o[k])), k
        else:
            assert g[k] == o[k], k
    for k in COUNTERS:
        assert g["counters"][k] == o["counters"][k], k
    if o["upper_bound"] < np.finfo(np.float64).max:
        assert bits_equal(g["best_point"], o["best_point"])
    assert report.balances(g)  # RunTelemetry::balances on the device's counters
    s.close()
    return g


@pytest.mark.parametrize("name", ["square_le5", "infeasible", "aggregate", "contract", "int_eq", "miqcqp_n6",
                                  "qcqp_n4"])
def test_solver_matches_oracle(name):
    p = problems()[name]
    compare(p, 12, bisection_budget=2, batch_parents=64, sample_points=2)
    compare(p, 5, bisection_budget=3, batch_parents=1, sample_points=1, sample_all=1)


@pytest.mark.parametrize("precision", ["fp64", "fp32", "lazy"])
def test_solver_matches_oracle_larger(precision):
    compare(G.qcqp_n4(), 30, bisection_budget=3, batch_parents=512, precision=precision)
    compare(G.qcqp_n4(2), 20, bisection_budget=4, batch_parents=256, precision=precision, relative_width=1)


def test_eviction_matches_oracle():
    g = compare(G.qcqp_n4(1), 25, bisection_budget=3, batch_parents=128, frontier_cap=300)
    assert g["counters"]["dropped_viable"] + g["counters"]["dropped_dominated"] > 0


def tied_model():
    # the objective depends on x0 alone, so every child split on x1..x3 has
    # its parent's lower bound: long runs of equal keys, and the selects of
    # both the cap and the next parents end inside a bucket of ties that
    # only pool position orders
    from cuminlp_gb300.problem import Problem
    p = Problem()
    v = [p.var(-1.0, 1.0) for _ in range(4)]
    p.set_objective(v[0] * v[0] - v[0])
    p.add_constraint(v[1] * v[2] + v[3], A.CMP_LE, 1.5)
    return p


@pytest.mark.parametrize("instance", [6, 13, 0])  # n = 11, 36, 44: the three branching scratch kinds
def test_solver_matches_oracle_wider(instance):
    # the branching policy keeps its scratch in local memory up to 32
    # variables and in global scratch above; both against the oracle, with
    # a cap small enough to evict
    compare(G.uneven_qcqp(instance), 6, bisection_budget=3, batch_parents=48, frontier_cap=400,
            sample_points=1)


@pytest.mark.parametrize("cap", [97, 1000])
def test_tied_lower_bounds_rank_by_position(cap):
    g = compare(tied_model(), 14, bisection_budget=2, batch_parents=40, frontier_cap=cap, sample_points=1)
    if cap == 97:
        assert g["counters"]["dropped_viable"] + g["counters"]["dropped_dominated"] > 0


def test_fp32_screen_identical_certified_bounds():
    p = G.qcqp_n4()
    dp = DeviceProblem(p)
    out = {}
    for prec in ("fp64", "fp32"):
        s = Solver(dp, batch_iter_limit=60, bisection_budget=3, batch_parents=1024, precision=prec)
        s.step(0)
        out[prec] = (s.outcome(), s.frontier())
        s.close()
    a, fa = out["fp64"]
    b, fb = out["fp32"]
    assert a["lower_bound"] == b["lower_bound"] and a["upper_bound"] == b["upper_bound"]
    assert np.array_equal(a["best_point"], b["best_point"])
    assert bits_equal(fa[1], fb[1]) and bits_equal(fa[0], fb[0])
    assert b["counters"]["certified_fp64"] < a["counters"]["certified_fp64"]


def test_one_parent_per_iteration_reproduces_reference_driver():
    # with one parent per iteration and every child sampled, the device
    # search expands boxes in the reference SearchDriver's order: its bounds
    # after a fixed expansion budget equal the driver restatement's (which
    # the golden fixtures pin to the reference's own code)
    for name, iters in (("aggregate", 4000), ("miqcqp_n6", 1500), ("qcqp_n4", 1500)):
        p = problems()[name]
        s = Solver(DeviceProblem(p), bisection_budget=2, batch_parents=1, sample_all=1, iter_limit=iters)
        s.step(0)
        g = s.outcome()
        s.close()
        ref = O.OracleProblem(p).solve_reference(iter_limit=iters, bisection_budget=2, sample_points=1, threads=1)
        assert g["lower_bound"] == ref["lower_bound"] and g["upper_bound"] == ref["upper_bound"], name
        assert g["frontier_size"] == ref["frontier_size"] and g["viable"] == ref["viable"], name


def test_batched_solver_certifies_the_reference_optimum():
    # instance 1 of the n=4 QCQP: the reference driver proves optimality (golden
    # fixture); the batched search must certify the same optimum within the
    # solver's gap
    p = G.qcqp_n4(1)
    ref = O.OracleProblem(p).solve_reference(iter_limit=20000, bisection_budget=3, sample_points=2, threads=1)
    assert ref["proven_optimal"] == 1
    for prec in ("fp64", "fp32"):
        s = Solver(DeviceProblem(p), bisection_budget=3, batch_parents=256, sample_points=2, precision=prec)
        s.step(0)
        g = s.outcome()
        s.close()
        assert g["stop_reason"] == "converged" and g["proven_optimal"] == 1
        tol = 1e-6 * max(1.0, abs(ref["upper_bound"]))
        assert abs(g["upper_bound"] - ref["upper_bound"]) <= tol
        assert abs(g["lower_bound"] - ref["lower_bound"]) <= tol


# The shapes bench.py times: 2^16 parents x 2^4 children per iteration
# (BisectionBudget B = 4), one sample per child.  From the root the pool
# grows 1 -> 16 -> 256 -> 4096 -> 65536 boxes, so iteration 5 is the first
# to expand a full batch of 2^16 parents (2^20 children); the oracle needs
# about a minute per such iteration for n = 32 on 16 host cores, and four
# times that for n = 64, so the n = 64 case stops after iteration 4 (4096
# parents, 65536 children) with the same options, buffers and launch shapes.
# (Measured on the GB300 host: the n = 32 case takes 14 s and the n = 64
# case at 4 iterations 4 s, so both run to iteration 5.)
@pytest.mark.parametrize("precision", ["fp64", "fp32", "lazy"])
def test_solver_matches_oracle_miqcqp_n32_bench_shape(precision):
    g = compare(G.miqcqp_n32(), 5, room=1 << 21, bisection_budget=4, batch_parents=1 << 16, frontier_cap=1 << 20,
                sample_points=1, precision=precision)
    assert g["counters"]["expansions"] > (1 << 12)


@pytest.mark.parametrize("precision", ["fp64", "fp32", "lazy"])
def test_solver_matches_oracle_miqcqp_n64_bench_shape(precision):
    compare(G.miqcqp_n64(), 5, room=1 << 21, bisection_budget=4, batch_parents=1 << 16, frontier_cap=1 << 22,
            sample_points=1, precision=precision)


def test_lazy_form_matches_oracle_small_problems():
    # the lazy form (FP32 children, FP64 verdict of each parent on
    # selection) on the fixture problems, with pruning at certification
    for name in ("square_le5", "infeasible", "aggregate", "contract", "int_eq", "miqcqp_n6"):
        compare(problems()[name], 12, bisection_budget=2, batch_parents=64, sample_points=2, precision="lazy")
        # every valid child sampled, whatever its bound
        compare(problems()[name], 8, bisection_budget=3, batch_parents=16, sample_points=1, sample_all=1,
                precision="lazy")


@pytest.mark.parametrize("instance", [0, 1, 2])
def test_lazy_form_certifies_the_plain_bounds(instance):
    # to the 1e-6 gap: the lazy form's certified bounds agree with the plain
    # FP64 form's within the solver's tolerance, and it spends FP64 on the
    # expanded boxes only
    p = G.qcqp_n4(instance)
    out = {}
    for prec in ("fp64", "lazy"):
        s = Solver(DeviceProblem(p), bisection_budget=2, batch_parents=1 << 21, frontier_cap=1 << 25,
                   sample_points=1, precision=prec, iter_limit=1 << 62)
        s.step(0)
        out[prec] = s.outcome()
        s.close()
    a, b = out["fp64"], out["lazy"]
    assert a["stop_reason"] == "converged" and b["stop_reason"] == "converged", (a, b)
    assert a["proven_optimal"] and b["proven_optimal"], (a, b)
    tol = 1e-6 * max(1.0, abs(a["upper_bound"]))
    assert abs(a["upper_bound"] - b["upper_bound"]) <= tol
    assert abs(a["lower_bound"] - b["lower_bound"]) <= tol
    assert b["lower_bound"] <= b["upper_bound"]
    c = b["counters"]
    assert c["certified_fp64"] < b["counters"]["bounded"] and c["screened_fp32"] > 0
    assert report.balances(b)


@pytest.mark.parametrize("precision", ["fp64", "lazy"])
def test_solver_n512_matches_oracle(precision):
    # the sampler's points shared by lane groups at n = 512, in the search
    from tests.test_gpu_roles import wide_qcqp
    compare(wide_qcqp(), 4, bisection_budget=3, batch_parents=64, sample_points=1, precision=precision)


@pytest.mark.parametrize("n_vars,seed", [(4, 1), (32, 2), (64, 3)])
def test_incremental_fp32_bounds_enclose_fp64(n_vars, seed):
    # the lazy form's incremental FP32 child bounds (common chain sums per
    # parent, split-variable terms per child) are sound: never above the
    # FP64 bound, and a constraint they prove violated is violated in FP64
    p = G.BY_N[n_vars]()
    dp = DeviceProblem(p)
    op = O.OracleProblem(p)
    assert op.set_program32(dp.program(1))
    rng = np.random.default_rng(seed)
    root = np.array(p.box_bounds)
    for _ in range(4):
        c = rng.uniform(root[:, 0], root[:, 1])
        w = (root[:, 1] - root[:, 0]) * rng.uniform(0.01, 0.3)
        lo, hi = np.maximum(c - w, root[:, 0]), np.minimum(c + w, root[:, 1])
        ints = np.array(p.var_kinds) != A.VAR_CONTINUOUS
        lo[ints], hi[ints] = np.ceil(lo[ints]), np.maximum(np.floor(hi[ints]), np.ceil(lo[ints]))
        box = np.stack([lo, hi], 1).reshape(-1)
        kinds, vids, widths, _ = O.bisection_choose(box, p.var_kinds, 6)
        n = int(np.prod(widths))
        fe32, lb32, ub32 = op.bound_inc32(box, kinds, vids, widths, n)
        fe64, lb64 = op.bound(box, kinds, vids, widths, n)
        assert np.all(lb32 <= lb64)
        assert not np.any(fe64.astype(bool) & ~fe32.astype(bool))


@pytest.mark.parametrize("precision", ["fp64", "lazy"])
def test_autotuned_launch_shape_changes_no_result(precision):
    # cmn_autotune times launch shapes (blocks per SM, lanes per box); a
    # solver on the tuned shape must give the untuned solver's search bit
    # for bit
    p = G.qcqp_n4(2)
    dp = DeviceProblem(p)
    t = dp.autotune(0 if precision == "fp64" else 1, 1 << 14)
    assert t["candidates"] >= 1 and t["blocks_per_sm"] >= 1 and t["lanes_cap"] >= 1
    assert t["ms_best"] <= t["ms_default"] * 1.05
    out = []
    for tune in (0, 1):
        s = Solver(dp, batch_iter_limit=20, bisection_budget=3, batch_parents=256, precision=precision,
                   autotune=tune)
        s.step(0)
        out.append((s.outcome(), s.frontier()))
        s.close()
    (a, fa), (b, fb) = out
    assert a["lower_bound"] == b["lower_bound"] and a["upper_bound"] == b["upper_bound"]
    assert a["counters"] == b["counters"]
    assert bits_equal(fa[1], fb[1]) and bits_equal(fa[0], fb[0])
