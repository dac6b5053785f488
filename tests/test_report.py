"""CPU: the reference's output grammar (PARAMS / finish block / RESULT) and
RunTelemetry's counter identities, on outcomes of the batched algorithm
(the oracle's restatement, which the GPU reproduces bit for bit)."""

from __future__ import annotations

import oracle as O
from cuminlp_gb300 import generators as G
from cuminlp_gb300 import report
from tests.test_oracle_pins import fixture_problems


def outcomes():
    fx = fixture_problems()
    for name in ("square_le5", "infeasible", "aggregate_fixture", "int_eq", "miqcqp_n6"):
        yield name, O.OracleProblem(fx[name]).solve_batched(iter_limit=2000, bisection_budget=3, batch_parents=32,
                                                            frontier_cap=150, threads=2)
    yield "qcqp_n4_1", O.OracleProblem(G.qcqp_n4(1)).solve_batched(iter_limit=20000, bisection_budget=3,
                                                                   batch_parents=256, threads=2)


def test_counters_balance():
    for name, o in outcomes():
        assert report.balances(o), name


def test_result_line_grammar():
    got = dict(outcomes())
    o = got["qcqp_n4_1"]
    assert o["proven_optimal"] == 1
    line = report.result_line(o)
    f = line.split("\t")
    assert f[0] == "RESULT" and f[1] == "sense=min"
    assert float(f[2].split("=")[1]) == o["upper_bound"] and float(f[3].split("=")[1]) == o["lower_bound"]
    mx = report.result_line(o, maximise=True).split("\t")
    assert mx[1] == "sense=max" and float(mx[2].split("=")[1]) == -o["upper_bound"]
    inf = report.result_line(got["infeasible"])
    assert inf.endswith("primal=none\tdual=none") or "primal=none" in inf


def test_finish_block():
    got = dict(outcomes())
    lines = report.finish_block(got["qcqp_n4_1"])
    assert lines[0] == "------------ Finished ------------"
    assert lines[1].endswith("<= min <= %g" % got["qcqp_n4_1"]["upper_bound"])
    assert "Proven optimal: no pending region can beat the incumbent." in lines
    assert "Stop reason: converged" in lines
    infeasible = report.finish_block(got["infeasible"])
    assert infeasible[0].startswith("Search space exhausted")
    assert "Outcome: infeasible" in infeasible and "Stop reason: exhausted" in infeasible
    assert report.params_line(3, 1) == "PARAMS\tpolicy=bisection_budget\tsource=named\tbisection_budget=3\tsample_points=1"
