"""CPU: the host aggregate driver (cuminlp_gb300.aggregate) against the
reference's own AggregateDriver (golden fixtures from oracle/_ref, with the
oracle behind both drivers' roles): the same bounds, stop reason, claims,
counters and best point, for each selection rule."""

from __future__ import annotations

import json
from pathlib import Path

from cuminlp_gb300.aggregate import AggregateDriver, WidestBranchPolicy
from tests.aggregate_roles import OracleAggregateRoles
from tests.test_oracle_pins import fixture_problems

GOLDEN = Path(__file__).resolve().parent / "golden"
COUNTERS = ("iterations", "fathomed", "fathomed_points", "bounded", "sampled", "enqueued", "witness_rejected",
            "pruned_duplicate", "pruned_infeasible", "pruned_dominated", "pending", "viable", "history_freed",
            "history_peak_live")


def test_aggregate_driver_matches_reference():
    problems = fixture_problems()
    cases = json.loads((GOLDEN / "aggdriver.json").read_text())
    assert len(cases) == 18
    for case in cases:
        p = problems[case["problem"]]
        roles = OracleAggregateRoles(p, case["N"], case["k"], case["Ns"], case["samples"])
        drv = AggregateDriver(WidestBranchPolicy(case["k"], case["N"]), WidestBranchPolicy(case["k"], case["Ns"]),
                              roles, case["rule"], case["iter_limit"], 1e-6)
        o = drv.solve(p)
        tag = (case["problem"], case["rule"])
        assert o["lower_bound"] == float.fromhex(case["lower_bound"]), tag
        assert o["upper_bound"] == float.fromhex(case["upper_bound"]), tag
        assert o["stop_reason"] == case["stop_reason"], tag
        assert int(o["proven_optimal"]) == case["proven_optimal"] and int(o["infeasible"]) == case["infeasible"], tag
        assert int(o["selection_rule_engaged"]) == case["selection_rule_engaged"], tag
        assert [o["counters"][k] for k in COUNTERS] == case["counters"], tag
        assert o["best_point"] == [float.fromhex(x) for x in case["best_point"]], tag
