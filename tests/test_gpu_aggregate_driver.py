"""The host aggregate driver over the device roles (cmn_bound_children,
cmn_sample) against the same driver over the oracle's roles: the trajectory
must be identical, so the device aggregate bounder and sampler decide every
prune and incumbent exactly as the oracle does."""

from __future__ import annotations

import pytest

from cuminlp_gb300 import generators as G
from cuminlp_gb300.aggregate import AggregateDriver, DeviceAggregateRoles, WidestBranchPolicy, solve_aggregate
from cuminlp_gb300.solver import DeviceProblem
from tests.aggregate_roles import OracleAggregateRoles
from tests.test_oracle_pins import fixture_problems

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cuminlp_gb300 import build
    build.build_library()


@pytest.mark.parametrize("rule", ["least-lower-bound", "reject-index"])
@pytest.mark.parametrize("name", ["aggregate_fixture", "miqcqp_n6", "cfg1b", "int_eq"])
def test_device_roles_reproduce_oracle_roles(name, rule):
    fx = fixture_problems()
    p = G.config1(1) if name == "cfg1b" else fx[name]
    k, N, Ns, S = 4, 256, 64, 2
    runs = []
    for roles in (DeviceAggregateRoles(DeviceProblem(p), N, k, Ns, S), OracleAggregateRoles(p, N, k, Ns, S)):
        drv = AggregateDriver(WidestBranchPolicy(k, N), WidestBranchPolicy(k, Ns), roles, rule, 300, 1e-6)
        runs.append(drv.solve(p))
    a, b = runs
    assert a == b


def test_solve_aggregate_converges_on_config1():
    o = solve_aggregate(G.config1(1), branch_fan_out=2, total_fan_out=1 << 10, sample_fan_out=1 << 6,
                        iter_limit=5000)
    assert o["stop_reason"] == "converged" and o["proven_optimal"]
