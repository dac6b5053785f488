"""GAMS models through the device path: parsed by the frontend, solved by the
batched device solver, compared bit for bit with the oracle's batched
restatement (frontier, bounds, incumbent, counters)."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import gams, report
from cuminlp_gb300.solver import DeviceProblem, Solver
from tests.conftest import bits_equal

pytestmark = pytest.mark.gpu
DATA = Path(__file__).resolve().parent / "data" / "gams"


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cuminlp_gb300 import build
    build.build_library()


@pytest.mark.parametrize("name", ["bilinear_max.gms", "circle_fixed.gms"])
def test_gams_model_solves_like_the_oracle(name):
    pm = gams.parse_file(DATA / name)
    opts = dict(bisection_budget=3, batch_parents=32, frontier_cap=4096, iter_limit=20000)
    s = Solver(DeviceProblem(pm.problem), **opts)
    s.step(0)
    g = s.outcome()
    s.close()
    o = O.OracleProblem(pm.problem).solve_batched(**opts)
    for k in ("lower_bound", "upper_bound", "stop_reason", "proven_optimal", "frontier_size", "viable"):
        if isinstance(g[k], float):
            assert bits_equal(np.float64(g[k]), np.float64(o[k])), k
        else:
            assert g[k] == o[k], k
    assert g["counters"] == o["counters"]
    if g["found_incumbent"]:
        assert bits_equal(g["best_point"], o["best_point"])
    assert report.balances(g)
    line = report.result_line(g, maximise=pm.sense == "max")
    assert line.startswith("RESULT\tsense=" + pm.sense)
