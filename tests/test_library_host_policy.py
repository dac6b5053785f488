"""The library's host builds of the branching policy and the region decode
(cmn_bisection_choose: the device policy of csrc/policy.cuh compiled for the
host; cmn_slot_bounds: the FMA-form decode) against the golden fixtures
generated from the reference's own BisectionBudgetCompositionPolicy::choose
(policy/bisection_budget.hpp) and decode::slot_bounds (region/decode.hpp).
No GPU."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from cuminlp_gb300.solver import bisection_choose, slot_bounds

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_library_policy_matches_reference():
    cases = json.loads((GOLDEN / "policy.json").read_text())
    assert len(cases) >= 200
    for c in cases:
        box = np.array([float.fromhex(v) for pair in c["box"] for v in pair])
        a = bisection_choose(box, c["kinds"], c["B"], c["max_cycle"], c["enumerate_cap"], c["relative"])
        got = [[k, v, w, d] for k, v, w, d in zip(a.kinds, a.var_ids, a.widths, a.domains)]
        assert got == c["slots"], c


def test_library_decode_matches_reference():
    cases = json.loads((GOLDEN / "decode.json").read_text())
    assert len(cases) > 400
    for c in cases:
        lo, hi = slot_bounds(c["kind"], float.fromhex(c["plo"]), float.fromhex(c["phi"]), c["part"], c["fan"])
        assert lo == float.fromhex(c["lo"]) and hi == float.fromhex(c["hi"]), c
