"""The library's host builds of the branching policy and the region decode
(cmn_bisection_choose: the device policy of csrc/policy.cuh compiled for the
host; cmn_slot_bounds: the FMA-form decode) against the golden fixtures
generated from the reference's own BisectionBudgetCompositionPolicy::choose
(policy/bisection_budget.hpp) and decode::slot_bounds (region/decode.hpp),
and against the oracle's restatements of both on random inputs.  No GPU."""

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


def random_box(rng, n):
    """Random variable kinds and bounds, with repeated widths (heap ties),
    degenerate variables and small integer domains."""
    kinds, box = [], []
    widths = rng.choice([0.5, 1.0, 2.0, 3.0, 7.5], size=3)
    for _ in range(n):
        k = int(rng.choice([0, 0, 0, 1, 2]))
        if k == 2:  # binary: [0, 1] or fixed
            lo, hi = [(0.0, 1.0), (0.0, 0.0), (1.0, 1.0)][int(rng.integers(3))]
        elif k == 1:
            lo = float(rng.integers(-5, 3))
            hi = lo + float(rng.integers(0, 9))
        else:
            lo = float(np.round(rng.uniform(-8.0, 2.0), 2))
            hi = lo + (0.0 if rng.random() < 0.1 else float(widths[int(rng.integers(3))]))
        kinds.append(k)
        box += [lo, hi]
    return np.array(box), kinds


def test_library_policy_matches_oracle_on_random_boxes():
    # the oracle's restatement is pinned to the reference by the goldens
    # above; here the two agree on 2,000 random boxes and option sets
    from oracle import bisection_choose as oracle_choose
    rng = np.random.default_rng(77)
    for _ in range(2000):
        n = int(rng.integers(1, 41))
        box, kinds = random_box(rng, n)
        B = int(rng.integers(1, 13))
        max_cycle = int(rng.choice([0, 0, int(rng.integers(1, 6))]))
        cap = int(rng.choice([0, 0, int(rng.integers(2, 64))]))
        rel = bool(rng.random() < 0.3)
        a = bisection_choose(box, kinds, B, max_cycle, cap, rel)
        k, v, w, d = oracle_choose(box, kinds, B, max_cycle, cap, rel)
        assert (a.kinds, a.var_ids, a.widths, a.domains) == (list(map(int, k)), list(map(int, v)),
                                                             list(map(int, w)), list(map(int, d))), (box, kinds, B)


def test_library_decode_matches_oracle_on_random_parts():
    from oracle import slot_bounds as oracle_bounds
    rng = np.random.default_rng(78)
    for _ in range(20000):
        kind = int(rng.integers(0, 4))
        if kind == 0:
            plo = float(rng.uniform(-1e3, 1e3))
            phi = plo + float(rng.choice([0.0, rng.uniform(0, 1e-6), rng.uniform(0, 1e3)]))
        else:
            plo = float(rng.integers(-50, 50))
            phi = plo + float(rng.integers(0, 40))
        fan = int(rng.integers(1, 65))
        part = int(rng.integers(0, fan))
        assert slot_bounds(kind, plo, phi, part, fan) == oracle_bounds(kind, plo, phi, part, fan), (kind, plo, phi)
