"""The FP32 screen against FP64 on the n=64 MIQCQP: 10^5 FP64
points per box inside the box's FP32 enclosure, and the FP32/FP64 width
ratios node by node, checked against the oracle's node enclosures."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import generators as G
from cuminlp_gb300 import screen_check as S
from cuminlp_gb300.solver import DeviceProblem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scale,at_origin", [(0.01, False), (0.3, False), (0.03, True)])
def test_fp64_points_lie_in_fp32_enclosures(scale, at_origin):
    p = G.miqcqp_n64()
    # boxes around the origin, which satisfies every constraint (zero
    # quadratic and linear terms, rhs >= 1), hold FP64-feasible points
    centre = np.zeros(p.n_vars) if at_origin else None
    r = S.point_containment(p, n_boxes=4, points_per_box=100_000, rng=np.random.default_rng(5), scale=scale,
                            dp=DeviceProblem(p), centre=centre)
    assert r["outside_fp32_enclosure"] == 0, r
    assert r["feasible_points_in_screened_out_boxes"] == 0, r
    if at_origin:
        assert r["fp64_feasible_points"] > 0 and r["fp32_kept_boxes"] == 4, r


def test_width_inflation_matches_oracle_node_enclosures():
    p = G.miqcqp_n64()
    rng = np.random.default_rng(9)
    nodes = S.pick_nodes(p, 16, rng)
    sets = [S.sample_boxes(p, 12, rng, s) for s in (1e-3, 1e-1)]
    rows = S.width_inflation(p, sets, nodes)
    assert all(r.contained for r in rows)
    op = O.OracleProblem(p)
    for k, (lo, hi) in enumerate(sets):
        enc = []
        for b in range(lo.shape[1]):
            box = np.stack([lo[:, b], hi[:, b]], 1).reshape(-1)
            l64, h64 = op.eval_nodes(box)
            l32, h32 = op.eval_nodes(box, fp32=True)
            enc.append((l64, h64, l32.astype(np.float64), h32.astype(np.float64)))
        for r in rows:
            w64 = np.array([e[1][r.node] - e[0][r.node] for e in enc])
            w32 = np.array([e[3][r.node] - e[2][r.node] for e in enc])
            ok = np.isfinite(w64) & np.isfinite(w32) & (w64 > 0)
            want = float(np.median(w32[ok] / w64[ok])) if ok.any() else None
            assert r.ratio_p50[k] == want, (r.node, k, r.ratio_p50[k], want)
            if want is not None:
                assert r.ratio_p50[k] >= 1.0
    summary = S.inflation_summary(p, rows, ["1e-3", "1e-1"])
    assert summary["all_contained"] and summary["nodes"] == len(nodes)
