"""CPU: the oracle's aggregate bound equals a fold, in Python, of the
oracle's pinned per-box evaluation over the decoded regions: region r is
child r // M; lb = min over feasible regions, hull_ub = max; a child with no
feasible region is (+inf, +inf, infeasible)
(backend/aggregate/kernels.cuh:32-47, replay.cuh:343-361)."""

from __future__ import annotations

import numpy as np

import oracle as O
from cuminlp_gb300 import _abi as A
from cuminlp_gb300 import generators as G
from tests.test_oracle_pins import fixture_problems


def decode_regions(box, vids, widths):
    """lo/hi planes (n, N) of every region, slot 0 least significant."""
    n = len(box) // 2
    N = int(np.prod(widths))
    lo = np.repeat(np.asarray(box[0::2], dtype=float)[:, None], N, 1)
    hi = np.repeat(np.asarray(box[1::2], dtype=float)[:, None], N, 1)
    prefix = 1
    for v, w in zip(vids, widths):
        for r in range(N):
            part = (r // prefix) % w
            lo[v, r], hi[v, r] = O.slot_bounds(A.SLOT_CONTINUOUS, box[2 * v], box[2 * v + 1], part, w)
        prefix *= w
    assert lo.shape[0] == n
    return lo, hi


def fold(lb, ub, fe, k):
    M = len(lb) // k
    out = []
    for c in range(k):
        s = slice(c * M, (c + 1) * M)
        live = fe[s] != 0
        if not live.any():
            out.append((np.inf, np.inf, 0))
        else:
            out.append((lb[s][live].min(), ub[s][live].max(), 1))
    return out


def test_aggregate_oracle_is_a_fold_of_box_evaluation():
    for p, vids, widths, k in ((G.qcqp_n4(), [1, 2, 0], [4, 4, 4], 4), (G.qcqp_n4(3), [3, 0], [8, 2], 2),
                               (fixture_problems()["infeasible"], [0], [8], 4)):
        box = p.root_box()
        op = O.OracleProblem(p)
        kinds = [A.SLOT_CONTINUOUS] * len(vids)
        N = int(np.prod(widths))
        lb, ub, fe = op.aggregate_bound(box, kinds, vids, widths, N, k, threads=1)
        lo, hi = decode_regions(box, vids, widths)
        elb, eub, efe = op.eval_boxes(lo, hi, threads=1)
        want = fold(elb, eub, efe, k)
        assert [(a, b, int(c)) for a, b, c in zip(lb, ub, fe)] == want
