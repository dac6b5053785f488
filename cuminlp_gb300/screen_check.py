"""Checks of the FP32 screen on the device: FP64 points inside FP32
enclosures, and the width inflation of FP32 enclosures node by node.

The screen (CMN_PRECISION_FP32_SCREEN) evaluates every node with its inputs
widened outward to FP32 and every operation directed, so its enclosure of a
box must contain the FP64 enclosure of the same box, and with it the FP64
value of every point in the box.  Both checks run through the public
evaluation call (cmn_eval_boxes):

- **Point containment.**  P uniform points per box (integer variables on
  their lattice) are evaluated in FP64, each as a degenerate box.  That
  enclosure holds the point's round-to-nearest FP64 value: an RN result lies
  between the RD and RU results of the same operation, and the interval
  operations are monotone in their endpoints.  Requiring it inside the box's
  FP32 enclosure is therefore the stronger test.  A box the screen proves
  infeasible must hold no point that FP64 keeps.
- **Width inflation.**  The FP32/FP64 width ratio of a node's enclosure,
  over many boxes.  A node's enclosure is the objective enclosure of the same
  DAG rooted at that node with no constraints.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _abi as A
from .problem import Problem
from .solver import DeviceProblem, eval_boxes


def sample_boxes(problem: Problem, n: int, rng: np.random.Generator, scale: float, centre=None):
    """n boxes inside the root box as (n_vars, n) lo/hi planes: uniform
    centres (or `centre`, clipped to the root box), half-widths up to
    `scale` of the root width, integer variables rounded inward to their
    lattice."""
    root = np.array(problem.box_bounds, dtype=np.float64)
    if centre is None:
        c = rng.uniform(root[:, 0:1], root[:, 1:2], (len(root), n))
    else:
        c = np.repeat(np.clip(np.asarray(centre, dtype=np.float64), root[:, 0], root[:, 1])[:, None], n, 1)
    w = rng.uniform(0, 1, (len(root), n)) * (root[:, 1:2] - root[:, 0:1]) * scale
    lo = np.maximum(c - w, root[:, 0:1])
    hi = np.minimum(c + w, root[:, 1:2])
    ints = np.array(problem.var_kinds) != A.VAR_CONTINUOUS
    lo[ints] = np.ceil(lo[ints])
    hi[ints] = np.maximum(np.floor(hi[ints]), lo[ints])
    return np.ascontiguousarray(lo), np.ascontiguousarray(hi)


def sample_points(lo: np.ndarray, hi: np.ndarray, var_kinds, n: int, rng: np.random.Generator) -> np.ndarray:
    """n uniform points of the box [lo, hi] as an (n_vars, n) plane; integer
    variables uniform over their lattice points."""
    x = lo[:, None] + rng.uniform(0, 1, (len(lo), n)) * (hi - lo)[:, None]
    x = np.minimum(np.maximum(x, lo[:, None]), hi[:, None])
    ints = np.array(var_kinds) != A.VAR_CONTINUOUS
    if ints.any():
        x[ints] = rng.integers(lo[ints].astype(np.int64)[:, None], hi[ints].astype(np.int64)[:, None] + 1,
                               (int(ints.sum()), n))
    return np.ascontiguousarray(x)


def point_containment(problem: Problem, n_boxes: int, points_per_box: int, rng: np.random.Generator,
                      scale: float = 0.05, dp: DeviceProblem | None = None, centre=None) -> dict:
    """FP64 points against the FP32 enclosure of their box.  Counts the
    points whose FP64 enclosure leaves the box's FP32 objective enclosure,
    and the FP64-feasible points in boxes the screen proves infeasible; both
    must be 0.  `centre` places every box around one point (a feasible one
    makes the second count meaningful)."""
    dp = dp or DeviceProblem(problem)
    lo, hi = sample_boxes(problem, n_boxes, rng, scale, centre)
    lb32, ub32, fe32 = eval_boxes(dp, lo, hi, A.PRECISION_FP32_SCREEN)
    outside = infeasible_kept = feasible = 0
    slack = []
    for b in range(n_boxes):
        x = sample_points(lo[:, b], hi[:, b], problem.var_kinds, points_per_box, rng)
        plb, pub, pfe = eval_boxes(dp, x, x, A.PRECISION_FP64)
        outside += int(np.count_nonzero((plb < lb32[b]) | (pub > ub32[b])))
        feasible += int(np.count_nonzero(pfe))
        if not fe32[b]:
            infeasible_kept += int(np.count_nonzero(pfe))
        # how much of the FP32 enclosure the points span
        span = float(pub.max() - plb.min())
        width = float(ub32[b] - lb32[b])
        slack.append(width / span if span > 0 else None)
    good = [s for s in slack if s is not None]
    return {"boxes": n_boxes, "points_per_box": points_per_box, "box_scale": scale,
            "centre": "uniform" if centre is None else "given point", "fp32_kept_boxes": int(np.count_nonzero(fe32)),
            "outside_fp32_enclosure": outside, "fp64_feasible_points": feasible,
            "feasible_points_in_screened_out_boxes": infeasible_kept,
            "fp32_width_over_point_span_p50": float(np.median(good)) if good else None}


def pick_nodes(problem: Problem, n_random: int, rng: np.random.Generator) -> list:
    """The objective root, every constraint root, and n_random other
    operation nodes (not constants or variables), in id order."""
    roots = {problem.objective_root} | {c.root_id for c in problem.constraints}
    ops = [nd.id for nd in problem.graph.nodes
           if nd.op not in (A.OP_CONST, A.OP_VAR) and nd.id not in roots]
    extra = rng.choice(ops, size=min(n_random, len(ops)), replace=False).tolist() if ops else []
    return sorted(roots | {int(i) for i in extra})


@dataclass
class NodeInflation:
    node: int
    ratio_p50: list   # per box set: median FP32/FP64 width ratio (None: no box of positive FP64 width)
    ratio_max: list
    contained: bool   # FP32 enclosure ⊇ FP64 enclosure on every box


def width_inflation(problem: Problem, box_sets: list, nodes: list) -> list:
    """Per node and per (lo, hi) box set, the FP32/FP64 width ratios of the
    node's enclosure."""
    arrays = problem.arrays()
    rows = []
    for nid in nodes:
        dp = DeviceProblem(problem, arrays=arrays, objective_root=nid, constraints=False)
        p50, pmax, contained = [], [], True
        for lo, hi in box_sets:
            lb64, ub64, _ = eval_boxes(dp, lo, hi, A.PRECISION_FP64)
            lb32, ub32, _ = eval_boxes(dp, lo, hi, A.PRECISION_FP32_SCREEN)
            contained = contained and bool(np.all(lb32 <= lb64) and np.all(ub32 >= ub64))
            w64 = ub64 - lb64
            w32 = ub32 - lb32
            ok = np.isfinite(w64) & np.isfinite(w32) & (w64 > 0)
            r = w32[ok] / w64[ok]
            p50.append(float(np.median(r)) if r.size else None)
            pmax.append(float(r.max()) if r.size else None)
        dp.close()
        rows.append(NodeInflation(int(nid), p50, pmax, contained))
    return rows


def inflation_summary(problem: Problem, rows: list, labels: list) -> dict:
    """Quantiles over nodes of each node's median ratio, per box set, with
    the objective and constraint roots apart."""
    obj = problem.objective_root
    cons = {c.root_id for c in problem.constraints}
    out = {"nodes": len(rows), "all_contained": all(r.contained for r in rows), "by_box_scale": {}}
    for k, lab in enumerate(labels):
        med = np.array([r.ratio_p50[k] for r in rows if r.ratio_p50[k] is not None])
        con = np.array([r.ratio_p50[k] for r in rows if r.node in cons and r.ratio_p50[k] is not None])
        o = [r.ratio_p50[k] for r in rows if r.node == obj]
        out["by_box_scale"][lab] = {
            "node_median_ratio_p50": float(np.median(med)) if med.size else None,
            "node_median_ratio_p90": float(np.quantile(med, 0.9)) if med.size else None,
            "node_median_ratio_max": float(med.max()) if med.size else None,
            "objective": o[0] if o else None,
            "constraint_roots_p50": float(np.median(con)) if con.size else None,
            "worst_box_ratio": max((r.ratio_max[k] for r in rows if r.ratio_max[k] is not None), default=None),
        }
    return out
