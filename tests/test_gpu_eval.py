"""Fused evaluator (a) on the GPU against the CPU oracle: bit-exact node
enclosures (signs of zero aside) in FP64 and in the FP32 screen, over
random, degenerate and zero-straddling boxes."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import _abi as A
from cuminlp_gb300 import generators as G
from cuminlp_gb300.solver import DeviceProblem, eval_boxes
from tests.conftest import bits_equal
from tests.gpu_common import ops_problem, random_boxes, with_objective

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cuminlp_gb300 import build
    build.build_library()


def check_eval(problem, n_boxes, seed, precision, scale=0.2):
    rng = np.random.default_rng(seed)
    lo, hi = random_boxes(problem, n_boxes, rng, scale)
    dp = DeviceProblem(problem)
    glb, gub, gfe = eval_boxes(dp, lo, hi, precision)
    olb, oub, ofe = O.OracleProblem(problem).eval_boxes(lo, hi, precision)
    assert bits_equal(glb, olb), np.flatnonzero(glb != olb)[:10]
    assert bits_equal(gub, oub)
    assert np.array_equal(gfe, ofe)
    return glb, gub, gfe


@pytest.mark.parametrize("precision", [A.PRECISION_FP64, A.PRECISION_FP32_SCREEN])
@pytest.mark.parametrize("n_vars,boxes,seed", [(4, 20000, 101), (32, 3000, 102), (64, 600, 103)])
def test_eval_boxes_match_oracle(n_vars, boxes, seed, precision):
    p = G.BY_N[n_vars]()
    lb, ub, fe = check_eval(p, boxes, seed, precision)
    assert np.all(lb <= ub)
    if n_vars == 4:
        assert 0 < fe.sum() < len(fe)  # both verdicts occur


@pytest.mark.parametrize("precision", [A.PRECISION_FP64, A.PRECISION_FP32_SCREEN])
def test_every_operator_matches_oracle(precision):
    check_eval(ops_problem(), 20000, 7, precision, scale=0.5)


@pytest.mark.parametrize("precision", [A.PRECISION_FP64, A.PRECISION_FP32_SCREEN])
def test_node_enclosures_match_oracle(precision):
    # each sampled node of the n=32 MIQCQP as the objective: its enclosure on every
    # box must equal the oracle's node-by-node evaluation
    p = G.miqcqp_n32()
    rng = np.random.default_rng(5)
    cands = [n.id for n in p.graph.nodes if n.op not in (A.OP_CONST,)]
    picks = sorted(set(rng.choice(cands, 60, replace=False).tolist()) | {p.objective_root})
    lo, hi = random_boxes(p, 512, rng, 0.3)
    op = O.OracleProblem(p)
    box0 = np.stack([lo[:, 3], hi[:, 3]], 1).reshape(-1)
    nlo, nhi = op.eval_nodes(box0, fp32=precision == A.PRECISION_FP32_SCREEN)
    for nid in picks:
        q = with_objective(p, nid)
        glb, gub, _ = eval_boxes(DeviceProblem(q), lo, hi, precision)
        olb, oub, _ = O.OracleProblem(q).eval_boxes(lo, hi, precision)
        assert bits_equal(glb, olb) and bits_equal(gub, oub), nid
        # and the whole-DAG oracle agrees on box 3
        assert bits_equal(np.float64(nlo[nid]), glb[3]) and bits_equal(np.float64(nhi[nid]), gub[3])


def test_fp32_screen_contains_fp64():
    p = G.miqcqp_n64()
    rng = np.random.default_rng(11)
    lo, hi = random_boxes(p, 2000, rng, 0.05)
    dp = DeviceProblem(p)
    lb64, ub64, fe64 = eval_boxes(dp, lo, hi, A.PRECISION_FP64)
    lb32, ub32, fe32 = eval_boxes(dp, lo, hi, A.PRECISION_FP32_SCREEN)
    assert np.all(lb32 <= lb64) and np.all(ub32 >= ub64)
    assert np.all(fe32 >= fe64)  # the screen never excludes what FP64 keeps


def test_enclosure_contains_sampled_points():
    p = G.miqcqp_n32()
    rng = np.random.default_rng(3)
    lo, hi = random_boxes(p, 256, rng, 0.1)
    dp = DeviceProblem(p)
    lb, ub, _ = eval_boxes(dp, lo, hi)
    op = O.OracleProblem(p)
    for b in range(0, 256, 8):
        for _ in range(20):
            x = rng.uniform(lo[:, b], hi[:, b])
            obj, _ = op.eval_point(x)
            assert lb[b] <= obj <= ub[b]
