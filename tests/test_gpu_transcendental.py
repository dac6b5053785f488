"""Exp, Log, Sin, Cos, Tanh and Pow on the device: enclosures, not tightest,
and unpinned by any reference result (the reference delegates them to the
un-vendored cuinterval library).  The bar is the one of the reference's own
aggregate_backend_test.cu:208-253: every FP64 point of a box evaluates, in
FP64 on the host, inside the box's device enclosure -- in FP64 and in the
FP32 screen -- and the FP64 enclosure is no wider than the exact range plus
a few ulps of widening."""

from __future__ import annotations

import math

import numpy as np
import pytest

from cuminlp_gb300 import _abi as A
from cuminlp_gb300.problem import Expr, Problem
from cuminlp_gb300.solver import DeviceProblem, eval_boxes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cuminlp_gb300 import build
    build.build_library()


def unary_problem(op: int, lo: float, hi: float) -> Problem:
    p = Problem()
    x = p.var(lo, hi)
    p.set_objective(Expr(p.graph, p.graph.emit(op, (x.id,))))
    return p


def pow_problem() -> Problem:
    p = Problem()
    x = p.var(0.0, 4.0)
    y = p.var(-2.0, 3.0)
    p.set_objective(Expr(p.graph, p.graph.emit(A.OP_POW, (x.id, y.id))))
    return p


def boxes(rng, lo, hi, n, max_width):
    c = rng.uniform(lo, hi, n)
    w = rng.uniform(0, max_width, n)
    w[: n // 8] = 0.0
    return np.maximum(c - w, lo), np.minimum(c + w, hi)


CASES = [
    (A.OP_EXP, -30.0, 30.0, np.exp),
    (A.OP_LOG, 1e-6, 1e3, np.log),
    (A.OP_SIN, -40.0, 40.0, np.sin),
    (A.OP_COS, -40.0, 40.0, np.cos),
    (A.OP_TANH, -8.0, 8.0, np.tanh),
]


def exact_range(f, lo, hi, op):
    """The function's range over [lo, hi] from a fine grid plus the known
    extrema (sin/cos), in FP64."""
    xs = np.linspace(lo, hi, 257)
    v = f(xs)
    r = [v.min(), v.max()]
    if op in (A.OP_SIN, A.OP_COS):
        shift = 0.5 if op == A.OP_SIN else 0.0
        j0, j1 = math.ceil(lo / math.pi - shift), math.floor(hi / math.pi - shift)
        for j in range(j0, j1 + 1):
            val = 1.0 if j % 2 == 0 else -1.0
            r = [min(r[0], val), max(r[1], val)]
    return r


@pytest.mark.parametrize("op,lo,hi,f", CASES)
def test_unary_enclosures_contain_fp64_points(op, lo, hi, f):
    rng = np.random.default_rng(op)
    p = unary_problem(op, lo, hi)
    dp = DeviceProblem(p)
    blo, bhi = boxes(rng, lo, hi, 4096, (hi - lo) * 0.05)
    for prec in (A.PRECISION_FP64, A.PRECISION_FP32_SCREEN):
        elo, ehi, _ = eval_boxes(dp, blo[None, :], bhi[None, :], prec)
        t = rng.uniform(0, 1, (blo.size, 32))
        pts = blo[:, None] + t * (bhi - blo)[:, None]
        pts[:, 0], pts[:, 1] = blo, bhi
        vals = f(pts)
        assert np.all(vals >= elo[:, None]) and np.all(vals <= ehi[:, None]), prec
    # FP64: at most the exact range widened by a few ulps (and a few ulps of
    # the grid's own approximation of the extremes)
    elo, ehi, _ = eval_boxes(dp, blo[None, :], bhi[None, :], A.PRECISION_FP64)
    for i in range(0, blo.size, 97):
        r = exact_range(f, blo[i], bhi[i], op)
        slack = 16 * np.spacing(max(abs(r[0]), abs(r[1]), 1e-300)) + 1e-9 * (r[1] - r[0])
        assert elo[i] >= r[0] - slack - (r[1] - r[0]) * 1e-3
        assert ehi[i] <= r[1] + slack + (r[1] - r[0]) * 1e-3


def test_pow_enclosure_contains_fp64_points():
    rng = np.random.default_rng(7)
    p = pow_problem()
    dp = DeviceProblem(p)
    xl, xh = boxes(rng, 0.0, 4.0, 2048, 0.2)
    yl, yh = boxes(rng, -2.0, 3.0, 2048, 0.3)
    lo = np.stack([xl, yl])
    hi = np.stack([xh, yh])
    for prec in (A.PRECISION_FP64, A.PRECISION_FP32_SCREEN):
        elo, ehi, _ = eval_boxes(dp, lo, hi, prec)
        t = rng.uniform(0, 1, (2, xl.size, 16))
        xs = xl[:, None] + t[0] * (xh - xl)[:, None]
        ys = yl[:, None] + t[1] * (yh - yl)[:, None]
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            vals = np.power(xs, ys)
        ok = np.isfinite(vals)
        assert np.all((vals >= elo[:, None]) | ~ok) and np.all((vals <= ehi[:, None]) | ~ok), prec
