"""Lane groups: a box evaluated by a group of lanes, each running its share
of the program's independent sum chains, gives the same bits as one lane
running the whole program.  Few boxes take the grouped path, many boxes the
one-lane path; the same boxes must agree, and both must equal the oracle."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import _abi as A
from cuminlp_gb300 import generators as G
from cuminlp_gb300.solver import DeviceProblem, eval_boxes
from tests.conftest import bits_equal
from tests.gpu_common import random_boxes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cuminlp_gb300 import build
    build.build_library()


def problems():
    ps = {"qcqp_n4": G.qcqp_n4(), "miqcqp_n32": G.miqcqp_n32(), "miqcqp_n64": G.miqcqp_n64()}
    for i in (0, 2, 10):
        ps[f"serving_{i}"] = G.serving_qcqp(i)
    ps["uneven_0"] = G.uneven_qcqp(0)
    return ps


@pytest.mark.parametrize("precision", [A.PRECISION_FP64, A.PRECISION_FP32_SCREEN])
@pytest.mark.parametrize("name", list(problems()))
def test_grouped_equals_one_lane(name, precision):
    p = problems()[name]
    dp = DeviceProblem(p)
    info = dp.info()
    assert info["program_slots"] > 0 or info["program_segments"] >= 1
    rng = np.random.default_rng(11)
    many = 120000  # above the resident threads: one lane per box
    lo, hi = random_boxes(p, many, rng, 0.3)
    lb1, ub1, fe1 = eval_boxes(dp, lo, hi, precision)
    for few in (1, 7, 64):  # grouped: up to lanes_per_box_max lanes per box
        lb2, ub2, fe2 = eval_boxes(dp, np.ascontiguousarray(lo[:, :few]), np.ascontiguousarray(hi[:, :few]),
                                   precision)
        assert bits_equal(lb2, lb1[:few]) and bits_equal(ub2, ub1[:few]), (name, few)
        assert np.array_equal(fe2, fe1[:few]), (name, few)
    # and both against the oracle on a sample
    op = O.OracleProblem(p)
    idx = np.arange(0, many, many // 200)
    olb, oub, ofe = op.eval_boxes(np.ascontiguousarray(lo[:, idx]), np.ascontiguousarray(hi[:, idx]), precision)
    assert bits_equal(lb1[idx], olb) and bits_equal(ub1[idx], oub)
    assert np.array_equal(fe1[idx], ofe)


def test_segments_reported():
    info = DeviceProblem(G.miqcqp_n32()).info()
    assert info["program_segments"] == 17  # objective + 16 constraints
    assert info["lanes_per_box_max"] >= 4
