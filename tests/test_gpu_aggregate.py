"""The aggregate bounder (AggregateBounder::bound_children, with the mask and
per-child Min/Max of backend/aggregate/) against the oracle: k children of
N / k contiguous regions each, refine slots first and branch slots last, as
aggregate/partition.hpp lays a partition out."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import _abi as A
from cuminlp_gb300 import generators as G
from cuminlp_gb300._lib import CmnError
from cuminlp_gb300.solver import Bounder, DeviceProblem
from tests.conftest import bits_equal
from tests.test_oracle_pins import fixture_problems

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cuminlp_gb300 import build
    build.build_library()


def layout(n_vars, k):
    """(slot kinds, var ids, widths) with the branch slot last."""
    C = A.SLOT_CONTINUOUS
    if n_vars == 4:
        return [C, C, C], [1, 2, 0], [8, 4, k]
    return [C, C, C], [5, 6, 4], [16, 8, k]


def check(p, kinds, vids, widths, box, k):
    n_regions = int(np.prod(widths))
    dp = DeviceProblem(p)
    b = Bounder(dp, kinds, n_regions)
    lb, ub, fe = b.bound_children(box, vids, widths, k)
    olb, oub, ofe = O.OracleProblem(p).aggregate_bound(box, kinds, vids, widths, n_regions, k)
    assert bits_equal(lb, olb) and bits_equal(ub, oub)
    assert np.array_equal(fe, ofe)
    # against the per-region bounder: the fold of its verdicts
    rfe, rlb = b.bound(box, vids, widths)
    M = n_regions // k
    for c in range(k):
        seg = slice(c * M, (c + 1) * M)
        live = rfe[seg] != 0
        if live.any():
            assert fe[c] == 1 and lb[c] == rlb[seg][live].min()
        else:
            assert fe[c] == 0 and lb[c] == np.inf and ub[c] == np.inf
    return lb, ub, fe


@pytest.mark.parametrize("k", [1, 2, 4, 16])
@pytest.mark.parametrize("n_vars", [4, 32])
def test_bound_children_matches_oracle(n_vars, k):
    p = G.BY_N[n_vars]()
    kinds, vids, widths = layout(n_vars, k)
    lb, ub, fe = check(p, kinds, vids, widths, p.root_box(), k)
    assert np.all(lb[fe == 1] <= ub[fe == 1])


def test_small_segments_span_warps():
    # M = 2: every warp holds 16 children, the per-lane atomic path
    p = G.qcqp_n4()
    kinds = [A.SLOT_CONTINUOUS, A.SLOT_CONTINUOUS]
    _, _, fe = check(p, kinds, [1, 0], [2, 64], p.root_box(), 64)
    assert 0 < fe.sum() <= 64


def test_infeasible_children_are_normalised():
    p = fixture_problems()["infeasible"]
    n = p.n_vars
    kinds = [A.SLOT_CONTINUOUS]
    lb, ub, fe = check(p, kinds, [0], [8], p.root_box(), 4)
    assert fe.tolist() == [0, 0, 0, 0] and np.all(lb == np.inf) and np.all(ub == np.inf)
    assert n >= 1


def test_k_must_divide_regions():
    p = G.qcqp_n4()
    b = Bounder(DeviceProblem(p), [A.SLOT_CONTINUOUS], 8)
    with pytest.raises(CmnError) as e:
        b.bound_children(p.root_box(), [0], [8], 3)
    assert e.value.status_name == "SHAPE_MISMATCH"
