"""The allocation-free sampler entry point (cmn_sample_noalloc).

It serves callers that cannot call cudaMalloc -- a process whose device
memory belongs to a pool it does not control, or code that must not grow
its device footprint -- by keeping its scratch in a fixed device array
inside the library.  Called through the C ABI, it must return exactly what
the ordinary sampler role returns for the same region and salt, on two
calls in a row (the second call reuses the scratch the first left
behind).  Collected last so that a run stopping at the first failure has
already run every other test."""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import _abi as A
from cuminlp_gb300 import generators as G
from cuminlp_gb300._lib import CmnError, check, lib
from cuminlp_gb300.problem import Problem
from cuminlp_gb300.solver import DeviceProblem, Sampler

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cuminlp_gb300 import build
    build.build_library()


def sample_noalloc(dp, kinds, n_regions, S, box, vids, widths, salt):
    kinds = np.ascontiguousarray(kinds, dtype=np.uint8)
    vids = np.ascontiguousarray(vids, dtype=np.uint64)
    widths = np.ascontiguousarray(widths, dtype=np.uint64)
    box = np.ascontiguousarray(box, dtype=np.float64)
    point = np.empty(dp.n_vars)
    cand = A.Candidate()
    check(lib().cmn_sample_noalloc(dp.handle, A.ptr(kinds), len(kinds), n_regions, S, A.ptr(box), A.ptr(vids),
                                   A.ptr(widths), salt, C.byref(cand), A.ptr(point), None))
    return bool(cand.found), cand.value, point, cand.index


@pytest.mark.parametrize("n_vars,B,S", [(4, 10, 4), (32, 12, 1), (512, 10, 2)])
def test_noalloc_sampler_matches_sampler_role(n_vars, B, S):
    # n = 512: a wide QCQP whose points are shared by lane groups
    if n_vars == 512:
        from tests.test_gpu_roles import wide_qcqp
        p = wide_qcqp()
    else:
        p = G.BY_N[n_vars]()
    dp = DeviceProblem(p)
    box = p.root_box()
    kinds, vids, widths, _ = O.bisection_choose(box, p.var_kinds, B)
    n_regions = int(np.prod(widths))
    role = Sampler(dp, kinds, n_regions, sample_points=S)
    for salt in (3, 4):  # two calls in a row through the shared scratch
        want = role.sample(box, vids, widths, salt)
        got = sample_noalloc(dp, kinds, n_regions, S, box, vids, widths, salt)
        assert got[0] == want.found
        assert got[1] == want.value and got[3] == want.index
        assert np.array_equal(got[2], want.point, equal_nan=True)  # all-NaN when nothing is found


def test_noalloc_sampler_infeasible_and_limits():
    p = Problem()
    x = p.var(0.0, 10.0)
    p.set_objective(x * x)
    p.add_constraint(x, A.CMP_LE, -100.0)
    dp = DeviceProblem(p)
    found, value, point, index = sample_noalloc(dp, [A.SLOT_CONTINUOUS], 4, 16, p.root_box(), [0], [4], 1)
    assert not found and np.isnan(point[0]) and index == -1
    with pytest.raises(CmnError) as e:
        sample_noalloc(dp, [A.SLOT_CONTINUOUS], 4, 16, p.root_box(), [0], [3], 1)
    assert e.value.status_name == "SHAPE_MISMATCH"
    big = Problem()
    xs = [big.var(-1.0, 1.0) for _ in range(9000)]
    big.set_objective(xs[0] * xs[1])
    dbig = DeviceProblem(big)
    with pytest.raises(CmnError) as e:
        sample_noalloc(dbig, [A.SLOT_CONTINUOUS], 2, 1, big.root_box(), [0], [2], 1)
    assert e.value.status_name == "INVALID_CONFIGURATION" and "8192" in str(e.value)
