"""Host side of the FP32 screen checks (cuminlp_gb300/screen_check.py): box
and point sampling, the node choice and the re-rooted problem description.
No GPU: the device half is test_gpu_screen_check.py."""

from __future__ import annotations

import numpy as np

from cuminlp_gb300 import _abi as A
from cuminlp_gb300 import generators as G
from cuminlp_gb300 import screen_check as S


def test_points_stay_in_their_box_and_on_the_lattice():
    p = G.miqcqp_n64()
    rng = np.random.default_rng(1)
    lo, hi = S.sample_boxes(p, 6, rng, 0.2)
    ints = np.array(p.var_kinds) != A.VAR_CONTINUOUS
    root = np.array(p.box_bounds)
    assert np.all(lo <= hi) and np.all(lo >= root[:, 0:1]) and np.all(hi <= root[:, 1:2])
    assert np.all(lo[ints] == np.round(lo[ints])) and np.all(hi[ints] == np.round(hi[ints]))
    for b in range(6):
        x = S.sample_points(lo[:, b], hi[:, b], p.var_kinds, 5000, rng)
        assert x.shape == (p.n_vars, 5000)
        assert np.all(x >= lo[:, b:b + 1]) and np.all(x <= hi[:, b:b + 1])
        assert np.all(x[ints] == np.round(x[ints]))
        # every lattice point of a narrow integer range is drawn
        wide = np.flatnonzero(ints & (hi[:, b] - lo[:, b] >= 1))
        for v in wide[:2]:
            assert set(np.unique(x[v]).tolist()) == set(range(int(lo[v, b]), int(hi[v, b]) + 1))


def test_node_choice_covers_the_roots_and_skips_leaves():
    p = G.miqcqp_n64()
    a = S.pick_nodes(p, 40, np.random.default_rng(7))
    b = S.pick_nodes(p, 40, np.random.default_rng(7))
    assert a == b == sorted(a)
    assert p.objective_root in a and all(c.root_id in a for c in p.constraints)
    assert len(a) == 1 + len(p.constraints) + 40
    ops = {nd.id: nd.op for nd in p.graph.nodes}
    assert all(ops[i] not in (A.OP_CONST, A.OP_VAR) for i in a)


def test_rerooted_description_shares_the_node_table():
    p = G.miqcqp_n32()
    arrays = p.arrays()
    nid = p.constraints[3].root_id
    d, keep = p.desc(arrays=arrays, objective_root=nid, constraints=False)
    assert d.objective_root == nid and d.n_constraints == 0 and not d.constraints
    assert d.nodes == arrays[0].ctypes.data and d.n_nodes == len(p.graph.nodes)
    d0, _ = p.desc()
    assert d0.objective_root == p.objective_root and d0.n_constraints == len(p.constraints)
