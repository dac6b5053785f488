"""Pins the CPU oracle before it is trusted as the checker.

- directed rounding and every interval operator of the QCQP path against
  exact rational arithmetic (each bound must be the nearest representable
  value on the correct side: the unique tightest enclosure);
- region decode, the BisectionBudget policy and the whole SearchDriver loop
  against golden fixtures produced by the reference's own host code
  (tests/golden/make_golden.py);
- the reference's known-answer cases (graph_replay_test.cu,
  backend_contract.hpp, aggregate_backend_test.cu, sample_discrete_test.cu).
"""

from __future__ import annotations

import json
import math
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import _abi as A
from cuminlp_gb300 import generators as G
from cuminlp_gb300.problem import Problem

GOLDEN = Path(__file__).resolve().parent / "golden"


def rand_doubles(rng: np.random.Generator, n: int) -> np.ndarray:
    mant = rng.uniform(1.0, 2.0, n)
    ex = rng.integers(-40, 40, n)
    sign = rng.choice([-1.0, 1.0], n)
    x = sign * mant * np.exp2(ex)
    special = np.array([0.0, -0.0, 1.0, -1.0, 0.5, 3.0, -7.25, 1e-300, 2.0 ** -1022, 1e300])
    return np.concatenate([x, special])



def is_rd(r: float, q: Fraction) -> bool:
    nxt = math.nextafter(r, math.inf)
    return (r == -math.inf or Fraction(r) <= q) and (math.isinf(nxt) or Fraction(nxt) > q)


def is_ru(r: float, q: Fraction) -> bool:
    prv = math.nextafter(r, -math.inf)
    return (r == math.inf or Fraction(r) >= q) and (math.isinf(prv) or Fraction(prv) < q)


def is_rd32(r: float, q: Fraction) -> bool:
    nxt = float(np.nextafter(np.float32(r), np.float32(np.inf)))
    return Fraction(r) <= q and (math.isinf(nxt) or Fraction(nxt) > q)


def is_ru32(r: float, q: Fraction) -> bool:
    prv = float(np.nextafter(np.float32(r), np.float32(-np.inf)))
    return Fraction(r) >= q and (math.isinf(prv) or Fraction(prv) < q)


def test_directed_rounding_is_exact():
    L = O.lib()
    rng = np.random.default_rng(1)
    a = rand_doubles(rng, 3000)
    b = rand_doubles(rng, 3000)
    rng.shuffle(b)
    for x, y in zip(a, b):
        x, y = float(x), float(y)
        s = Fraction(x) + Fraction(y)
        assert is_rd(L.orc_add_rd(x, y), s) and is_ru(L.orc_add_ru(x, y), s)
        p = Fraction(x) * Fraction(y)
        if abs(p) > Fraction(2.0 ** -1000) or p == 0:
            assert is_rd(L.orc_mul_rd(x, y), p) and is_ru(L.orc_mul_ru(x, y), p)
        if y != 0.0:
            q = Fraction(x) / Fraction(y)
            if abs(q) > Fraction(2.0 ** -1000) and abs(q) < Fraction(2.0 ** 1000):
                assert is_rd(L.orc_div_rd(x, y), q) and is_ru(L.orc_div_ru(x, y), q)


def test_directed_rounding_fp32_is_exact():
    L = O.lib()
    rng = np.random.default_rng(2)
    a = rng.uniform(-1e4, 1e4, 3000).astype(np.float32)
    b = (rng.uniform(-1, 1, 3000) * np.exp2(rng.integers(-30, 30, 3000))).astype(np.float32)
    for x, y in zip(a, b):
        x, y = float(x), float(y)
        s = Fraction(x) + Fraction(y)
        assert is_rd32(L.orc_addf_rd(x, y), s) and is_ru32(L.orc_addf_ru(x, y), s)
        p = Fraction(x) * Fraction(y)
        assert is_rd32(L.orc_mulf_rd(x, y), p) and is_ru32(L.orc_mulf_ru(x, y), p)
    for d in rand_doubles(rng, 2000):
        d = float(d)
        if abs(d) > 1e30 or (d != 0 and abs(d) < 1e-30):
            continue
        q = Fraction(d)
        assert is_rd32(L.orc_d2f_rd(d), q) and is_ru32(L.orc_d2f_ru(d), q)


def rand_interval(rng, kind):
    x = float(rng.uniform(-50, 50))
    w = float(rng.uniform(0, 30)) * (2.0 ** int(rng.integers(-20, 1)))
    if kind == 0:
        return (x, x + w)
    if kind == 1:
        return (abs(x), abs(x) + w)
    if kind == 2:
        return (-abs(x) - w, -abs(x))
    if kind == 3:
        return (0.0, w)
    return (-w, 0.0)


@pytest.mark.parametrize("fp32", [False, True])
def test_interval_operators_are_tightest(fp32):
    rng = np.random.default_rng(3 + fp32)
    chk_lo = is_rd32 if fp32 else is_rd
    chk_hi = is_ru32 if fp32 else is_ru
    conv = (lambda v: float(np.float32(v))) if fp32 else (lambda v: v)
    for _ in range(3000):
        a = tuple(map(conv, rand_interval(rng, int(rng.integers(0, 5)))))
        b = tuple(map(conv, rand_interval(rng, int(rng.integers(0, 5)))))
        a = (min(a), max(a))
        b = (min(b), max(b))
        fa = [Fraction(v) for v in a]
        fb = [Fraction(v) for v in b]
        cases = {
            A.OP_ADD: (fa[0] + fb[0], fa[1] + fb[1]),
            A.OP_SUB: (fa[0] - fb[1], fa[1] - fb[0]),
        }
        prods = [x * y for x in fa for y in fb]
        cases[A.OP_MUL] = (min(prods), max(prods))
        if fa[0] >= 0:
            sq = (fa[0] ** 2, fa[1] ** 2)
        elif fa[1] <= 0:
            sq = (fa[1] ** 2, fa[0] ** 2)
        else:
            sq = (Fraction(0), max(fa[0] ** 2, fa[1] ** 2))
        cases[A.OP_SQR] = sq
        cases[A.OP_NEG] = (-fa[1], -fa[0])
        if fb[0] > 0 or fb[1] < 0:
            quots = [x / y for x in fa for y in fb]
            cases[A.OP_DIV] = (min(quots), max(quots))
        for op, (qlo, qhi) in cases.items():
            lo, hi = O.interval_op(op, a, b, fp32=fp32)
            assert chk_lo(lo, qlo), (op, a, b, lo, qlo)
            assert chk_hi(hi, qhi), (op, a, b, hi, qhi)


def test_decode_matches_reference():
    cases = json.loads((GOLDEN / "decode.json").read_text())
    assert len(cases) > 400
    for c in cases:
        lo, hi = O.slot_bounds(c["kind"], float.fromhex(c["plo"]), float.fromhex(c["phi"]), c["part"], c["fan"])
        assert lo == float.fromhex(c["lo"]) and hi == float.fromhex(c["hi"]), c


def test_decode_known_answers():
    # region/decode.hpp: fan-out 4 of [0, 10]; top part snaps to the parent
    parts = [O.slot_bounds(A.SLOT_CONTINUOUS, 0.0, 10.0, p, 4) for p in range(4)]
    assert parts == [(0.0, 2.5), (2.5, 5.0), (5.0, 7.5), (7.5, 10.0)]
    assert O.slot_bounds(A.SLOT_INTEGER_ENUMERATE, 2.4, 5.6, 1, 50) == (4.0, 4.0)
    assert O.slot_bounds(A.SLOT_INTEGER_ENUMERATE, 0.0, 3.0, 10, 50) == (3.0, 3.0)
    assert O.slot_bounds(A.SLOT_BINARY_ENUMERATE, 0.0, 1.0, 1, 2) == (1.0, 1.0)


def test_bisection_policy_matches_reference():
    cases = json.loads((GOLDEN / "policy.json").read_text())
    assert len(cases) >= 200
    n_ties = 0
    for c in cases:
        box = np.array([float.fromhex(v) for pair in c["box"] for v in pair])
        kinds, vids, widths, dom = O.bisection_choose(box, c["kinds"], c["B"], c["max_cycle"], c["enumerate_cap"],
                                                      c["relative"])
        got = [[int(k), int(v), int(w), int(d)] for k, v, w, d in zip(kinds, vids, widths, dom)]
        assert got == c["slots"], c
        w = box[1::2] - box[0::2]
        n_ties += len(w) != len(set(w.tolist()))
    assert n_ties > 50  # equal widths exercise the heap's tie order


def fixture_problems():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.fixture_problems()


def test_driver_restatement_matches_reference():
    cases = json.loads((GOLDEN / "driver.json").read_text())
    probs = fixture_problems()
    for c in cases:
        op = O.OracleProblem(probs[c["problem"]])
        r = op.solve_reference(iter_limit=c["iter_limit"], bisection_budget=c["B"], sample_points=c["samples"],
                               threads=1)
        assert r["lower_bound"] == float.fromhex(c["lower_bound"]), c["problem"]
        assert r["upper_bound"] == float.fromhex(c["upper_bound"]), c["problem"]
        assert r["stop_reason"] == c["stop_reason"], c["problem"]
        assert r["proven_optimal"] == c["proven_optimal"] and r["infeasible"] == c["infeasible"]
        rc = r["counters"]
        for k in ("fathomed", "fathomed_points", "bounded", "sampled", "enqueued", "witness_rejected",
                  "pruned_duplicate", "pruned_infeasible", "pruned_dominated"):
            assert rc[k] == c["counters"][k], (c["problem"], k)
        assert rc["iterations"] == c["counters"]["iterations"]
        assert r["frontier_size"] == c["counters"]["pending"] and r["viable"] == c["counters"]["viable"]
        want = [float.fromhex(v) for v in c["best_point"]]
        if want:
            assert np.array_equal(r["best_point"], np.array(want)), c["problem"]


def test_known_answer_square_le5():
    # graph_replay_test.cu:77-84 -- x in [0,10], obj x^2, x <= 5, fan-out 4
    p = Problem()
    x = p.var(0.0, 10.0)
    p.set_objective(x * x)
    p.add_constraint(x, A.CMP_LE, 5.0)
    op = O.OracleProblem(p)
    fe, lb = op.bound(p.root_box(), [A.SLOT_CONTINUOUS], [0], [4], 4)
    assert lb.tolist() == [0.0, 6.25, 25.0, 56.25]
    assert fe.tolist() == [1, 1, 1, 0]
    found, val, pt, idx = op.sample(np.array([0.0, 5.0]), [A.SLOT_CONTINUOUS], [0], [4], 4, 16, 1)
    assert found and not math.isnan(pt[0]) and val == pt[0] * pt[0]


def test_known_answer_infeasible_has_nan_witness():
    p = Problem()
    x = p.var(0.0, 10.0)
    p.set_objective(x * x)
    p.add_constraint(x, A.CMP_LE, -100.0)
    op = O.OracleProblem(p)
    found, val, pt, idx = op.sample(p.root_box(), [A.SLOT_CONTINUOUS], [0], [4], 4, 16, 1)
    assert not found and math.isnan(pt[0])


def test_sampler_determinism_and_salt():
    p = Problem()
    x = p.var(0.0, 10.0)
    p.set_objective(x * x)
    p.add_constraint(x, A.CMP_LE, 5.0)
    op = O.OracleProblem(p)
    box = np.array([0.0, 5.0])
    a = op.sample(box, [A.SLOT_CONTINUOUS], [0], [4], 4, 32, 7)
    b = op.sample(box, [A.SLOT_CONTINUOUS], [0], [4], 4, 32, 7)
    c = op.sample(box, [A.SLOT_CONTINUOUS], [0], [4], 4, 32, 8)
    assert a[1] == b[1] and np.array_equal(a[2], b[2])
    assert a[1] != c[1]


def test_discrete_samples_on_lattice():
    # sample_discrete_test.cu:173-204: integers land in [ceil lb, floor ub]
    L = O.lib()
    for i in range(2000):
        lb, ub = -3.7 + 0.01 * i, 4.2 + 0.003 * i
        v = L.orc_sample_discrete(lb, ub, 3, i, 5, 11)
        assert v == math.floor(v)
        if math.ceil(lb) <= math.floor(ub):
            assert math.ceil(lb) <= v <= math.floor(ub)
        else:
            assert v == math.ceil(lb)
        f = L.orc_sample_discrete_f32(lb, ub, 3, i, 5, 11)
        assert f == math.floor(f)
        if math.ceil(np.float32(lb)) <= math.floor(np.float32(ub)):
            assert math.ceil(np.float32(lb)) <= f <= math.floor(np.float32(ub))
    assert L.orc_sample_discrete(2.3, 2.7, 0, 0, 0, 0) == 3.0  # no integer inside: clamps to ceil(lb)


def test_sample_hash_splitmix():
    # the SplitMix64 finaliser over the four mixed coordinates
    L = O.lib()
    M = (1 << 64) - 1

    def ref(v, i, r, s):
        x = (v * 0x9E3779B97F4A7C15) & M
        x ^= (i * 0xBF58476D1CE4E5B9) & M
        x ^= (r * 0x94D049BB133111EB) & M
        x ^= (s * 0xD6E8FEB86659FD93) & M
        x = (x + 0x9E3779B97F4A7C15) & M
        x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M
        x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M
        return x ^ (x >> 31)

    rng = np.random.default_rng(5)
    for _ in range(500):
        v, i, r, s = (int(t) for t in rng.integers(0, 1 << 40, 4))
        assert L.orc_sample_hash(v, i, r, s) == ref(v, i, r, s)


def contract_model():
    p = Problem()
    v = [p.bin_var(), p.bin_var(), p.int_var(0.0, 3.0), p.int_var(0.0, 3.0), p.var(-2.0, 2.0), p.var(-2.0, 2.0)]
    obj = (v[0] - 1.0) * (v[0] - 1.0)
    for i in range(1, 6):
        obj = obj + (v[i] - 1.0) * (v[i] - 1.0)
    p.set_objective(obj)
    p.add_constraint(v[0] + v[1], A.CMP_LE, 1.0)
    return p


def test_backend_contract_on_oracle_roles():
    # backend_contract.hpp:103-288 with the model of backend_contract_test.cu
    p = contract_model()
    op = O.OracleProblem(p)
    box = p.root_box()
    enum_kinds = [A.SLOT_BINARY_ENUMERATE] * 2 + [A.SLOT_INTEGER_ENUMERATE] * 2
    found, val, pt, idx = op.enumerate(box, enum_kinds, [0, 1, 2, 3], [2, 2, 4, 4], 64)
    assert found
    assert val == sum((x - 1.0) ** 2 for x in pt) and pt[0] + pt[1] <= 1.0
    assert all(x == round(x) for x in pt[:4])
    fe, lb = op.bound(box, enum_kinds, [0, 1, 2, 3], [2, 2, 4, 4], 64)
    assert lb[fe == 1].min() <= val + 1e-9
    found, val, pt, idx = op.sample(box, [A.SLOT_CONTINUOUS] * 2, [4, 5], [2, 2], 4, 4, 7)
    assert found and abs(val - sum((x - 1.0) ** 2 for x in pt)) < 1e-12
    assert all(box[2 * i] <= pt[i] <= box[2 * i + 1] for i in range(6))


def test_aggregate_fixture_enclosure():
    # aggregate_backend_test.cu:55-70, 208-253: enclosure at random points
    p = Problem()
    x = p.var(-2.0, 3.0)
    y = p.var(-1.0, 4.0)
    p.set_objective(x * x + y + 0.5 * (y * y) - x)
    p.add_constraint(x * x + y, A.CMP_LE, 6.0)
    op = O.OracleProblem(p)
    fe, lb = op.bound(p.root_box(), [A.SLOT_CONTINUOUS] * 2, [0, 1], [8, 8], 64)
    rng = np.random.default_rng(31415)
    for r in range(64):
        i, j = r % 8, r // 8
        xl, yl = -2.0 + 5.0 * i / 8, -1.0 + 5.0 * j / 8
        for _ in range(60):
            px, py = xl + rng.uniform(0, 5 / 8), yl + rng.uniform(0, 5 / 8)
            obj, feas = op.eval_point([px, py])
            assert lb[r] <= obj + 1e-12
            if feas:
                assert fe[r] == 1


def test_batched_search_agrees_with_reference_driver():
    # one parent per iteration and every child sampled: the batched search
    # expands boxes in the reference's order and certifies the same bounds
    for name in ("square_le5", "aggregate_fixture", "contract_model", "int_eq"):
        p = fixture_problems()[name]
        op = O.OracleProblem(p)
        ref = op.solve_reference(iter_limit=20000, bisection_budget=2, sample_points=2, threads=1)
        bat = op.solve_batched(iter_limit=20000, bisection_budget=2, sample_points=2, batch_parents=1, sample_all=1,
                               threads=1)
        tol = 1e-6 * max(1.0, abs(ref["upper_bound"]))
        assert abs(bat["upper_bound"] - ref["upper_bound"]) <= tol, name
        assert abs(bat["lower_bound"] - ref["lower_bound"]) <= tol or (
            bat["proven_optimal"] and ref["stop_reason"] == "converged"), name


def test_batched_fp32_screen_matches_fp64():
    for p in (G.qcqp_n4(),):
        op = O.OracleProblem(p)
        a = op.solve_batched(iter_limit=3000, bisection_budget=3, batch_parents=64)
        b = op.solve_batched(iter_limit=3000, bisection_budget=3, batch_parents=64, precision="fp32")
        assert a["lower_bound"] == b["lower_bound"] and a["upper_bound"] == b["upper_bound"]
        assert np.array_equal(a["best_point"], b["best_point"])
        ca, cb = a["counters"], b["counters"]
        assert ca["enqueued"] == cb["enqueued"] and ca["bounded"] == cb["bounded"]
        assert ca["pruned_infeasible"] + ca["pruned_dominated"] == cb["pruned_infeasible"] + cb["pruned_dominated"]
        assert cb["certified_fp64"] < ca["certified_fp64"]


def test_fp32_enclosure_contains_fp64():
    p = G.miqcqp_n32()
    op = O.OracleProblem(p)
    rng = np.random.default_rng(9)
    root = p.root_box().reshape(-1, 2)
    for _ in range(4):
        c = rng.uniform(root[:, 0], root[:, 1])
        w = rng.uniform(0, 1, len(c)) * (root[:, 1] - root[:, 0]) * 0.1
        box = np.stack([np.maximum(c - w, root[:, 0]), np.minimum(c + w, root[:, 1])], 1).reshape(-1)
        lo64, hi64 = op.eval_nodes(box)
        lo32, hi32 = op.eval_nodes(box, fp32=True)
        ok = ~np.isnan(lo64)
        assert np.all(lo32[ok].astype(np.float64) <= lo64[ok])
        assert np.all(hi32[ok].astype(np.float64) >= hi64[ok])


@pytest.mark.parametrize("n_vars", [4, 32, 64])
def test_hardware_rounding_bound_equals_error_free_transformations(n_vars):
    # the bench's timed CPU path (the host's FE_DOWNWARD mode, round-up as a
    # negated round-down) gives the oracle's bounds bit for bit, signs of
    # zero included
    from cuminlp_gb300 import generators as G
    p = G.BY_N[n_vars]()
    op = O.OracleProblem(p)
    box = p.root_box()
    kinds, vids, widths, _ = O.bisection_choose(box, p.var_kinds, 9)
    n = int(np.prod(widths))
    fe, lb = op.bound(box, kinds, vids, widths, n, threads=4)
    fe2, lb2 = op.bound(box, kinds, vids, widths, n, threads=4, hardware_rounding=True)
    assert np.array_equal(fe, fe2)
    assert np.array_equal(lb.view(np.uint64), lb2.view(np.uint64))
