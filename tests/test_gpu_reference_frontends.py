"""The reference's host-side callers of the hot path, unchanged, over this
library's C ABI on the GPU (oracle/_ref/ref_gpu):

- its AggregateDriver (aggregate/driver.hpp:137-420) over the aggregate
  roles of include/cuminlp_gb300/aggregate_backend.hpp (cmn_bound_children,
  cmn_sample) must reproduce the golden runs of the same driver over the
  oracle's roles (tests/golden/aggdriver.json) bit for bit;
- its GAMS frontend (source/gams/frontend.cpp) lowers a model and the
  lowered Problem crosses the C ABI into the library's solver: the
  lowering of this repository's own models must equal the golden lowering
  (tests/golden/gams.json), and the device solve of every lowered model
  whose operators the oracle bounds must equal the oracle's batched solve
  bit for bit.  The reference's own test models (test/data/gams, copied to
  oracle/_ref/gams by oracle/build_ref.sh) run through the same path.
"""

from __future__ import annotations

import json
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import _abi as A
from cuminlp_gb300.problem import Constraint, Problem
from tests.conftest import bits_equal
from tests.golden.make_golden import AGG_CASES, fixture_problems, hx, problem_text

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
EXE = ROOT / "oracle" / "_ref" / "ref_gpu"
OWN_MODELS = ROOT / "tests" / "data" / "gams"
REF_MODELS = ROOT / "oracle" / "_ref" / "gams"
KINDS = ["syntax", "non_scalar", "discrete", "unsupported_function", "unrepresentable", "io"]
# operators the oracle bounds (oracle.c op_supported_interval)
ORACLE_OPS = {A.OP_VAR, A.OP_CONST, A.OP_ADD, A.OP_SUB, A.OP_MUL, A.OP_DIV, A.OP_SQR, A.OP_NEG, A.OP_SQRT,
              A.OP_POWN, A.OP_ABS, A.OP_MIN, A.OP_MAX}
SOLVE = dict(iter_limit=4000, bisection_budget=3, batch_parents=64)


@pytest.fixture(scope="module", autouse=True)
def _harness():
    from cuminlp_gb300 import build
    from oracle import build as ob
    if not ob.available():
        pytest.skip("oracle/_ref/cuminlp_ref_gpu.cuh is absent (written by oracle/build_ref.sh where the "
                    "reference tree is mounted)")
    lib = build.build_library()
    ob.compile_ref_gpu()
    ob.link_ref_gpu(lib)


def run_harness(args: list, text: str | None = None) -> list:
    with tempfile.TemporaryDirectory() as d:
        o = Path(d) / "out.txt"
        if text is not None:
            i = Path(d) / "in.txt"
            i.write_text(text)
            argv = [str(EXE), *args, str(i), str(o)]
        else:
            argv = [str(EXE), args[0], args[1], str(o), *args[2:]]
        proc = subprocess.run(argv, capture_output=True, text=True, timeout=900)
        assert proc.returncode == 0, proc.stderr
        return o.read_text().splitlines()


# ------------------------------------------------------------ aggregate
@pytest.mark.parametrize("idx", range(len(AGG_CASES) * 3))
def test_reference_aggregate_driver_over_device_roles(idx):
    want = json.loads((GOLDEN / "aggdriver.json").read_text())[idx]
    p = fixture_problems()[want["problem"]]
    head = (f"{want['iter_limit']} {want['k']} {want['N']} {want['Ns']} {want['samples']} {want['rule']} "
            f"{hx(1e-6)}\n")
    lines = run_harness(["aggdriver"], head + problem_text(p))
    f0 = lines[0].split()
    assert f0[0] == want["lower_bound"] and f0[1] == want["upper_bound"]
    assert f0[2] == want["stop_reason"]
    assert int(f0[3]) == want["proven_optimal"] and int(f0[4]) == want["infeasible"]
    assert int(f0[5]) == want["selection_rule_engaged"]
    assert [int(x) for x in lines[1].split()] == want["counters"]
    assert lines[2].split()[1:] == want["best_point"]


# ------------------------------------------------------------ GAMS
def parse_lowering(out: list) -> dict:
    """The lowering records the harness prints (oracle/ref_gams.cpp's
    format) plus the solve record."""
    head = out[0].split()
    if head[0] == "err":
        return {"error": KINDS[int(head[1])], "line": int(head[2])}
    r = {"sense": head[1], "objvar_kept": bool(int(head[2])), "n_warnings": int(head[6]), "nodes": [], "vars": [],
         "cons": []}
    for line in out[1:]:
        f = line.split()
        if f[0] == "node":
            r["nodes"].append((int(f[1]), int(f[2]), int(f[3]), int(f[4]), float.fromhex(f[5]), int(f[6]), int(f[7])))
        elif f[0] == "var":
            r["vars"].append((float.fromhex(f[1]), float.fromhex(f[2]), int(f[3]), f[4]))
        elif f[0] == "obj":
            r["obj"] = int(f[1])
        elif f[0] == "con":
            r["cons"].append((int(f[1]), int(f[2]), float.fromhex(f[3]), f[4]))
        elif f[0] == "solve":
            r["solve"] = {"lower_bound": float.fromhex(f[1]), "upper_bound": float.fromhex(f[2]),
                          "stop_reason": int(f[3]), "proven_optimal": int(f[4]), "infeasible": int(f[5]),
                          "iterations": int(f[6]), "expansions": int(f[7]), "bounded": int(f[8])}
        elif f[0] == "solve_error":
            r["solve_error"] = (int(f[1]), " ".join(f[2:]))
    return r


def problem_of(r: dict) -> Problem:
    """The lowered Problem, rebuilt node for node."""
    p = Problem()
    for op, n_in, in0, in1, c, vi, ie in r["nodes"]:
        p.graph.emit(op, tuple(x for x in (in0, in1)[:n_in]), constant=c, var_index=vi, int_exp=ie)
    for lb, ub, k, _ in r["vars"]:
        p.box_bounds.append((lb, ub))
        p.var_kinds.append(k)
    p.objective_root = r["obj"]
    p.constraints = [Constraint(root, cmp, rhs) for root, cmp, rhs, _ in r["cons"]]
    return p


def gams(path: Path) -> dict:
    return parse_lowering(run_harness(["gams", str(path), str(SOLVE["iter_limit"]), str(SOLVE["bisection_budget"]),
                                       str(SOLVE["batch_parents"])]))


def check_against_oracle(r: dict) -> None:
    ops = {n[0] for n in r["nodes"]}
    if not ops <= ORACLE_OPS:
        return
    assert "solve" in r, r.get("solve_error")
    o = O.OracleProblem(problem_of(r)).solve_batched(frontier_cap=1 << 20, **SOLVE)
    g = r["solve"]
    assert bits_equal(np.float64(g["lower_bound"]), np.float64(o["lower_bound"]))
    assert bits_equal(np.float64(g["upper_bound"]), np.float64(o["upper_bound"]))
    assert g["proven_optimal"] == o["proven_optimal"] and g["infeasible"] == o["infeasible"]
    assert g["expansions"] == o["counters"]["expansions"] and g["bounded"] == o["counters"]["bounded"]


@pytest.mark.parametrize("name", sorted(p.name for p in OWN_MODELS.glob("*.gms")))
def test_own_models_lower_as_golden_and_solve_like_the_oracle(name):
    golden = parse_lowering(json.loads((GOLDEN / "gams.json").read_text())[name])
    r = gams(OWN_MODELS / name)
    for k in ("error", "line", "sense", "objvar_kept", "n_warnings", "obj", "vars", "cons"):
        assert r.get(k) == golden.get(k), k
    if "error" in r:
        return
    assert len(r["nodes"]) == len(golden["nodes"])
    for a, b in zip(r["nodes"], golden["nodes"]):
        assert a[:4] == b[:4] and a[5:] == b[5:]
        assert np.float64(a[4]).tobytes() == np.float64(b[4]).tobytes()
    check_against_oracle(r)


def ref_models():
    return sorted(p.name for p in REF_MODELS.glob("*.gms")) if REF_MODELS.is_dir() else []


@pytest.mark.parametrize("name", ref_models())
def test_reference_models_through_the_c_abi(name):
    r = gams(REF_MODELS / name)
    assert "error" not in r, r
    if "solve_error" in r:  # an operator without an interval form on the device
        ops = {n[0] for n in r["nodes"]}
        assert not ops <= ORACLE_OPS, r["solve_error"]
        pytest.skip(f"{name}: {r['solve_error'][1]}")
    s = r["solve"]
    assert s["lower_bound"] <= s["upper_bound"]
    check_against_oracle(r)
