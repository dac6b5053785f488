"""CPU: the GAMS scalar-format frontend against the reference's own frontend
(source/gams/frontend.cpp, compiled from the reference sources into
oracle/_ref/ref_gams): the lowered Problem must be node for node the same --
ops, operands, constants to the bit, variable boxes, kinds and names,
constraints, sense and warnings -- or the same rejection (kind and line)."""

from __future__ import annotations

import json
import math
import os
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import gams
from tests.gams_ref import REF_GAMS, our_lowering, parse_lowering, reference_lowering

HERE = Path(__file__).resolve().parent
DATA = HERE / "data" / "gams"
REF_DATA = Path(os.environ["CMN_REFERENCE"]) / "test" / "data" / "gams" if os.environ.get("CMN_REFERENCE") else None


def same(r: dict, o: dict):
    if "error" in r or "error" in o:
        assert r == o
        return
    for k in ("sense", "objvar_kept", "n_warnings", "obj", "vars", "cons"):
        assert r[k] == o[k], k
    assert len(r["nodes"]) == len(o["nodes"])
    for i, (a, b) in enumerate(zip(r["nodes"], o["nodes"])):
        assert a[:4] == b[:4] and a[5:] == b[5:], i
        assert math.copysign(1, a[4]) == math.copysign(1, b[4]) and (a[4] == b[4] or (a[4] != a[4] and b[4] != b[4]))


def test_own_models_match_reference_golden():
    golden = json.loads((HERE / "golden" / "gams.json").read_text())
    assert set(golden) == {p.name for p in DATA.glob("*.gms")}
    for name, lines in golden.items():
        same(parse_lowering(lines), our_lowering(DATA / name))


@pytest.mark.skipif(REF_DATA is None or not (REF_GAMS.exists() and REF_DATA.exists()),
                    reason="CMN_REFERENCE unset or the reference frontend not built here")
def test_reference_corpus_lowers_identically():
    files = sorted(REF_DATA.glob("*.gms"))
    assert files
    for f in files:
        same(reference_lowering(f), our_lowering(f))


def test_rejections():
    for name, kind in (("indexed.gms", "non_scalar"), ("unsupported.gms", "unsupported_function")):
        with pytest.raises(gams.ParseError) as e:
            gams.parse_file(DATA / name)
        assert e.value.kind == kind
    with pytest.raises(gams.ParseError) as e:
        gams.parse("Variables x, o; Equations e; e.. o =E= y; Model m /all/; Solve m using nlp minimizing o;")
    assert "undeclared identifier" in str(e.value)
    with pytest.raises(gams.ParseError) as e:
        gams.parse("Variables x; Equations e; e.. x =L= 1;")
    assert e.value.kind == "unrepresentable"


def test_semantics_of_a_maximisation():
    pm = gams.parse_file(DATA / "bilinear_max.gms")
    assert pm.sense == "max" and pm.var_names == ["x", "y", "z"] and pm.constraint_names == ["cap", "pair"]
    op = O.OracleProblem(pm.problem)
    for x, y, z in ((1.0, 2.0, 1.0), (0.5, 0.25, 2.0), (3.0, 1.5, 0.0)):
        obj, feas = op.eval_point(np.array([x, y, z]))
        want = -(3 * x * y - (x - 1) ** 2 + 2 * z - 0.5 * y * y)  # the solver minimises the negation
        assert abs(obj - want) <= 1e-12 * max(1.0, abs(want))
        assert feas == ((x + 2 * y + z <= 6) and (x * y >= 0.5))
