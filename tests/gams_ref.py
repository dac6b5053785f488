"""Helpers of the GAMS frontend parity tests: run the reference frontend
(oracle/_ref/ref_gams, built from the reference sources) and compare its
lowered Problem with this frontend's, node for node."""

from __future__ import annotations

import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
REF_GAMS = ROOT / "oracle" / "_ref" / "ref_gams"
KINDS = ["syntax", "non_scalar", "discrete", "unsupported_function", "unrepresentable", "io"]


def reference_lowering(path) -> dict:
    out = subprocess.run([str(REF_GAMS), str(path)], capture_output=True, text=True, check=True).stdout.splitlines()
    return parse_lowering(out)


def parse_lowering(out: list) -> dict:
    """The records ref_gams prints (see oracle/ref_gams.cpp) as a dict."""
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
    return r


def our_lowering(path) -> dict:
    from cuminlp_gb300 import gams
    try:
        pm = gams.parse_file(path)
    except gams.ParseError as e:
        return {"error": e.kind, "line": e.line}
    p = pm.problem
    nodes = []
    for nd in p.graph.nodes:
        ins = list(nd.inputs) + [-1, -1]
        nodes.append((nd.op, len(nd.inputs), ins[0], ins[1], nd.constant if nd.op == 1 else 0.0,
                      nd.var_index if nd.op == 0 else 0, nd.int_exp if nd.op == 14 else 0))
    vars_ = [(lb, ub, k, name) for (lb, ub), k, name in zip(p.box_bounds, p.var_kinds, pm.var_names)]
    cons = [(c.root_id, c.cmp, c.rhs, name) for c, name in zip(p.constraints, pm.constraint_names)]
    return {"sense": pm.sense, "objvar_kept": pm.objvar_kept, "n_warnings": len(pm.warnings), "nodes": nodes,
            "vars": vars_, "obj": p.objective_root, "cons": cons}
