"""Generates the golden fixtures in this directory from the reference's own
host code (oracle/_ref/ref_harness, built by oracle/build_ref.sh from the
reference sources).

Run in the container that mounts the reference:
    python tests/golden/make_golden.py
The fixtures are committed; the tests only read them.
"""

from __future__ import annotations

import json
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from cuminlp_gb300 import _abi as A  # noqa: E402
from cuminlp_gb300 import generators as G  # noqa: E402
from cuminlp_gb300.problem import Problem  # noqa: E402

HARNESS = ROOT / "oracle" / "_ref" / "ref_harness"


def hx(x: float) -> str:
    return float(x).hex()


def problem_text(p: Problem) -> str:
    nodes, lb, ub, kinds, cons = p.arrays()
    out = [str(len(nodes))]
    for nd in nodes:
        out.append(f"{nd['op']} {nd['n_in']} {nd['in0']} {nd['in1']} {nd['var_index']} {hx(nd['constant'])} "
                   f"{nd['int_exp']}")
    out.append(str(len(lb)))
    for a, b, k in zip(lb, ub, kinds):
        out.append(f"{hx(a)} {hx(b)} {k}")
    out.append(str(p.objective_root))
    out.append(str(len(cons)))
    for c in cons:
        out.append(f"{c['root']} {c['cmp']} {hx(c['rhs'])}")
    return "\n".join(out) + "\n"


def run(cmd: str, text: str) -> list[str]:
    with tempfile.TemporaryDirectory() as d:
        i, o = Path(d) / "in.txt", Path(d) / "out.txt"
        i.write_text(text)
        subprocess.run([str(HARNESS), cmd, str(i), str(o)], check=True)
        return o.read_text().splitlines()


# ---------------------------------------------------------------- decode
def decode_cases():
    rng = G.SplitMix64(7)
    cases = [
        # region/decode.hpp known answers (decode_test.cpp:48-185)
        (0, 0.0, 10.0, p, 4) for p in range(4)
    ]
    cases += [(0, 5.0, 5.0, 0, 4), (0, -3.0, 7.0, 0, 1)]
    cases += [(2, 0.0, 3.0, p, 50) for p in range(4)]
    cases += [(2, 2.4, 5.6, p, 50) for p in range(3)]
    cases += [(2, 0.0, 3.0, 10, 50), (3, 0.0, 1.0, 0, 2), (3, 0.0, 1.0, 1, 2)]
    for _ in range(400):
        kind = rng.integer(0, 3)
        lo = rng.uniform_range(-50, 50)
        hi = lo + rng.uniform_range(0, 30)
        if kind >= 2:
            lo, hi = float(int(lo)), float(int(hi))
        fan = rng.integer(1, 9)
        part = rng.integer(0, fan - 1) if kind < 2 else rng.integer(0, 12)
        cases.append((kind, lo, hi, part, fan))
    text = "".join(f"{k} {hx(a)} {hx(b)} {p} {f}\n" for k, a, b, p, f in cases)
    outs = run("decode", text)
    return [{"kind": k, "plo": hx(a), "phi": hx(b), "part": p, "fan": f,
             "lo": o.split()[0], "hi": o.split()[1]} for (k, a, b, p, f), o in zip(cases, outs)]


# ---------------------------------------------------------------- policy
def policy_cases():
    rng = G.SplitMix64(11)
    cases = []
    for t in range(300):
        n = rng.integer(1, 12)
        kinds = [rng.integer(0, 2) for _ in range(n)]
        box = []
        equal_width = rng.uniform() < 0.5  # ties are where heap order matters
        for k in kinds:
            if k == A.VAR_BINARY:
                box.append((0.0, 1.0) if rng.uniform() < 0.8 else (1.0, 1.0))
            elif k == A.VAR_INTEGER:
                a = float(rng.integer(-5, 5))
                box.append((a, a + float(rng.integer(0, 20))))
            else:
                if equal_width:
                    a = float(rng.integer(-4, 4))
                    box.append((a, a + 2.0 ** rng.integer(-2, 3)))
                else:
                    a = rng.uniform_range(-10, 10)
                    box.append((a, a + rng.uniform_range(0, 8)))
        cases.append(("B", rng.integer(1, 9), rng.integer(0, 8) if t % 4 == 0 else 0,
                      rng.integer(0, 10) if t % 5 == 0 else 0, int(t % 2), kinds, box))
    lines = []
    for c in cases:
        if c[0] == "B":
            _, B, mc, ec, rel, kinds, box = c
            head = f"B {B} {mc} {ec} {rel} {len(kinds)}"
        else:
            _, pn, ecap, mc, kinds, box = c
            head = f"G {pn} {ecap} {mc} {len(kinds)}"
        body = " ".join(str(k) for k in kinds) + " " + " ".join(f"{hx(a)} {hx(b)}" for a, b in box)
        lines.append(head + " " + body + "\n")
    outs = run("policy", "".join(lines))
    res = []
    for c, o in zip(cases, outs):
        v = [int(x) for x in o.split()]
        cnt = v[0]
        slots = [v[1 + 4 * j:5 + 4 * j] for j in range(cnt)]
        d = {"tag": c[0], "kinds": c[-2], "box": [[hx(a), hx(b)] for a, b in c[-1]], "slots": slots}
        if c[0] == "B":
            d.update(B=c[1], max_cycle=c[2], enumerate_cap=c[3], relative=c[4])
        else:
            d.update(partition_num=c[1], enumerate_cap=c[2], max_cycle=c[3])
        res.append(d)
    return res


# ---------------------------------------------------------------- driver
def fixture_problems():
    """Small problems from the reference's own tests plus seeded QCQPs."""
    out = {}
    # graph_replay_test.cu:77-84: x in [0,10], x^2, x <= 5
    p = Problem()
    x = p.var(0.0, 10.0)
    p.set_objective(x * x)
    p.add_constraint(x, A.CMP_LE, 5.0)
    out["square_le5"] = p
    # graph_replay_test.cu:87-94: infeasible everywhere
    p = Problem()
    x = p.var(0.0, 10.0)
    p.set_objective(x * x)
    p.add_constraint(x, A.CMP_LE, -100.0)
    out["infeasible"] = p
    # aggregate_backend_test.cu:55-70
    p = Problem()
    x = p.var(-2.0, 3.0)
    y = p.var(-1.0, 4.0)
    p.set_objective(x * x + y + 0.5 * (y * y) - x)
    p.add_constraint(x * x + y, A.CMP_LE, 6.0)
    out["aggregate_fixture"] = p
    # backend_contract_test.cu:32-50
    p = Problem()
    v = [p.bin_var(), p.bin_var(), p.int_var(0.0, 3.0), p.int_var(0.0, 3.0), p.var(-2.0, 2.0), p.var(-2.0, 2.0)]
    obj = (v[0] - 1.0) * (v[0] - 1.0)
    for i in range(1, 6):
        obj = obj + (v[i] - 1.0) * (v[i] - 1.0)
    p.set_objective(obj)
    p.add_constraint(v[0] + v[1], A.CMP_LE, 1.0)
    out["contract_model"] = p
    # an equality-constrained integer problem (enumeration + EQ predicate)
    p = Problem()
    a, b, c = p.int_var(0.0, 5.0), p.int_var(0.0, 5.0), p.var(-1.0, 1.0)
    p.set_objective(a * b - 3.0 * a + c * c)
    p.add_constraint(a + b, A.CMP_EQ, 5.0)
    out["int_eq"] = p
    for i in range(3):
        out[f"qcqp_n4_{i}"] = G.qcqp_n4(i)
    out["miqcqp_n6"] = G.qcqp(G.QCQPSpec(n=6, m=2, n_int=2, int_lb=0, int_ub=3, cont_lb=-2, cont_ub=2,
                                         rhs=(1.0, 4.0)), G.seed_for(9, 0))
    return out


DRIVER_RUNS = [
    ("square_le5", 400, 2, 4), ("infeasible", 200, 2, 4), ("aggregate_fixture", 600, 2, 2),
    ("contract_model", 800, 3, 2), ("int_eq", 600, 3, 3), ("qcqp_n4_0", 1500, 2, 1), ("qcqp_n4_1", 1500, 3, 2),
    ("qcqp_n4_2", 1200, 1, 1), ("miqcqp_n6", 1000, 3, 1),
]


def driver_cases(problems):
    res = []
    for name, iters, B, S in DRIVER_RUNS:
        text = f"{iters} {B} {S} {hx(1e-6)}\n" + problem_text(problems[name])
        lines = run("driver", text)
        h = lines[0].split()
        c = [int(x) for x in lines[1].split()]
        bp = lines[2].split()
        res.append({
            "problem": name, "iter_limit": iters, "B": B, "samples": S,
            "lower_bound": h[0], "upper_bound": h[1], "stop_reason": h[2], "proven_optimal": int(h[3]),
            "infeasible": int(h[4]),
            "counters": dict(zip(["iterations", "fathomed", "fathomed_points", "bounded", "sampled", "enqueued",
                                  "witness_rejected", "pruned_duplicate", "pruned_infeasible", "pruned_dominated",
                                  "pending", "viable"], c)),
            "best_point": bp[1:],
        })
    return res


# (problem, policy, iter_limit, B, partition_num, enumerate_cap, max_cycle,
# samples): policies as make_policy builds them (policy/greedy_enum.hpp:204)
POLICY_RUNS = [
    ("contract_model", "G", 600, 0, 2, 4, 3, 2), ("int_eq", "G", 400, 0, 2, 6, 3, 2),
    ("qcqp_n4_0", "G", 1500, 0, 2, 2, 2, 1), ("miqcqp_n6", "G", 800, 0, 2, 4, 3, 1),
    ("qcqp_n4_1", "W", 1500, 0, 3, 2, 2, 2), ("aggregate_fixture", "W", 600, 0, 2, 2, 2, 2),
    ("contract_model", "W", 600, 0, 2, 3, 4, 1),
    ("square_le5", "R", 400, 2, 2, 1, 0, 4), ("miqcqp_n6", "R", 800, 3, 2, 1, 0, 1),
]


def policy_header(run_: tuple) -> str:
    _, pk, iters, B, pn, ecap, mc, S = run_
    return f"{pk} {iters} {B} {pn} {ecap} {mc} {S} {hx(1e-6)}\n"


def driver_policy_cases(problems):
    """The reference SearchDriver with GreedyEnum, WidthFirst and relative
    BisectionBudget (the oracle behind its roles)."""
    res = []
    for r in POLICY_RUNS:
        lines = run("driverp", policy_header(r) + problem_text(problems[r[0]]))
        h = lines[0].split()
        res.append({
            "problem": r[0], "policy": r[1], "iter_limit": r[2], "B": r[3], "partition_num": r[4],
            "enumerate_cap": r[5], "max_cycle": r[6], "samples": r[7],
            "lower_bound": h[0], "upper_bound": h[1], "stop_reason": h[2], "proven_optimal": int(h[3]),
            "infeasible": int(h[4]), "counters": [int(x) for x in lines[1].split()],
            "best_point": lines[2].split()[1:],
        })
    return res


AGG_CASES = (("square_le5", 300), ("infeasible", 50), ("aggregate_fixture", 400), ("int_eq", 100),
             ("miqcqp_n6", 300), ("qcqp_n4_1", 600))


def aggdriver_cases(problems):
    """The reference AggregateDriver (WidestBranchPolicy k=2, N=16, sampler
    N=8 with 2 points) with the oracle behind its roles, per selection rule."""
    res = []
    for name, iters in AGG_CASES:
        for rule in ("least-lower-bound", "reject-index", "reject-index-stale"):
            head = f"{iters} 2 16 8 2 {rule} {hx(1e-6)}\n"
            out = run("aggdriver", head + problem_text(problems[name]))
            f0 = out[0].split()
            res.append({"problem": name, "iter_limit": iters, "k": 2, "N": 16, "Ns": 8, "samples": 2, "rule": rule,
                        "lower_bound": f0[0], "upper_bound": f0[1], "stop_reason": f0[2], "proven_optimal": int(f0[3]),
                        "infeasible": int(f0[4]), "selection_rule_engaged": int(f0[5]),
                        "counters": [int(x) for x in out[1].split()], "best_point": out[2].split()[1:]})
    return res


def gams_cases():
    """The reference frontend's lowering of this repository's own .gms
    models (tests/data/gams), as oracle/_ref/ref_gams prints it."""
    out = {}
    for f in sorted((ROOT / "tests" / "data" / "gams").glob("*.gms")):
        res = subprocess.run([str(ROOT / "oracle" / "_ref" / "ref_gams"), str(f)], capture_output=True, text=True,
                             check=True)
        out[f.name] = res.stdout.splitlines()
    return out


def main():
    if not HARNESS.exists():
        raise SystemExit("oracle/_ref/ref_harness missing: run oracle/build_ref.sh first")
    (HERE / "decode.json").write_text(json.dumps(decode_cases(), indent=0))
    (HERE / "policy.json").write_text(json.dumps(policy_cases(), indent=0))
    (HERE / "driver.json").write_text(json.dumps(driver_cases(fixture_problems()), indent=1))
    (HERE / "driver_policies.json").write_text(json.dumps(driver_policy_cases(fixture_problems()), indent=1))
    (HERE / "gams.json").write_text(json.dumps(gams_cases(), indent=1))
    (HERE / "aggdriver.json").write_text(json.dumps(aggdriver_cases(fixture_problems()), indent=1))
    print("golden fixtures written")


if __name__ == "__main__":
    main()
