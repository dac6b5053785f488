"""The reference's own code on the GPU beside this library.

oracle/_ref/ref_gpu (oracle/ref_gpu.cu) is compiled from the reference's
headers, as oracle/amalgamate.py writes them, and links libcuminlp_gb300.so
through the adapter include/cuminlp_gb300/region_backend.hpp.  These tests:

- run the reference's SearchDriver (search/driver.hpp:137-537) over this
  library's roles -- the drop-in -- with BisectionBudget, and with
  GreedyEnum, WidthFirst and relative BisectionBudget as make_policy builds
  them (policy/greedy_enum.hpp:204-223), and require the golden runs of the
  same driver over the oracle bit for bit: bounds, stop reason, claims,
  counters and the best point;
- run the same driver over the CPU oracle's roles on all host cores with the
  host's directed rounding (the "oracle" backend the bench times) and
  require the same golden runs;
- run the same driver over the reference's own CUDA graph backend
  (backend/graph/*, with the build's interval operators standing in for the
  missing cuinterval) and require the same golden runs: this pins the
  oracle's sampler and decode, which the goldens put behind the driver, to
  the reference's device code (graph/subregion_sampler.cuh:53-199);
- compare the bounder and sampler roles of both backends on the same
  compositions of configs 1-3, bit for bit.
"""

from __future__ import annotations

import json
import subprocess
import tempfile
from pathlib import Path

import pytest

from cuminlp_gb300 import generators as G
from tests.golden.make_golden import POLICY_RUNS, fixture_problems, hx, policy_header, problem_text

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
EXE = ROOT / "oracle" / "_ref" / "ref_gpu"
COUNTERS = ["iterations", "fathomed", "fathomed_points", "bounded", "sampled", "enqueued", "witness_rejected",
            "pruned_duplicate", "pruned_infeasible", "pruned_dominated", "pending", "viable"]


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


def run_harness(args: list[str], text: str) -> list[str]:
    with tempfile.TemporaryDirectory() as d:
        i, o = Path(d) / "in.txt", Path(d) / "out.txt"
        i.write_text(text)
        proc = subprocess.run([str(EXE), *args, str(i), str(o)], capture_output=True, text=True, timeout=900)
        assert proc.returncode == 0, proc.stderr
        return o.read_text().splitlines()


def check_run(lines: list[str], want: dict, counters) -> None:
    h = lines[0].split()
    assert h[0] == want["lower_bound"] and h[1] == want["upper_bound"]
    assert h[2] == want["stop_reason"]
    assert int(h[3]) == want["proven_optimal"] and int(h[4]) == want["infeasible"]
    got = [int(x) for x in lines[1].split()]
    assert got == counters
    assert lines[2].split()[1:] == want["best_point"]


def driver_runs():
    return json.loads((GOLDEN / "driver.json").read_text())


@pytest.mark.parametrize("backend", ["gb300", "graph", "oracle"])
@pytest.mark.parametrize("idx", range(9))
def test_reference_driver_bisection(backend, idx):
    want = driver_runs()[idx]
    p = fixture_problems()[want["problem"]]
    head = f"B {want['iter_limit']} {want['B']} 2 1 0 {want['samples']} {hx(1e-6)}\n"
    lines = run_harness(["driver", backend], head + problem_text(p))
    check_run(lines, want, [want["counters"][k] for k in COUNTERS])


@pytest.mark.parametrize("backend", ["gb300", "graph", "oracle"])
@pytest.mark.parametrize("idx", range(len(POLICY_RUNS)))
def test_reference_driver_policies(backend, idx):
    want = json.loads((GOLDEN / "driver_policies.json").read_text())[idx]
    run_ = POLICY_RUNS[idx]
    assert want["problem"] == run_[0] and want["policy"] == run_[1]
    lines = run_harness(["driver", backend], policy_header(run_) + problem_text(fixture_problems()[run_[0]]))
    check_run(lines, want, want["counters"])


def roles(problem, B: int, samples: int, n_salts: int, which: str = "bs", frac: float = 1.0) -> dict:
    lines = run_harness(["roles"], f"{B} {samples} 3 {n_salts} {which} {hx(frac)}\n" + problem_text(problem))
    out = {}
    for ln in lines:
        k, _, v = ln.partition(" ")
        out.setdefault(k, []).append(v)
    return out


@pytest.mark.parametrize("n_vars,B,S,frac", [(4, 10, 4, 1.0), (32, 12, 2, 1.0), (32, 12, 2, 0.05), (64, 10, 1, 1.0),
                                             (64, 12, 2, 0.02)])
def test_roles_match_reference_graph_backend(n_vars, B, S, frac):
    # the root boxes of the n=32 and n=64 MIQCQPs hold no feasible sample;
    # the small boxes around the origin do, so the witnesses are compared there
    r = roles(G.BY_N[n_vars](), B, S, 4, frac=frac)
    assert int(r["n_regions"][0]) == 1 << B
    assert int(r["bound_mismatch_feasible"][0]) == 0
    assert int(r["bound_mismatch_lb"][0]) == 0
    assert int(r["sample_mismatch"][0]) == 0
    if frac < 1.0:
        assert int(r["sample_found"][0]) == 4
