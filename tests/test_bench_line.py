"""bench.py's JSON line, assembled on CPU: every device leg is replaced by a
stub of the same return shape, and the line must carry every key of the
bench contract (metric, value, roofline, cpu_baseline, e2e, gpu_launches,
clocks ...) with the whole-job numbers computed from the legs' counts."""

from __future__ import annotations

import io
import json
import sys
from contextlib import redirect_stdout
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402
from cuminlp_gb300 import generators as G  # noqa: E402
from cuminlp_gb300 import solver as S  # noqa: E402


class _Cudart:
    def set_device(self, d):
        pass


class _Clocks:
    def __init__(self, gpu):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        pass

    def summary(self):
        return {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "power_w_max": 300.0, "samples": 5, "reasons": []}


class _DeviceProblem:
    def __init__(self, problem, **kw):
        self.n_vars = problem.n_vars

    def autotune(self, precision, n_boxes):
        return {"blocks_per_sm": 5, "lanes_cap": 1, "ms_best": 1.0, "ms_default": 1.0, "candidates": 30}

    def info(self):
        return {"n_nodes": 10819, "buffer_node_count": 7982, "program_length": 2854, "program_slots": 0,
                "flops_per_box": 28930.0, "bytes_per_box": 529.0}


def _solver_run(dp, rt, precision, steps, warmup, **kw):
    return {"ms": 60.0 * steps, "wall_ms": 61.0 * steps,
            "delta": {"bounded": (1 << 20) * steps, "screened_fp32": 0, "certified_fp64": (1 << 20) * steps,
                      "expansions": (1 << 16) * steps, "sampled": (1 << 20) * steps},
            "phases": [[0.1, 43.0, 17.0, 0.8, 60.0]] * steps, "kernels_per_iter": 42,
            "lazy_phases": [[20.0, 43.0]] * steps if precision == "lazy" else [],
            "outcome": {"lower_bound": -1.0, "upper_bound": 1.0, "frontier_size": 1 << 20}}


def _e2e_run(dp, problem, steps, warmup):
    return {"value": 16e6, "unit": "boxes/s", "h2d_bytes_per_step": 6176, "d2h_bytes_per_step": 9437464,
            "regions_per_call": 1 << 20, "ms_per_step": 65.0, "units": (1 << 20) * steps, "ms": 65.0 * steps}


@pytest.fixture
def stubbed(monkeypatch):
    monkeypatch.setattr(bench, "Cudart", _Cudart)
    monkeypatch.setattr(bench, "Clocks", _Clocks)
    monkeypatch.setattr(bench, "fma_peak", lambda precision: 1.04 if precision == 0 else 70.0)
    monkeypatch.setattr(bench, "solver_run", _solver_run)
    monkeypatch.setattr(bench, "e2e_run", _e2e_run)
    monkeypatch.setattr(bench, "cpu_rate", lambda problem, seconds, threads: (75e3, {
        "children_per_step": 1024, "steps": 10, "seconds": 0.1}))
    monkeypatch.setattr(bench, "time_to_gap", lambda *a, **k: {"seconds": 0.165, "proven": True})
    monkeypatch.setattr(bench, "batch_run", lambda *a, **k: {"value": 9e6})
    monkeypatch.setattr(bench, "serving_run", lambda *a, **k: {"latency_p99_ms": 1.0})
    monkeypatch.setattr(bench, "screen_check_run", lambda *a, **k: {"point_containment": []})
    monkeypatch.setattr(bench, "miqcqp_n32_run", lambda *a, **k: {"plain_fp64": {"value": 17e6}})
    monkeypatch.setattr(bench, "reference_gpu_run", lambda *a, **k: {"miqcqp_n64_bound": {"speedup": 2.0}})
    monkeypatch.setattr(S, "DeviceProblem", _DeviceProblem)
    small = G.qcqp_n4(0)
    monkeypatch.setattr(G, "serving_qcqp", lambda i: small)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)


def _line(monkeypatch, argv):
    monkeypatch.setattr(sys, "argv", ["bench.py"] + argv)
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_ours(bench.parse_args())
    lines = [ln for ln in buf.getvalue().splitlines() if ln.strip()]
    assert len(lines) == 1
    return json.loads(lines[0])


def test_default_line_carries_the_contract(stubbed, monkeypatch):
    d = _line(monkeypatch, ["--steps", "5", "--warmup", "3"])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "roofline", "cpu_baseline", "e2e", "gpu_launches", "clocks"):
        assert k in d, k
    assert d["n_gpus"] == 1 and d["steps"] == 5 and d["warmup"] == 3 and d["higher_is_better"] is True
    assert d["value"] == pytest.approx(5 * (1 << 20) / (0.3))  # boxes over the timed region
    assert d["ms_per_step"] == pytest.approx(60.0)
    assert "workload" in d["config"]
    r = d["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic", "phase"):
        assert k in r, k
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    # the stub's longest phase is the FP32 bound (43 ms of 60; the FP64 verdict beside it 20 ms)
    assert r["phase"] == "bound" and r["achieved"] == pytest.approx((1 << 20) * 28930.0 / 43e-3 / 1e12)
    assert set(d["phase_rooflines"]) == {"certify", "bound", "sample"}
    # every phase carries its DRAM traffic per launch from the ncu capture
    certify = d["phase_rooflines"]["certify"]
    assert certify["traffic"] == pytest.approx(bench.VERDICT_DRAM_BYTES_PER_BOX * (1 << 16))
    assert all(v["traffic"] > 0 for v in d["phase_rooflines"].values())
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == 75e3 and cb["sample"]
    e = d["e2e"]
    assert set(e) == {"value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"}
    assert e["value"] == pytest.approx(5 * (1 << 20) / 0.325)
    assert d["gpu_launches"] == 42 * 5
    assert d["clocks"]["sm_mhz"] == 2070.0 and d["clocks"]["reasons"] == []
    for k in ("time_to_gap", "batch_uneven", "serving", "fp32_screen_check", "miqcqp_n32_solver", "reference_gpu"):
        assert d[k] is not None, k
    for k in ("plain_fp64", "lazy", "fp32_screen_fp64_certify", "roofline_plain_fp64"):
        assert k in d, k


def test_skip_flags_leave_the_extra_legs_empty(stubbed, monkeypatch):
    d = _line(monkeypatch, ["--no-ttg", "--no-batch", "--no-serve", "--no-screen-check", "--no-n32",
                            "--no-reference-gpu"])
    for k in ("time_to_gap", "batch_uneven", "serving", "fp32_screen_check", "miqcqp_n32_solver", "reference_gpu"):
        assert d[k] is None, k
    assert d["e2e"]["value"] > 0


def test_quick_line(stubbed, monkeypatch):
    d = _line(monkeypatch, ["--quick", "--steps", "2", "--warmup", "1"])
    assert d["quick"] is True and d["lazy_boxes/s"] == pytest.approx(2 * (1 << 20) / 0.12)
    assert {"fp64_ms", "lazy_ms", "fp32_ms"} <= set(d)


def test_a_failing_extra_leg_is_recorded_not_fatal(stubbed, monkeypatch):
    def boom(*a, **k):
        raise RuntimeError("out of device memory")

    monkeypatch.setattr(bench, "miqcqp_n32_run", boom)
    monkeypatch.setattr(bench, "batch_run", boom)
    d = _line(monkeypatch, ["--steps", "2", "--warmup", "1"])
    assert d["miqcqp_n32_solver"] == {"error": "RuntimeError: out of device memory"}
    assert d["batch_uneven"] == {"error": "RuntimeError: out of device memory"}
    assert d["value"] > 0 and d["e2e"]["value"] > 0
    sv = d["serving"]
    assert sv["workload"] == bench.serving_workload() and sv["runs"] == [{"latency_p99_ms": 1.0}] * 3
    assert sv["time_to_gap_run"]["latency_p99_ms"] == 1.0 and "n=4" in sv["time_to_gap_run"]["workload"]
