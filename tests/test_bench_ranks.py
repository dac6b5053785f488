"""The N>1 path of bench.py on CPU: two gloo ranks on 127.0.0.1.

The solver runs as independent replicas, one instance per GPU, with no
collective on the data path; the only cross-rank steps are the barriers
around the timed region and the reduction of the per-rank counts and
times. These tests run those steps as two processes (spawned, no GPU):
the whole-job rate is the units all ranks processed over the slowest
rank's time, and the reference arm prints one line, from rank 0 only."""

from __future__ import annotations

import io
import json
import os
import socket
import sys
from contextlib import redirect_stdout
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank: int, world: int, port: int):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})


def _rate_rank(rank: int, world: int, port: int, out: str):
    sys.path.insert(0, str(ROOT))
    import bench
    _env(rank, world, port)
    _, r, _, dist = bench.dist_setup(None)
    try:
        bench.barrier(dist)
        # rank r processed (r + 1) * 1000 units in (r + 1) * 10 ms
        value, t_max = bench.job_rate(dist, (r + 1) * 1000.0, (r + 1) * 10.0)
        bench.barrier(dist)
        Path(out, f"rate{r}.json").write_text(json.dumps({"value": value, "t_max": t_max}))
    finally:
        dist.destroy_process_group()


def _reference_rank(rank: int, world: int, port: int, out: str):
    sys.path.insert(0, str(ROOT))
    import bench
    _env(rank, world, port)

    def fast_rate(problem, seconds, threads):
        return 1234.5, {"children_per_step": 8, "steps": 1, "seconds": 0.0}

    bench.cpu_rate = fast_rate  # the host sampler is timed elsewhere
    sys.argv = ["bench.py", "--impl", "reference", "--gpus", str(world), "--steps", "2", "--warmup", "1"]
    args = bench.parse_args()
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(args)
    import torch.distributed as dist
    if dist.is_initialized():
        dist.destroy_process_group()
    Path(out, f"ref{rank}.txt").write_text(buf.getvalue())


def _spawn(fn, world: int, out: Path):
    import torch.multiprocessing as mp
    mp.start_processes(fn, args=(world, _free_port(), str(out)), nprocs=world, join=True, start_method="spawn")


def test_job_rate_sums_units_over_slowest_rank(tmp_path):
    pytest.importorskip("torch.distributed")
    _spawn(_rate_rank, 2, tmp_path)
    for r in range(2):
        got = json.loads((tmp_path / f"rate{r}.json").read_text())
        assert got["t_max"] == 20.0
        assert got["value"] == pytest.approx(3000.0 / 20e-3)


def test_reference_arm_prints_from_rank0_only(tmp_path):
    pytest.importorskip("torch.distributed")
    _spawn(_reference_rank, 2, tmp_path)
    assert (tmp_path / "ref1.txt").read_text() == ""
    lines = (tmp_path / "ref0.txt").read_text().strip().splitlines()
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["steps"] == 2
    assert line["value"] == pytest.approx(1234.5)
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def test_replicas_are_distinct_instances():
    """Each rank solves its own seeded n=64 MIQCQP instance, the bench's
    headline shape (independent replicas)."""
    from cuminlp_gb300 import generators as G
    a, b = G.miqcqp_n64(0), G.miqcqp_n64(1)
    assert a.n_vars == b.n_vars and len(a.constraints) == len(b.constraints)
    consts = [[n.constant for n in p.graph.nodes] for p in (a, b)]
    assert consts[0] != consts[1]


def test_cpu_model_on_x86_and_arm(tmp_path):
    """The CPU baseline names the host's cores: x86 from its model name
    line, aarch64 (no such line) from the implementer and part fields."""
    sys.path.insert(0, str(ROOT))
    import bench
    x86 = tmp_path / "x86"
    x86.write_text("processor\t: 0\nvendor_id\t: GenuineIntel\nmodel name\t: Some Xeon CPU @ 2.00GHz\n")
    assert bench.cpu_info(str(x86))[0] == "Some Xeon CPU @ 2.00GHz"
    arm = tmp_path / "arm"
    arm.write_text("processor\t: 0\nBogoMIPS\t: 2000.00\nCPU implementer\t: 0x41\nCPU architecture: 8\n"
                   "CPU variant\t: 0x0\nCPU part\t: 0xd4f\nCPU revision\t: 0\n\nprocessor\t: 1\n"
                   "CPU implementer\t: 0x41\nCPU part\t: 0xd4f\n")
    assert bench.cpu_info(str(arm))[0] == "Arm Neoverse-V2"
    other = tmp_path / "other"
    other.write_text("CPU implementer\t: 0x61\nCPU part\t: 0x123\n")
    assert bench.cpu_info(str(other))[0] == "arm implementer 0x61 part 0x123"
    assert bench.cpu_info(str(tmp_path / "missing"))[0] == "unknown"
