"""The continuous-batching server: requests of mixed sizes arriving while
others run are admitted as slots and box-pool memory free up, and every
result is bit-for-bit the one the same request gets alone (a one-slot
batch) and from the oracle's batched restatement."""

from __future__ import annotations

import threading
import time

import numpy as np
import pytest

import oracle as O
from cuminlp_gb300 import generators as G
from cuminlp_gb300._lib import CmnError
from cuminlp_gb300.solver import Batch, DeviceProblem, Server
from tests.test_gpu_batch import same_outcome
from tests.test_oracle_pins import fixture_problems

pytestmark = pytest.mark.gpu

SHARED = dict(bisection_budget=4, batch_parents=16, frontier_cap=256, sample_points=1)
CLASSES = [(8, 3), (16, 3), (32, 2), (64, 2)]


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cuminlp_gb300 import build
    build.build_library()


def requests():
    fx = fixture_problems()
    ps = [G.serving_qcqp(i) for i in range(14)] + [fx["square_le5"], fx["miqcqp_n6"], G.qcqp_n4(1)]
    limits = [300 + 97 * (i % 7) for i in range(len(ps))]
    return ps, limits


def alone(dp, iter_limit, shared=SHARED):
    b = Batch(1, dp.n_vars, dp.info()["program_slots"], **shared)
    s = b.add(dp, iter_limit=iter_limit)
    b.step(0)
    out = b.outcome(s)
    b.close()
    return out


def submit_stream(server, dps, limits, seed=7, mean_gap_s=0.002):
    """Submits from another thread with exponential gaps (a Poisson stream)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(mean_gap_s, size=len(dps))
    ids = [None] * len(dps)

    def run():
        for i, (dp, il) in enumerate(zip(dps, limits)):
            time.sleep(gaps[i])
            ids[i] = server.submit(dp, iter_limit=il)

    t = threading.Thread(target=run)
    t.start()
    t.join()
    return ids


def test_server_results_same_alone_and_in_mix():
    ps, limits = requests()
    dps = [DeviceProblem(p) for p in ps]
    slots = max(dp.info()["program_slots"] for dp in dps)
    srv = Server([(v, n, slots) for v, n in CLASSES], iterations_per_round=3, **SHARED)
    ids = submit_stream(srv, dps, limits)
    got = [srv.wait(i, timeout_ms=120000) for i in ids]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(ps) and st["queued"] == 0 and st["running"] == 0
    assert st["latency_p99_ms"] >= st["latency_p50_ms"] > 0
    for k, (dp, il, g) in enumerate(zip(dps, limits, got)):
        same_outcome(g, alone(dp, il), f"request {k}")
    # and the alone runs are the oracle's batched search
    for k in (0, 3, 14, 15, 16):
        o = O.OracleProblem(ps[k]).solve_batched(iter_limit=limits[k], **SHARED)
        same_outcome(got[k], o, f"request {k} vs oracle")


def test_lazy_server_results_same_alone_and_as_the_oracle():
    # the lazy form in every class: each result the one-slot batch's and
    # the oracle's (which restates the lazy form from the compiled programs)
    shared = dict(SHARED, precision="lazy")
    ps, limits = requests()
    dps = [DeviceProblem(p) for p in ps]
    slots = max(dp.info()["program_slots"] for dp in dps)
    srv = Server([(v, n, slots) for v, n in CLASSES], iterations_per_round=3, **shared)
    ids = submit_stream(srv, dps, limits)
    got = [srv.wait(i, timeout_ms=120000) for i in ids]
    srv.close()
    for k, (dp, il, g) in enumerate(zip(dps, limits, got)):
        same_outcome(g, alone(dp, il, shared), f"request {k}")
    for k in (0, 3, 14, 15, 16):
        op = O.OracleProblem(ps[k])
        op.set_program32(dps[k].program(1))
        op.set_program64(dps[k].program(0))
        o = op.solve_batched(iter_limit=limits[k], **shared)
        same_outcome(got[k], o, f"request {k} vs oracle")


def test_server_admits_by_pool_memory():
    ps, limits = requests()
    dps = [DeviceProblem(p) for p in ps[:8]]
    slots = max(dp.info()["program_slots"] for dp in dps)
    probe = Batch(1, 64, slots, **SHARED)
    from cuminlp_gb300._lib import lib
    per_slot = int(lib().cmn_batch_slot_bytes(probe.handle))
    probe.close()
    budget = 2 * per_slot
    srv = Server([(64, 6, slots)], pool_budget_bytes=budget, iterations_per_round=2, **SHARED)
    ids = [srv.submit(dp, iter_limit=il) for dp, il in zip(dps, limits)]
    got = [srv.wait(i, timeout_ms=120000) for i in ids]
    st = srv.stats()
    srv.close()
    assert st["pool_bytes_peak"] <= budget
    assert st["completed"] == len(dps)
    for k, (dp, il, g) in enumerate(zip(dps, limits, got)):
        same_outcome(g, alone(dp, il), f"request {k}")


def test_server_rejects_and_times_out():
    srv = Server([(8, 1)], **SHARED)
    big = DeviceProblem(G.serving_qcqp(3) if G.serving_qcqp(3).n_vars > 8 else G.miqcqp_n32())
    with pytest.raises(CmnError) as e:
        srv.submit(big)
    assert e.value.status_name == "INVALID_CONFIGURATION"
    # a negative tolerance never closes the gap: the request runs until its
    # boxes degenerate, far longer than the wait
    small = DeviceProblem(next(p for p in (G.serving_qcqp(i) for i in range(20)) if p.n_vars == 8))
    rid = srv.submit(small, iter_limit=10 ** 9, tolerance=-1.0)
    with pytest.raises(CmnError) as e:
        srv.wait(rid, timeout_ms=20)
    assert e.value.status_name == "TIMEOUT"
    assert srv.poll(rid) is None
    srv.close()  # abandons the running request
