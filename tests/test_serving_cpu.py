"""Host logic of the serving loop (no GPU): admission order, slot and memory
limits, continuous admission as solves finish, latency bookkeeping."""
import threading
import time

import numpy as np
import pytest

from quantit_gb300 import serving


def _fake_solver(log, lock, active, peak):
    def run(req, **kw):
        with lock:
            active[0] += 1
            peak[0] = max(peak[0], active[0])
            log.append(("start", req.rid, time.perf_counter()))
        time.sleep(0.01 + 0.002 * (req.rid % 3))
        with lock:
            active[0] -= 1
        return -0.4 * req.L - 0.01 * req.delta, 3
    return run


def test_admission_respects_slots_order_and_memory():
    reqs = [serving.SolveRequest(i, L=8 + 4 * (i % 3), delta=0.5, D=16, seed=i, arrival=0.0) for i in range(12)]
    log, lock, active, peak = [], threading.Lock(), [0], [0]
    eng = serving.ServingEngine(slots=3, memory_budget=250, solver=_fake_solver(log, lock, active, peak),
                                footprint=lambda r: 100)  # memory admits two at a time, slots three
    res = eng.run(reqs, realtime=False)
    assert [r.rid for r in res] == list(range(12))
    assert all(r.error is None for r in res)
    assert peak[0] <= 2 and eng.peak_concurrency == 2
    assert eng.peak_memory <= 250
    starts = [rid for kind, rid, _ in sorted(log, key=lambda x: x[2])]
    assert starts[:2] == [0, 1] or starts[:2] == [1, 0]
    admitted = sorted(res, key=lambda r: r.admitted)
    assert [r.rid for r in admitted] == list(range(12))  # first come, first served
    for r in res:
        assert r.arrival <= r.admitted <= r.started <= r.done
        assert r.energy == pytest.approx(-0.4 * r.L - 0.005)


def test_oversized_request_runs_alone_and_errors_are_reported():
    def solver(req, **kw):
        if req.rid == 2:
            raise RuntimeError("boom")
        time.sleep(0.005)
        return -1.0, 1
    reqs = [serving.SolveRequest(i, 8, 1.0, 8, i, arrival=0.001 * i) for i in range(5)]
    eng = serving.ServingEngine(slots=4, memory_budget=100, solver=solver,
                                footprint=lambda r: 500 if r.rid == 1 else 10)
    res = eng.run(reqs, realtime=True)
    assert res[2].error and "boom" in res[2].error
    assert all(r.error is None for i, r in enumerate(res) if i != 2)
    # the oversized request shares the device with nobody
    big = res[1]
    for r in res:
        if r.rid != 1:
            assert r.done <= big.admitted or r.admitted >= big.done


def test_realtime_arrivals_are_not_admitted_early():
    reqs = serving.poisson_requests(6, rate=200.0, seed=3, lengths=(8,), bonds=(8,))
    eng = serving.ServingEngine(slots=2, memory_budget=10 ** 9, solver=lambda r, **k: (-1.0, 1),
                                footprint=lambda r: 1)
    res = eng.run(reqs, realtime=True)
    for r in res:
        assert r.admitted >= r.arrival - 1e-6


def test_poisson_stream_and_queue_model():
    reqs = serving.poisson_requests(200, rate=4.0, seed=1)
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) > 0)
    assert 1 / 4.0 * 0.8 < np.mean(np.diff(arr)) < 1 / 4.0 * 1.2
    assert {r.L for r in reqs} == {16, 32, 64, 128}
    assert {r.D for r in reqs} == {32, 64, 128, 256, 512}
    assert all(0.0 <= r.delta <= 2.0 for r in reqs)
    lat = serving.fifo_latencies([0.0, 0.0, 5.0], [2.0, 2.0, 1.0])
    assert lat == [2.0, 4.0, 1.0]
    s = serving.summarize(lat, 6.0, 3)
    assert s["solves_per_s"] == 0.5 and s["p50_s"] == 2.0


def test_footprint_grows_with_size():
    a = serving.footprint_bytes(16, 32)
    b = serving.footprint_bytes(16, 64)
    c = serving.footprint_bytes(64, 64)
    assert 0 < a < b < c
    assert serving.footprint_bytes(128, 512) < 40 * 2 ** 30


def test_ramp_stages():
    """A random start is swept at D/4 and D/2 (where at least 32) before D."""
    assert serving.ramp_stages(512) == [128, 256, 512]
    assert serving.ramp_stages(128) == [32, 64, 128]
    assert serving.ramp_stages(64) == [32, 64]
    assert serving.ramp_stages(32) == [32]


def test_results_carry_the_solver_truncated_weight():
    reqs = [serving.SolveRequest(i, 8, 1.0, 8, i) for i in range(3)]
    eng = serving.ServingEngine(slots=2, memory_budget=10 ** 9, footprint=lambda r: 1,
                                solver=lambda r, **k: (-1.0 - r.rid, 2, 1e-9 * (r.rid + 1)))
    seen = []
    res = eng.run(reqs, realtime=False, on_done=lambda r: seen.append(r.rid))
    assert sorted(seen) == [0, 1, 2]
    assert [r.truncated_weight for r in res] == [1e-9 * (i + 1) for i in range(3)]
    assert [r.energy for r in res] == [-1.0, -2.0, -3.0]
    # a two-value solver leaves the truncated weight unknown
    eng2 = serving.ServingEngine(slots=1, memory_budget=10 ** 9, footprint=lambda r: 1, solver=lambda r, **k: (-1.0, 1))
    import math
    assert all(math.isnan(r.truncated_weight) for r in eng2.run(reqs[:1], realtime=False))
