"""Scheduler of the continuous-batching server, on CPU with a fake slot solver:
admission by (simulated) free HBM, slots refilled as requests finish, arrival
order respected, a failing request reported."""
import threading
import time

import pytest

from insilico_gb300 import serve


class FakeSolver:
    active = 0
    peak = 0
    lock = threading.Lock()

    def __init__(self, dt=0.02, fail_rid=None):
        self.dt = dt
        self.fail_rid = fail_rid

    def run(self, r):
        with FakeSolver.lock:
            FakeSolver.active += 1
            FakeSolver.peak = max(FakeSolver.peak, FakeSolver.active)
        time.sleep(self.dt * r.side / 8)
        with FakeSolver.lock:
            FakeSolver.active -= 1
        if r.rid == self.fail_rid:
            raise RuntimeError("injected failure")
        r.newton_iters = 1
        return r

    def close(self):
        pass


def reset():
    FakeSolver.active = FakeSolver.peak = 0


def test_slots_bound_concurrency_and_all_requests_finish():
    reset()
    reqs = serve.make_requests(24, rate=0.0)
    srv = serve.Server(slots=4, memory_budget=1 << 50, reserve_bytes=0, solver_factory=lambda: FakeSolver(0.005))
    done, wall = srv.run(reqs, realtime=False)
    assert len(done) == 24 and FakeSolver.peak == 4
    assert all(r.finish >= r.start >= r.arrival - 1e-9 for r in done)


def test_admission_by_memory_budget_serialises_large_requests():
    reset()
    reqs = [serve.Request(i, 40, 1.0, 0.0) for i in range(6)]
    need = serve.footprint_bytes(40)
    srv = serve.Server(slots=4, memory_budget=int(1.5 * need), reserve_bytes=0, solver_factory=lambda: FakeSolver(0.005))
    done, _ = srv.run(reqs, realtime=False)
    assert len(done) == 6 and FakeSolver.peak == 1


def test_arrivals_are_respected():
    reset()
    reqs = serve.make_requests(6, rate=50.0)
    srv = serve.Server(slots=2, memory_budget=1 << 50, reserve_bytes=0, solver_factory=lambda: FakeSolver(0.002))
    done, _ = srv.run(reqs, realtime=True)
    for r in done:
        assert r.start + 1e-3 >= r.arrival


def test_failed_request_is_reported():
    reset()
    reqs = serve.make_requests(5, rate=0.0)
    srv = serve.Server(slots=2, memory_budget=1 << 50, reserve_bytes=0, solver_factory=lambda: FakeSolver(0.001, fail_rid=3))
    with pytest.raises(RuntimeError, match="injected failure"):
        srv.run(reqs, realtime=False)


def test_footprint_grows_with_side():
    assert serve.footprint_bytes(48) > 4 * serve.footprint_bytes(24) > 0
