"""The native server's scheduler on CPU (isl_serve_* with simulated work, no
GPU): batches formed in arrival order up to max_batch, at most max_batches
running at once, admission by a (simulated) free-HBM budget, arrivals
respected, invalid requests refused at submit."""
import numpy as np
import pytest

from insilico_gb300 import _abi as A
from insilico_gb300 import serve


def fake_server(max_batch=4, max_batches=2, budget=1 << 50, us_per_elem=0.2):
    return serve.Server(device=0, max_batch=max_batch, max_batches=max_batches, reserve_bytes=0,
                        test_budget_bytes=budget, test_fake_us_per_elem=us_per_elem)


def max_overlap(done):
    """Largest number of batches running at the same time."""
    spans = {}
    for r in done:
        a, b = spans.get(r.batch_id, (r.start, r.finish))
        spans[r.batch_id] = (min(a, r.start), max(b, r.finish))
    events = sorted([(a, 1) for a, _ in spans.values()] + [(b, -1) for _, b in spans.values()])
    cur = peak = 0
    for _, d in events:
        cur += d
        peak = max(peak, cur)
    return peak


def test_batches_bounded_and_all_requests_finish():
    reqs = serve.make_requests(24, rate=0.0, side_range=(4, 12))
    srv = fake_server(max_batch=4, max_batches=2)
    done, wall = srv.run(reqs, realtime=False)
    srv.close()
    assert len(done) == 24 and all(r.status == A.ISL_OK and r.converged for r in done)
    sizes = {}
    for r in done:
        sizes.setdefault(r.batch_id, []).append(r.rid)
        assert r.batch_size <= 4 and r.finish >= r.start >= r.submit
    assert len(sizes) >= 6 and all(len(v) == done[v[0]].batch_size for v in sizes.values())
    # batches take the queue in arrival order
    first = {b: min(v) for b, v in sizes.items()}
    assert [first[b] for b in sorted(first)] == sorted(first.values())
    assert max_overlap(done) <= 2
    assert all(np.array_equal(r.u, np.zeros(3 * (r.side + 1) ** 3)) for r in done)


def test_admission_by_memory_budget_runs_large_requests_one_at_a_time():
    # a budget smaller than any request: each runs alone, admitted only when
    # the GPU is idle (so an oversized request still runs)
    reqs = [serve.Request(i, 20, 1.0, 0.0) for i in range(6)]
    srv = fake_server(max_batch=8, max_batches=4, budget=1)
    done, _ = srv.run(reqs, realtime=False)
    srv.close()
    assert len(done) == 6 and all(r.batch_size == 1 for r in done)
    assert max_overlap(done) == 1


def test_arrivals_are_respected():
    reqs = serve.make_requests(6, rate=40.0, side_range=(4, 6))
    srv = fake_server(max_batch=8, max_batches=2)
    done, _ = srv.run(reqs, realtime=True)
    srv.close()
    subs = [r.submit for r in sorted(done, key=lambda q: q.arrival)]
    assert subs == sorted(subs)
    for r in done:
        assert r.start >= r.submit - 1e-9


def test_invalid_requests_are_refused_at_submit():
    srv = fake_server()
    r = serve.Request(0, 4, 1.0)
    a = serve.request_arrays(r)
    bad = dict(a)
    bad["conn"] = a["conn"].copy()
    bad["conn"][0, 0] = len(a["X"])  # node id out of range
    with pytest.raises(A.IslError):
        srv.submit(r, bad)
    bad = dict(a)
    bad["comp"] = a["comp"].copy()
    bad["comp"][0] = 3  # component out of range
    with pytest.raises(A.IslError):
        srv.submit(r, bad)
    srv.close()


def test_footprint_grows_with_side():
    assert serve.footprint_bytes(48) > 4 * serve.footprint_bytes(24) > 0


def test_size_ratio_groups_requests_of_similar_size():
    """size_ratio > 1: a batch holds only requests whose element count is
    within that factor of its first request's; the first request of each
    batch is still the oldest one queued."""
    reqs = serve.make_requests(24, rate=0.0, side_range=(4, 16))
    srv = serve.Server(device=0, max_batch=8, max_batches=2, reserve_bytes=0, test_budget_bytes=1 << 50,
                       test_fake_us_per_elem=0.2, size_ratio=2.0, batch_window_us=200_000)
    done, _ = srv.run(reqs, realtime=False)
    srv.close()
    assert len(done) == 24 and all(r.status == A.ISL_OK for r in done)
    batches = {}
    for r in done:
        batches.setdefault(r.batch_id, []).append(r)
    for members in batches.values():
        head = min(members, key=lambda q: q.rid)
        for q in members:
            assert q.side ** 3 <= 2.0 * head.side ** 3 and 2.0 * q.side ** 3 >= head.side ** 3
    first = {b: min(q.rid for q in v) for b, v in batches.items()}
    assert [first[b] for b in sorted(first)] == sorted(first.values())
    # without the ratio the same queue forms fewer, mixed batches
    srv = serve.Server(device=0, max_batch=8, max_batches=2, reserve_bytes=0, test_budget_bytes=1 << 50,
                       test_fake_us_per_elem=0.2, batch_window_us=200_000)
    done0, _ = srv.run([serve.Request(r.rid, r.side, r.mu) for r in reqs], realtime=False)
    srv.close()
    assert len({r.batch_id for r in done0}) < len(batches)


def test_largest_first_order():
    """order = 1: each batch starts from the largest queued request (the
    oldest among equals).  One batch at a time, one request per batch: the
    first request starts at once and runs for 1.3 s (simulated), while the
    others queue; they then run largest first."""
    reqs = [serve.Request(i, s, 1.0, 0.0) for i, s in enumerate([40, 5, 9, 7, 9, 3, 6])]
    srv = serve.Server(device=0, max_batch=1, max_batches=1, reserve_bytes=0, test_budget_bytes=1 << 50,
                       test_fake_us_per_elem=20.0, order=1)
    done, _ = srv.run(reqs, realtime=False)
    srv.close()
    assert all(r.status == A.ISL_OK for r in done)
    started = [r.rid for r in sorted(done, key=lambda q: q.start)]
    assert started == [0, 2, 4, 3, 6, 1, 5]
