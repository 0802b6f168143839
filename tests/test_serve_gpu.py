"""Served hyperelastic Newton solves on the GPU (the native server).

* plain (FP64 tangent + FP64 CG) and mixed (FP32 tangent + FP32 CG, FP64
  residual) requests reproduce the oracle's run of the reference driver
  (solid/CompressibleDriver.hpp:156-214, absolute tolerance on ||R||/N and
  ||dU||/N) within 1e-8 relative L2, with the same Newton iteration count on
  the plain path;
* a request's result is bitwise the same alone (a batch of one) and inside a
  batch of other requests (shared launches with per-request reductions);
* a request that fails (a degenerate element) is reported with its status,
  and requests in other batches are not affected.
"""
import numpy as np
import pytest

from insilico_gb300 import _abi as A
from insilico_gb300 import serve

from helpers import oracle_newton_driver

pytestmark = pytest.mark.gpu

WINDOW = 200_000  # us: requests submitted together form one batch


@pytest.mark.parametrize("precision", [A.PREC_FP64, A.PREC_FP32, A.PREC_MIXED])
def test_served_newton_matches_oracle_driver(precision):
    reqs = [serve.Request(0, side=3, mu=1.7), serve.Request(1, side=5, mu=0.3), serve.Request(2, side=4, mu=6.0)]
    srv = serve.Server(precision=precision, max_batch=8, max_batches=2, batch_window_us=WINDOW)
    done, _ = srv.run([serve.Request(r.rid, r.side, r.mu) for r in reqs], realtime=False)
    srv.close()
    assert all(r.status == A.ISL_OK and r.converged for r in done), [(r.status, r.error) for r in done]
    assert len({r.batch_id for r in done}) == 1  # one batch of three
    for r, got in zip(reqs, done):
        uo, newton = oracle_newton_driver(r, serve.NEWTON_TOL, serve.MAX_NEWTON)
        assert np.linalg.norm(got.u - uo) <= 1e-8 * np.linalg.norm(uo), (precision, r.rid)
        if precision == A.PREC_FP64:
            assert got.newton_iters == newton


@pytest.mark.parametrize("persistent", [0, 1])
@pytest.mark.parametrize("precision", [A.PREC_FP32, A.PREC_MIXED])
def test_one_request_per_batch_matches_oracle_driver(precision, persistent):
    """max_batch = 1: every request on its own context and stream, through
    the single-system solvers (the block CG on padded node blocks: the x = 1
    face fixes u_x only), several at once; the graph path (persistent 0, the
    server's default) and the one-launch solve (1).  Sides 10 and 12 give
    1,210 and 2,028 block rows.  Each result reproduces the oracle's run of
    the reference driver within 1e-8, and the same request gives the same
    bits in a second run."""
    reqs = [serve.Request(0, side=3, mu=1.7), serve.Request(1, side=10, mu=0.3), serve.Request(2, side=12, mu=6.0),
            serve.Request(3, side=4, mu=0.12)]
    out = []
    for _ in range(2):
        srv = serve.Server(precision=precision, max_batch=1, max_batches=3, persistent=persistent)
        done, _ = srv.run([serve.Request(r.rid, r.side, r.mu) for r in reqs], realtime=False)
        srv.close()
        assert all(r.status == A.ISL_OK and r.converged and r.batch_size == 1 for r in done), \
            [(r.status, r.error) for r in done]
        out.append(done)
    for r, got, again in zip(reqs, out[0], out[1]):
        uo, _ = oracle_newton_driver(r, serve.NEWTON_TOL, serve.MAX_NEWTON)
        assert np.linalg.norm(got.u - uo) <= 1e-8 * np.linalg.norm(uo), (precision, r.rid)
        assert np.array_equal(got.u, again.u) and got.cg_iters == again.cg_iters


def test_result_same_alone_and_in_a_batch():
    reqs = serve.make_requests(6, rate=0.0, side_range=(3, 7))
    # alone: a batching server given a single request (a batch of one)
    alone = serve.Server(max_batch=8, max_batches=1, batch_window_us=WINDOW)
    ref, _ = alone.run([serve.Request(reqs[2].rid, reqs[2].side, reqs[2].mu)], realtime=False)
    alone.close()
    mix = serve.Server(max_batch=8, max_batches=2, batch_window_us=WINDOW)
    done, wall = mix.run(reqs, realtime=False)
    mix.close()
    got = [r for r in done if r.rid == reqs[2].rid][0]
    assert got.batch_size > 1 and ref[0].batch_size == 1
    assert got.converged and ref[0].converged
    assert np.array_equal(got.u, ref[0].u)
    assert got.newton_iters == ref[0].newton_iters and got.cg_iters == ref[0].cg_iters
    stats = serve.latency_stats(done, wall)
    assert stats["n"] == 6 and stats["p99_s"] >= stats["p50_s"] > 0


def test_failed_request_is_reported_and_isolated():
    good = [serve.Request(0, 3, 1.0), serve.Request(2, 4, 2.0)]
    bad = serve.Request(1, 3, 1.0)
    a = serve.request_arrays(bad)
    a["conn"] = a["conn"].copy()
    a["conn"][0, [0, 1]] = a["conn"][0, [1, 0]]  # an inverted element: det J < 0
    srv = serve.Server(max_batch=1, max_batches=2)
    tickets = [srv.submit(good[0]), srv.submit(bad, a), srv.submit(good[1])]
    import ctypes as C
    out = []
    for t, r in zip(tickets, [good[0], bad, good[1]]):
        state = C.c_int()
        assert srv.L.isl_serve_wait(srv.h, t, 600.0, C.byref(state)) == A.ISL_OK
        out.append((state.value, srv.error(t)))
        srv.collect(t, r, (r.side + 1) ** 3)
    srv.close()
    assert out[1][0] == 3 and bad.status == A.ISL_ERR_DEGENERATE and "isl_assemble" in out[1][1]
    assert out[0][0] == 2 and out[2][0] == 2
    assert good[0].converged and good[1].converged
