"""Served hyperelastic Newton solves on the GPU.

* the plain FP64 path reproduces the oracle's Newton solution (rel L2 1e-8);
* the mixed path (FP32 tangent + FP32 CG, FP64 residual) converges to the same
  solution within 1e-8 relative L2;
* a request's result is bitwise the same alone and in a mix of concurrent
  requests (continuous batching does not change results).
"""
import numpy as np
import pytest

from insilico_gb300 import serve

from helpers import oracle_newton

pytestmark = pytest.mark.gpu


def test_plain_and_mixed_newton_match_oracle():
    req = serve.Request(0, side=3, mu=1.7)
    uo = oracle_newton(req)
    plain = serve.NewtonSolver(mixed=False)
    rp = plain.run(serve.Request(0, side=3, mu=1.7))
    mixed = serve.NewtonSolver(mixed=True)
    rm = mixed.run(serve.Request(0, side=3, mu=1.7))
    assert rp.converged and rm.converged
    assert np.linalg.norm(rp.u - uo) <= 1e-8 * np.linalg.norm(uo)
    assert np.linalg.norm(rm.u - uo) <= 1e-8 * np.linalg.norm(uo)
    plain.close()
    mixed.close()


def test_result_same_alone_and_in_mix():
    reqs = serve.make_requests(6, rate=0.0, side_range=(3, 7))
    alone = serve.Server(slots=1)
    ref, _ = alone.run([serve.Request(r.rid, r.side, r.mu) for r in reqs[:1]], realtime=False)
    alone.close()
    mix = serve.Server(slots=4)
    done, wall = mix.run(reqs, realtime=False)
    mix.close()
    got = [r for r in done if r.rid == reqs[0].rid][0]
    assert got.converged and ref[0].converged
    assert np.array_equal(got.u, ref[0].u)
    stats = serve.latency_stats(done, wall)
    assert stats["n"] == 6 and stats["p99_s"] >= stats["p50_s"] > 0
