"""Served hyperelastic Newton solves: the workload and a thin binding of the
native server (isl_serve_* in include/isl_gpu.h, insilico_gb300/csrc/isl_serve.cpp).

Each request is a compressible neo-Hookean cube (solid::HyperElastic with
mat::hypel::NeoHookeanCompressible) on a hex8 mesh of side s, pulled along x
in 5 load steps: x = 0 clamped, u_x prescribed on x = 1
(reference/06-elastic/PulledSheet.hpp:35-60), the prescribed value scaled
by (k+1)/k at load step k and Newton iterations until ||R||/N or ||dU||/N
falls below the tolerance (solid/CompressibleDriver.hpp:156-214).

The server (C++) forms batches of queued requests in arrival order, admits
them by free HBM, runs each batch's Newton iterations in shared launches on
its own stream, runs several batches at once, and completes each request as
soon as its own Newton loop ends.  This module builds the request arrays,
submits them (all at once, or at their Poisson arrival times from a host
thread) and collects results and latencies; the timing is the server's own
clock (seconds since the server was created).
"""
from __future__ import annotations

import ctypes as C
import threading
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _abi as A
from . import workloads as W

# Newton tolerance on ||R||/N and ||dU||/N (absolute, as the reference
# driver's): the quadratic phase takes both below 1e-12 in 4 iterations per
# load step for mu in [0.1, 10] on the unit cube, far above the round-off
# floor (about 1e-19 mu)
NEWTON_TOL = 1e-12
MAX_NEWTON = 12


@dataclass
class Request:
    rid: int
    side: int
    mu: float
    arrival: float = 0.0          # seconds after the stream starts
    load_steps: int = 5
    pull: float = 0.3             # stretch 1.3 of the unit cube
    # results
    start: float = 0.0
    finish: float = 0.0
    submit: float = 0.0
    newton_iters: int = 0
    cg_iters: int = 0
    u: Optional[np.ndarray] = None
    converged: bool = True
    status: int = 0
    batch_id: int = -1
    batch_size: int = 0
    error: str = ""
    history: list = field(default_factory=list)

    @property
    def lam(self):
        # bulk modulus 10 mu  ->  lambda = K - 2 mu / 3
        return 10.0 * self.mu - 2.0 * self.mu / 3.0

    @property
    def latency(self):
        return self.finish - self.submit


def make_requests(n: int, rate: float, seed: int = W.SEED_BASE + 4, side_range=(8, 48)) -> List[Request]:
    """n requests with Poisson arrivals at `rate` per second, side U{8..48},
    mu log-uniform [0.1, 10]."""
    g = W.rng(seed, 0)
    sides = g.integers(side_range[0], side_range[1] + 1, n)
    mus = 10.0 ** W.rng(seed, 1).uniform(-1.0, 1.0, n)
    gaps = W.rng(seed, 2).exponential(1.0 / rate, n) if rate > 0 else np.zeros(n)
    t = np.cumsum(gaps) - gaps[0]
    return [Request(i, int(sides[i]), float(mus[i]), float(t[i])) for i in range(n)]


def request_arrays(r: Request):
    """Mesh, coefficients and first-load-step Dirichlet values of a request."""
    X, conn = W.unit_cube("hex", r.side, r.side, r.side)
    ne = len(conn)
    left = np.nonzero(np.abs(X[:, 0]) < 1e-9)[0]
    right = np.nonzero(np.abs(X[:, 0] - 1.0) < 1e-9)[0]
    nodes = np.concatenate([np.repeat(left, 3), right]).astype(np.int64)
    comps = np.concatenate([np.tile(np.arange(3), len(left)), np.zeros(len(right), dtype=np.int64)]).astype(np.int32)
    vals = np.concatenate([np.zeros(3 * len(left)), np.full(len(right), r.pull / r.load_steps)])
    return {"X": np.ascontiguousarray(X), "conn": np.ascontiguousarray(conn, dtype=np.int64),
            "lam": np.full(ne, r.lam), "mu": np.full(ne, r.mu), "node": nodes, "comp": comps, "val": vals}


def footprint_bytes(side: int) -> int:
    """Rough peak device memory of one request (the server's own estimate is
    the one that admits)."""
    ne = side ** 3
    neq = 3 * (side + 1) ** 3
    nnz = 81 * neq
    pairs = ne * 576
    return int(nnz * 28 + pairs * 28 + ne * 300 * 8 + neq * 160)


class Server:
    """Binding of the native continuous-batching server."""

    def __init__(self, device: int = 0, precision: int = A.PREC_FP32, max_batch: int = 64, max_batches: int = 4,
                 reserve_bytes: int = 8 << 30, lin_tol: Optional[float] = None, test_budget_bytes: int = 0,
                 test_fake_us_per_elem: float = 0.0, batch_window_us: int = 0, size_ratio: float = 0.0,
                 persistent: int = 0, order: int = 0):
        self.L = A.load()
        self.precision = precision
        self.lin_tol = lin_tol if lin_tol is not None else (1e-6 if precision == A.PREC_FP32 else 1e-10)
        cfg = A.ServeConfig(max_batch, max_batches, precision, reserve_bytes, 0, test_budget_bytes,
                            test_fake_us_per_elem, batch_window_us, size_ratio, persistent, order)
        self.h = C.c_void_p()
        st = self.L.isl_serve_create(C.byref(self.h), device, C.byref(cfg))
        if st != A.ISL_OK:
            raise A.IslError(st, "isl_serve_create")
        self.h2d_bytes = 0
        self.d2h_bytes = 0

    def close(self):
        if self.h:
            self.L.isl_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, r: Request, arrays: Optional[dict] = None) -> int:
        """Queue request r (its arrays from request_arrays unless given)."""
        a = arrays if arrays is not None else request_arrays(r)
        q = A.ServeRequest()
        q.shape, q.n_nodes, q.coords = A.HEX, len(a["X"]), A.d(a["X"])
        q.n_elem, q.conn = len(a["conn"]), A.i64(a["conn"])
        q.ncomp, q.kernel, q.material, q.quad_degree = 3, A.KERNEL_HYPERELASTIC, A.MAT_NEOHOOKE, 3
        q.coef0, q.coef1, q.body = A.d(a["lam"]), A.d(a["mu"]), None
        q.n_fixed, q.fixed_node, q.fixed_comp, q.fixed_value = len(a["node"]), A.i64(a["node"]), A.i32(a["comp"]), A.d(a["val"])
        q.load_steps, q.max_newton, q.tolerance, q.lin_tol = r.load_steps, MAX_NEWTON, NEWTON_TOL, self.lin_tol
        t = C.c_int64()
        st = self.L.isl_serve_submit(self.h, C.byref(q), C.byref(t))
        if st != A.ISL_OK:
            raise A.IslError(st, "isl_serve_submit")
        # inputs the server copied: coordinates, connectivity, lambda, mu, Dirichlet lists
        self.h2d_bytes += sum(v.nbytes for v in a.values())
        return t.value

    def collect(self, ticket: int, r: Request, n_nodes: int):
        u = np.zeros(n_nodes * 3)
        s = A.ServeStats()
        st = self.L.isl_serve_result(self.h, ticket, A.d(u), C.byref(s))
        r.status = st
        if st != A.ISL_OK:
            r.converged = False
            r.u = None
            r.error = self.error(ticket)
        else:
            r.u = u
            r.converged = bool(s.converged)
            self.d2h_bytes += u.nbytes
        r.newton_iters, r.cg_iters = int(s.newton_iters), int(s.cg_iters)
        r.submit, r.start, r.finish = s.t_submit, s.t_admit, s.t_finish
        r.batch_id, r.batch_size = int(s.batch_id), int(s.batch_size)
        self.L.isl_serve_release(self.h, ticket)
        return r

    def counters(self):
        """(kernel launches of the finished batches, batches formed)"""
        n, b = C.c_int64(), C.c_int64()
        self.L.isl_serve_counters(self.h, C.byref(n), C.byref(b))
        return n.value, b.value

    def times(self):
        """Host seconds of the finished batches: setup, assembly, solve, whole
        batches; and the Newton iterations they ran."""
        v = [C.c_double() for _ in range(4)]
        t = C.c_int64()
        self.L.isl_serve_times(self.h, *[C.byref(x) for x in v], C.byref(t))
        return {"setup_s": v[0].value, "assemble_s": v[1].value, "solve_s": v[2].value, "batches_s": v[3].value,
                "newton_ticks": t.value}

    def error(self, ticket: int) -> str:
        return self.L.isl_serve_error(self.h, ticket).decode()

    def run(self, requests: List[Request], realtime: bool = True, timeout_s: float = 3600.0):
        """Serve the requests; realtime: submit each at its arrival time (a
        host thread), else all at once.  Returns (requests with results, wall
        seconds from the first submit to the last finish)."""
        order = sorted(requests, key=lambda q: q.arrival)
        tickets = {}
        errors = []

        def submitter():
            t0 = time.perf_counter()
            for r in order:
                if realtime:
                    wait = r.arrival - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(wait)
                try:
                    tickets[r.rid] = self.submit(r)
                except Exception as ex:  # reported to the caller
                    errors.append((r.rid, repr(ex)))
        th = threading.Thread(target=submitter, daemon=True)
        th.start()
        th.join()
        failed = []
        for r in order:
            if r.rid not in tickets:
                continue
            state = C.c_int()
            st = self.L.isl_serve_wait(self.h, tickets[r.rid], timeout_s, C.byref(state))
            if st != A.ISL_OK:
                raise A.IslError(st, f"request {r.rid} did not finish")
            self.collect(tickets[r.rid], r, (r.side + 1) ** 3)
            if r.status != A.ISL_OK:
                failed.append((r.rid, r.status))
        if errors:
            raise RuntimeError(f"requests not submitted: {errors[:3]}")
        done = sorted(order, key=lambda q: q.rid)
        wall = max(r.finish for r in done) - min(r.submit for r in done)
        return done, wall


def latency_stats(reqs: List[Request], wall: float):
    lat = np.array([r.latency for r in reqs])
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "solves_per_s": len(reqs) / wall, "n": len(reqs), "wall_s": wall,
            "newton_iters": int(sum(r.newton_iters for r in reqs)), "cg_iters": int(sum(r.cg_iters for r in reqs)),
            "batches": len({r.batch_id for r in reqs}), "max_batch": max(r.batch_size for r in reqs)}
