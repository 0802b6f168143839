"""Continuous-batching server for hyperelastic Newton solves (served Newton workload).

Each request is a compressible neo-Hookean cube (solid::HyperElastic with
mat::hypel::NeoHookeanCompressible) on a hex8 mesh of side s, pulled along x
in 5 load steps (reference/06-elastic/PulledSheet.hpp:35-58 boundary
conditions, solid/CompressibleDriver.hpp:156-214 load stepping and Newton
loop).  The server keeps every admitted request's mesh, CSR pattern, matrix
and iterate resident on the GPU across its Newton iterations.

Scheduling:
  * K slots, each an isl_ctx with its own CUDA stream driven by its own host
    thread (ctypes releases the GIL inside every library call), so the
    assembly and CG kernels of all admitted requests overlap on the device;
  * a request is admitted when it has arrived, a slot is free and its
    estimated device footprint fits the free HBM minus a reserve;
  * finished requests free their slot immediately and the next arrival is
    admitted (continuous batching, not a FIFO of whole batches).

Precision: the mixed mode assembles the tangent in FP32 with FP64 internal
forces (ISL_PREC_FP32) and solves each Newton step inexactly with FP32 CG;
the plain mode uses FP64 throughout (ISL_PREC_FP64 + FP64 CG).  A request's
result does not depend on what else is running: every context computes with
fixed-order reductions on its own buffers.
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _abi as A
from .system import System
from . import workloads as W


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
    newton_iters: int = 0
    cg_iters: int = 0
    u: Optional[np.ndarray] = None
    converged: bool = True
    history: list = field(default_factory=list)

    @property
    def lam(self):
        # bulk modulus 10 mu  ->  lambda = K - 2 mu / 3
        return 10.0 * self.mu - 2.0 * self.mu / 3.0

    @property
    def latency(self):
        return self.finish - self.arrival


def make_requests(n: int, rate: float, seed: int = W.SEED_BASE + 4, side_range=(8, 48)) -> List[Request]:
    """n requests with Poisson arrivals at `rate` per second, side U{8..48},
    mu log-uniform [0.1, 10]."""
    g = W.rng(seed, 0)
    sides = g.integers(side_range[0], side_range[1] + 1, n)
    mus = 10.0 ** W.rng(seed, 1).uniform(-1.0, 1.0, n)
    gaps = W.rng(seed, 2).exponential(1.0 / rate, n) if rate > 0 else np.zeros(n)
    t = np.cumsum(gaps) - gaps[0]
    return [Request(i, int(sides[i]), float(mus[i]), float(t[i])) for i in range(n)]


def footprint_bytes(side: int) -> int:
    """Estimated peak device memory of one request (pattern build included)."""
    ne = side ** 3
    neq = 3 * (side + 1) ** 3
    nnz = 81 * neq
    pairs = ne * 576
    persistent = nnz * (4 + 4 + 4 + 8) + pairs * 4 + ne * (300 * 8 + 24 * 12) + neq * 120
    transient = pairs * 24
    return int(persistent + transient)


class NewtonSolver:
    """Runs requests on one isl_ctx (one slot)."""

    def __init__(self, device: int = 0, mixed: bool = True):
        self.S = System(device=device)
        self.mixed = mixed

    def close(self):
        self.S.close()

    def run(self, r: Request, max_newton: int = 30, rtol: float = 1e-10, lin_tol_mixed: float = 1e-6,
            lin_tol_plain: float = 1e-10):
        S = self.S
        X, conn = W.unit_cube("hex", r.side, r.side, r.side)
        S.upload_mesh(A.HEX, X, conn)
        S.create_field(1, 3)
        first = r.pull / r.load_steps

        def diri(x):
            m = np.zeros((len(x), 3), dtype=bool)
            v = np.zeros((len(x), 3))
            left = np.abs(x[:, 0]) < 1e-9
            right = np.abs(x[:, 0] - 1.0) < 1e-9
            m[left] = True
            m[right, 0] = True
            v[right, 0] = first
            return m, v
        S.constrain_boundary(diri)
        neq = S.number_dofs()
        S.register_pattern()
        ne = len(conn)
        S.set_hyperelastic("neohooke", np.full(ne, r.lam), np.full(ne, r.mu), 3)
        S.set_values(np.zeros(S.ndofobj * 3))
        prec = A.PREC_FP32 if self.mixed else A.PREC_FP64
        meth = A.SOLVE_CG_FP32_IR if self.mixed else A.SOLVE_CG_FP64
        lin_tol = lin_tol_mixed if self.mixed else lin_tol_plain
        r.newton_iters = r.cg_iters = 0
        r.converged = True
        norm0 = None
        for step in range(r.load_steps):
            S.scale_constraints(float(step + 1) if step == 0 else (step + 1) / step)
            for it in range(max_newton):
                S.assemble(prec, incremental=True, with_residual=True)
                b = S.rhs()
                conv1 = float(np.linalg.norm(b)) / neq
                if norm0 is None or it == 0:
                    norm0 = conv1 if it == 0 else norm0
                r.history.append((step, it, conv1))
                if conv1 <= rtol * max(norm0, 1e-300) and it > 0:
                    break
                cg_it, _, st = S.solve(meth, tol=lin_tol, check=False)
                if st not in (A.ISL_OK, A.ISL_ERR_NOT_CONVERGED):
                    S._chk(st, "isl_solve")
                r.cg_iters += cg_it
                S.distribute(add=True)
                r.newton_iters += 1
            else:
                r.converged = False
        r.u = S.values()
        return r


class Server:
    """Continuous batching over K slots with admission by free HBM."""

    def __init__(self, slots: int = 8, device: int = 0, mixed: bool = True, reserve_bytes: int = 8 << 30,
                 memory_budget: Optional[int] = None, solver_factory=None):
        make = solver_factory or (lambda: NewtonSolver(device, mixed))
        self.slots = [make() for _ in range(slots)]
        self.device = device
        self.reserve = reserve_bytes
        self.budget = memory_budget  # simulated free-HBM budget (tests); None = cudaMemGetInfo
        self.lock = threading.Lock()
        self.in_use = 0

    def close(self):
        for s in self.slots:
            s.close()

    def free_hbm(self) -> int:
        if self.budget is not None:
            return self.budget - self.in_use
        import ctypes as C
        f, t = C.c_int64(), C.c_int64()
        A.load().isl_device_memory(self.device, C.byref(f), C.byref(t))
        # reservations of admitted requests count in full (conservative: part
        # of them is already allocated and visible in the free figure)
        return f.value - self.in_use

    def run(self, requests: List[Request], realtime: bool = True):
        """Serve requests (sorted by arrival); returns them with timings."""
        pending = sorted(requests, key=lambda q: q.arrival)
        free_slots = list(range(len(self.slots)))
        done: List[Request] = []
        cv = threading.Condition()
        t0 = time.perf_counter()
        active = {}
        errors = []

        def worker(slot: int, req: Request, need: int):
            try:
                req.start = time.perf_counter() - t0
                self.slots[slot].run(req)
                req.finish = time.perf_counter() - t0
            except Exception as ex:  # reported to the caller
                errors.append((req.rid, repr(ex)))
                req.finish = time.perf_counter() - t0
                req.converged = False
            with cv:
                free_slots.append(slot)
                self.in_use -= need
                done.append(req)
                active.pop(req.rid, None)
                cv.notify_all()

        i = 0
        with cv:
            while i < len(pending) or active:
                now = time.perf_counter() - t0
                if i < len(pending) and free_slots:
                    req = pending[i]
                    if not realtime:
                        req.arrival = min(req.arrival, now)
                    need = footprint_bytes(req.side)
                    fits = self.free_hbm() - need >= self.reserve
                    if req.arrival <= now and (fits or not active):
                        # a request larger than the budget still runs alone
                        slot = free_slots.pop()
                        self.in_use += need
                        th = threading.Thread(target=worker, args=(slot, req, need), daemon=True)
                        active[req.rid] = th
                        i += 1
                        th.start()
                        continue
                    wait = max(0.0, req.arrival - now) if req.arrival > now else 0.05
                    cv.wait(timeout=min(wait, 0.05) if wait > 0 else 0.05)
                else:
                    cv.wait(timeout=0.05)
        if errors:
            raise RuntimeError(f"requests failed: {errors[:3]}")
        return sorted(done, key=lambda q: q.rid), time.perf_counter() - t0


def latency_stats(reqs: List[Request], wall: float):
    lat = np.array([r.latency for r in reqs])
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "solves_per_s": len(reqs) / wall, "n": len(reqs), "wall_s": wall,
            "newton_iters": int(sum(r.newton_iters for r in reqs)), "cg_iters": int(sum(r.cg_iters for r in reqs))}
