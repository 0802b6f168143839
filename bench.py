"""Benchmark of the GB300 assembly + Krylov hot path (one JSON line on rank 0).

Workload (N=1): 3-D linear elasticity, hex8 64^3 (65^3 nodes, 811,200 active
DOFs, 63.7M nonzeros), per-element E log-uniform [1e3, 1e5] and nu U[0.2, 0.45],
face x = 0 clamped, traction (1, 0, 0) on x = 1, 2x2x2 Gauss.  One step =
assemble K and f (FP64 element kernels, FP64 + FP32 CSR) + FP32 CG inside FP64
iterative refinement to the tolerance at which the solution is within 1e-8
relative L2 of the FP64 reference solution.  The plain FP64 GPU path (FP64 CG)
is measured at its own tolerance for the same error bar and reported beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--n 64]

--impl reference times the reference algorithm's CPU implementation (the
oracle restatement; the reference itself needs Eigen/Boost that are not
available) with all host threads on the same workload and metric.
Multi-GPU: replicas only (each rank solves its own copy; no collective).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "assembly GDOF/s & solve time at rel err≤1e-8 vs plain FP64 GPU; p50/p99 latency"
UNIT = "DOF/s"
ERR_BAR = 1e-8


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(name="spmv_fp32_c2"):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", f"{name}.md")
    try:
        with open(p) as f:
            for line in f:
                if line.strip().startswith("traffic_bytes_per_launch"):
                    return float(line.split("=")[1].split()[0])
    except Exception:
        pass
    return None


def ncu_traffic_ratio(name):
    """DRAM traffic over algorithmic bytes of a kernel from its committed ncu summary."""
    p = os.path.join(ROOT, "profiles", f"{name}.md")
    try:
        with open(p) as f:
            for line in f:
                if line.strip().startswith("traffic_ratio_to_algorithmic"):
                    return float(line.split("=")[1].split()[0])
    except Exception:
        pass
    return None


class Clocks:
    """nvidia-smi sampler for the timed region."""

    def __init__(self, index: int):
        self.f = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as f:
            for line in f:
                t = [x.strip() for x in line.split(",")]
                if len(t) >= 9:
                    rows.append(t)
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        load = [s for s in sm if s > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


L2_BYTES = 129 * 2 ** 20
_flush_buf = {}


def l2_flush(device):
    """Write a buffer twice the size of L2 (torch owns it; not timed)."""
    import torch
    if device not in _flush_buf:
        _flush_buf[device] = torch.empty(2 * L2_BYTES, dtype=torch.uint8, device=f"cuda:{device}")
    _flush_buf[device].fill_(len(_flush_buf) & 0xFF)
    torch.cuda.synchronize(device)


# sliced-ELL / block-row SpMV variants by autotune kind (isl_solver.cu)
SSPMV_KERNEL = {102: "k_sspmv_batch<2,8>", 104: "k_sspmv_batch<4,8>", 108: "k_sspmv_batch<8,6>"}
BSPMV_KERNEL = {1: "k_bspmv_pap<1>", 2: "k_bspmv_pap<2>", 3: "k_bspmv_pap<4>", 5: "k_bspmv_batch<2,4>",
                6: "k_bspmv_batch<4,3>", 7: "k_bspmv_batch<8,2>", 4: "k_brow_spmv<4>", 8: "k_brow_spmv<8>",
                16: "k_brow_spmv<16>"}
BSPMV_DIR_KERNEL = {5: "k_bspmv_dir<2,4>", 6: "k_bspmv_dir<4,3>", 7: "k_bspmv_dir<8,2>"}

WORKLOAD_DESC = {
    "c1": "c1 Q1 Poisson {n}^2 (heat::Laplace, kappa_e = exp(N(0,0.5)), nodal source U[0,1], g = 0)",
    "c2": "c2 hex8 linear elasticity {n}^3 (HyperElastic<StVenant> at u = 0, per-element E, nu; traction on x = 1)",
    "c3": "c3 tet10 Poisson {n}^3 hex -> 6 tets, jittered (heat::Laplace, kappa_e = exp(N(0,1)))",
}


def max_over_ranks(value, pg):
    """The largest value over all ranks (replicas: the slowest rank's time)."""
    if pg is None:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def spmv_bytes(nnz, n, v, col=4):
    """Algorithmic bytes of one CSR SpMV: nnz (v + col) + 4 (N + 1) + 2 N v
    (col = 2 with 16-bit column offsets)."""
    return nnz * (v + col) + 4 * (n + 1) + 2 * n * v


def log(*a):
    print("[bench]", *a, file=sys.stderr, flush=True)


def calibrate(S, method, x_ref, tols):
    """Loosest tolerance whose solution is within ERR_BAR of the FP64 reference."""
    from insilico_gb300 import _abi as A
    for tol in tols:
        it, rr, _ = S.solve(method, tol=tol)
        x = S.solution()
        err = float(np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref))
        log(f"calibrate method={method} tol={tol:g} iters={it} err={err:.3e}")
        if err <= ERR_BAR:
            return tol, err, it
    return tols[-1], err, it


REF_TOLS = [1e-9, 1e-10, 1e-11, 1e-12]
ORACLE_TOL = 1e-12  # the FP64 oracle solution every result is compared with


def workload_config(name, n, neq, nnz, nelem, world):
    """The `config` object of a c1/c2/c3 line: identical for the GPU arm and
    the reference arm, which run the same workload."""
    return {"workload": WORKLOAD_DESC[name].format(n=n), "active_dofs": int(neq), "nnz": int(nnz),
            "elements": int(nelem), "parallelism": "replicas" if world > 1 else "single",
            "l2": "inputs larger than L2 (FP64 CSR %.0f MB)" % (nnz * 12 / 1e6) if nnz * 12 > 2 * L2_BYTES
            else "L2 flushed before every timed step (FP64 CSR %.1f MB)" % (nnz * 12 / 1e6)}


def oracle_leg(p, threads):
    """The reference algorithm (oracle port) on the host cores at the full
    size of workload p: DOF numbering, constraints and the triplet pattern
    (setup, untimed), the assembly with the OpenMP element loop (timed), and
    Eigen-3.2-style Jacobi CG to ORACLE_TOL with its residual history (timed;
    the iteration count of any looser tolerance follows from the history).
    Its solution is the FP64 oracle solution of the error reports."""
    import oracle as O
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import oracle_problem
    t0 = time.perf_counter()
    P, _ = oracle_problem(p, assemble=False)
    P.pattern()
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    rp, ci, v, b = P.assemble(incremental=True, nthreads=threads)
    t_asm = time.perf_counter() - t0
    t0 = time.perf_counter()
    x, it, rr, hist = O.cg(rp, ci, v, b, tol=ORACLE_TOL, nthreads=threads, history=True)
    t_cg = time.perf_counter() - t0
    # one thread: the assembly's fixed part (clearing values and right-hand
    # side) plus the element loop over one element in 32, scaled, and 8 CG
    # iterations (the element loop and the iterations cost in proportion)
    esample = max(1, p.nelem // 32)
    P.element_range(0, 0)
    t0 = time.perf_counter()
    P.assemble(incremental=True, nthreads=1)
    t_fixed1 = time.perf_counter() - t0
    P.element_range(0, esample)
    t0 = time.perf_counter()
    P.assemble(incremental=True, nthreads=1)
    t_asm1 = t_fixed1 + max(0.0, time.perf_counter() - t0 - t_fixed1) * p.nelem / esample
    P.element_range(0, -1)
    t0 = time.perf_counter()
    O.cg(rp, ci, v, b, tol=0.0, max_iter=8, nthreads=1)
    t_iter1 = (time.perf_counter() - t0) / 9
    return {"P": P, "csr": (rp, ci, v, b), "x": x, "t_setup": t_setup, "t_asm": t_asm, "t_cg": t_cg,
            "iters": it, "t_iter": t_cg / (it + 1), "hist": hist, "neq": P.neq, "threads": threads,
            "t_asm1": t_asm1, "t_iter1": t_iter1}


def oracle_rate(leg, tol):
    """Assembly + solve throughput of the reference algorithm at tolerance
    tol: the timed full-size assembly plus the CG iterations that tolerance
    takes (from the residual history) at the timed cost per iteration."""
    import oracle as O
    its = O.iters_to(leg["hist"], tol)
    its = leg["iters"] if its is None else its
    t = leg["t_asm"] + leg["t_iter"] * (its + 1)
    return leg["neq"] / t, its, t


def assembly_roofline(p, S, asm_ms, hbm, src):
    """The mixed assembly against the HBM roofline with the algorithmic bytes
    of one assembly: coordinates, connectivity, per-element coefficients, DOF
    status and values, the FP64 values and their FP32 copy, the right-hand
    side; element matrices, contribution lists and element lists are
    implementation cost and not counted."""
    ncoef = 1 if p.kernel == "laplace" else 2
    b = (len(p.X) * p.X.shape[1] * 8 + p.nelem * p.conn.shape[1] * 4 + p.nelem * ncoef * 8 +
         S.ndofobj * p.ncomp * (1 + 8) + S.nnz * (8 + 4) + S.neq * 8)
    ach = b / (asm_ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm, "bytes": int(b),
            "ms": asm_ms, "peak_source": src, "kernels": "element phase + gather phase of one mixed assembly "
                                                       "(CUDA-event phase timers)"}


def run_reference(args):
    """--impl reference: the reference algorithm (the oracle restatement of
    inSilico's assembly and Eigen CG; the reference itself needs Eigen 3.2 /
    Boost 1.55, which are not available) on the host cores, on the same c2
    64^3 workload, metric and config as the GPU arm.  Setup (numbering,
    constraints, triplet pattern) is outside the timed steps, as on the GPU.
    The solve tolerance is chosen as on the GPU: the loosest of 1e-9..1e-12
    at which the FP64 CG solution is within 1e-8 of the FP64 solution to
    1e-12.  Each step is a bounded sample: the assembly of one eighth of the
    elements (the element loop's cost is linear in the elements), timed and
    scaled to all of them, plus 32 CG iterations on the full matrix, timed and
    scaled to the iteration count of that tolerance."""
    from insilico_gb300 import workloads as W
    import oracle as O
    threads = os.cpu_count() or 1
    world = int(os.environ.get("WORLD_SIZE", "1"))
    name = "c2"
    n = args.n or 64
    p = W.config(name, n=n)
    leg = oracle_leg(p, threads)
    rp, ci, v, b = leg["csr"]
    tol = REF_TOLS[-1]
    for t in REF_TOLS:
        xt, _, _ = O.cg(rp, ci, v, b, tol=t, nthreads=threads)
        if np.linalg.norm(xt - leg["x"]) <= ERR_BAR * np.linalg.norm(leg["x"]):
            tol = t
            break
    its = O.iters_to(leg["hist"], tol)
    kit = 32
    vals, steps = [], []
    P = leg["P"]
    esample = max(1, p.nelem // 8)
    for step in range(args.warmup + args.steps):
        # the per-assembly cost outside the element loop (clearing the values
        # and the right-hand side), then the element loop over the sample
        P.element_range(0, 0)
        t0 = time.perf_counter()
        P.assemble(incremental=True, nthreads=threads)
        t_fixed = time.perf_counter() - t0
        P.element_range(0, esample)
        t0 = time.perf_counter()
        P.assemble(incremental=True, nthreads=threads)
        t_asm = t_fixed + max(0.0, time.perf_counter() - t0 - t_fixed) * (p.nelem / esample)
        t0 = time.perf_counter()
        O.cg(rp, ci, v, b, tol=0.0, max_iter=kit, nthreads=threads)
        t_it = (time.perf_counter() - t0) / kit
        t_step = t_asm + t_it * (its + 1)
        if step >= args.warmup:
            vals.append(leg["neq"] / t_step)
            steps.append(t_step)
    val = float(statistics.median(vals))
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(statistics.median(steps)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Philox; no dataset)",
            "config": workload_config(name, n, leg["neq"], len(ci), p.nelem, world),
            "solve_tol": tol, "cg_iters": its, "assembly_s": leg["t_asm"], "cg_iter_s": leg["t_iter"],
            "setup_s": leg["t_setup"],
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"per step: the assembly of {esample} of the {p.nelem} elements (OpenMP, "
                                       f"{threads} threads), its element loop scaled to all, + {kit} Jacobi-CG "
                                       f"iterations on the full "
                                       f"{leg['neq']}-DOF matrix, scaled to the {its} iterations of tol {tol:g}; "
                                       f"numbering and pattern once, outside the steps (full assembly in setup: "
                                       f"{leg['t_asm']:.2f} s)"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def serve_batch_spmv(requests, local):
    """The dominant kernel of the served mixed path, timed alone: the batched
    FP32 SpMV of a batch built as the server builds one (the first 16 requests
    of the stream as instances of one context, FP32 tangent)."""
    from insilico_gb300 import _abi as A
    from insilico_gb300 import serve
    from insilico_gb300.system import System
    S = System(device=local)
    arrs = [serve.request_arrays(r) for r in requests]
    S.upload_batch(A.HEX, [(a["X"], a["conn"]) for a in arrs])
    S.create_field(1, 3)
    off = np.cumsum([0] + [len(a["X"]) for a in arrs])
    S.constrain(np.concatenate([a["node"] + off[k] for k, a in enumerate(arrs)]),
                np.concatenate([a["comp"] for a in arrs]), np.concatenate([a["val"] for a in arrs]))
    S.number_dofs()
    S.register_pattern()
    S.set_hyperelastic("neohooke", np.concatenate([a["lam"] for a in arrs]), np.concatenate([a["mu"] for a in arrs]), 3)
    S.set_option(A.OPT_BATCHED_SOLVE, 1)
    S.set_option(A.OPT_SPMV32_KIND, 104)
    S.assemble(A.PREC_FP32, incremental=True, with_residual=True)
    S.solve(A.SOLVE_CG_FP32_IR, tol=1e-6, check=False)
    ms = S.time_spmv(A.PREC_FP32, 30)
    b = spmv_bytes(S.nnz, S.neq, 4, 2 if S.get_option(A.OPT_SHORT_COLUMNS) else 4)
    out = {"ms": ms, "bytes": b, "neq": S.neq, "nnz": S.nnz, "instances": len(requests)}
    S.close()
    return out


def serve_request_spmv(requests, local):
    """The dominant kernel of the served mixed path with one request per
    batch, timed alone: the FP32 block SpMV (padded node blocks; the direction
    update folded in where the autotuned variant has it) of each of the given
    requests, each in its own context set up as the server sets one up.  The
    contexts' launches go round-robin, one launch each and no launch before
    it, so each matrix (up to about 130 MB) comes from HBM: the other
    contexts' matrices have pushed it out of L2."""
    from insilico_gb300 import _abi as A
    from insilico_gb300 import serve
    from insilico_gb300.system import System
    systems, nbytes = [], []
    for r in requests:
        a = serve.request_arrays(r)
        S = System(device=local)
        S.upload_mesh(A.HEX, a["X"], a["conn"])
        S.create_field(1, 3)
        S.constrain(a["node"], a["comp"], a["val"])
        S.number_dofs()
        S.register_pattern()
        S.set_hyperelastic("neohooke", a["lam"], a["mu"], 3)
        S.set_option(A.OPT_PERSISTENT, 0)
        S.assemble(A.PREC_FP32, incremental=True, with_residual=True)
        S.solve(A.SOLVE_CG_FP32_IR, tol=1e-6, check=False)
        S.time_spmv(A.PREC_FP32, 1)
        nbr = (r.side + 1) ** 2 * r.side  # DOF objects left active: all but the clamped x = 0 face
        kind = S.get_option(A.OPT_SPMV32_KIND) if not S.get_option(A.OPT_BLOCKED) else None
        folded = bool(S.get_option(A.OPT_BLOCKED)) and S.get_option(A.OPT_FOLD_DIRECTION) and \
            S.time_kernels(1)["block_kind"] in BSPMV_DIR_KERNEL
        col_b = 2 if (folded and S.get_option(A.OPT_SHORT_COLUMNS)) else 4
        nbytes.append(S.get_option(A.OPT_NBLOCKS) * (36 + col_b) + (16 if folded else 8) * 3 * nbr + 8 * ((nbr + 31) // 32))
        systems.append(S)
        assert kind is None, "c5 requests are node-blocked (padded blocks)"
    ms = 0.0
    rounds = 3
    for _ in range(rounds):
        for S in systems:
            ms += S.time_spmv(A.PREC_FP32, -1)
    out = {"ms": ms / (rounds * len(systems)), "bytes": sum(nbytes) / len(systems),
           "neq": int(np.mean([S.neq for S in systems])), "nblocks": int(np.mean([S.get_option(A.OPT_NBLOCKS) for S in systems])),
           "requests": len(systems), "sides": [r.side for r in requests], "folded": bool(folded)}
    for S in systems:
        S.close()
    return out


def run_serve(args, rank, world, local, pg):
    """c5: served neo-Hookean Newton requests (PulledSheet boundary conditions,
    5 load steps to stretch 1.3) through the native server.  The same seeded
    request stream runs through
      * the mixed server (--batch requests per batch, --slots batches at
        once; by default one request per batch and 8 at once, each request's
        FP32 block CG on padded node blocks): FP32 tangent + FP32 CG to 1e-6
        per Newton step (inexact Newton), FP64 residual;
      * the same server at the plain path's linear tolerance: FP64 + FP32
        matrices, FP32 CG with FP64 reliable updates to 1e-10;
      * the shared-launch server: batches of up to 12 requests sharing every
        launch of a Newton iteration (batched scalar CG), 4 batches at once,
        FP32 as the mixed server;
      * the plain path: one request per batch, FP64 tangent + FP64 CG (point
        Jacobi, CSR: the reference's algorithm) to 1e-10, 8 at once;
    closed loop (all requests queued at t = 0: throughput and latency under
    full load) and open loop (Poisson arrivals at half the plain path's
    closed-loop throughput)."""
    from insilico_gb300 import _abi as A
    from insilico_gb300 import serve
    A.load(build_if_missing=True)
    nreq = args.requests
    win = args.batch_window_us
    ratio = args.size_ratio
    arms = {
        "mixed": dict(precision=A.PREC_FP32, max_batch=args.batch, max_batches=args.slots, batch_window_us=win,
                      size_ratio=ratio),
        "mixed_equal_tol": dict(precision=A.PREC_MIXED, max_batch=args.batch, max_batches=args.slots, lin_tol=1e-10,
                                batch_window_us=win, size_ratio=ratio),
        "mixed_shared_launches": dict(precision=A.PREC_FP32, max_batch=12, max_batches=4, batch_window_us=20000),
        "plain": dict(precision=A.PREC_FP64, max_batch=1, max_batches=8),
    }
    for kw in arms.values():
        kw["persistent"] = args.persist
        kw["order"] = args.order
    if args.c5_mixed_only:  # configuration sweeps of the mixed server (no line is printed)
        arms = {"mixed": arms["mixed"]}
    out = {}
    clocks = None
    for m, kw in arms.items():
        srv = serve.Server(device=local, **kw)
        warm = serve.make_requests(max(3, args.slots), rate=0.0, seed=W_SEED_WARM, side_range=(8, 16))
        srv.run(warm, realtime=False)
        l0, b0 = srv.counters()
        srv.h2d_bytes = srv.d2h_bytes = 0
        clk = Clocks(local) if m == "mixed" else None
        done, wall = srv.run(serve.make_requests(nreq, rate=0.0), realtime=False)
        if clk is not None:
            clocks = clk.stop()
        l1, b1 = srv.counters()
        bad = [(r.rid, r.status, r.error) for r in done if r.status != A.ISL_OK]
        if bad:
            raise RuntimeError(f"c5 {m}: requests failed: {bad[:3]}")
        out[m] = {"closed": serve.latency_stats(done, wall), "u": {r.rid: r.u for r in done},
                  "converged": all(r.converged for r in done), "launches": l1 - l0, "batches": b1 - b0,
                  "h2d": srv.h2d_bytes, "d2h": srv.d2h_bytes, "srv": srv, "times": srv.times()}
        log(f"c5 {m} closed loop: {out[m]['closed']} host: {out[m]['times']}")
    if args.c5_mixed_only:
        out["mixed"]["srv"].close()
        return
    rate = 0.5 * out["plain"]["closed"]["solves_per_s"]
    for m in ("plain", "mixed"):
        done, wall = out[m]["srv"].run(serve.make_requests(nreq, rate=rate), realtime=True)
        out[m]["open"] = serve.latency_stats(done, wall)
        log(f"c5 {m} open loop at {rate:.2f}/s: {out[m]['open']}")
    for m in arms:
        out[m]["srv"].close()
    reqs = serve.make_requests(nreq, rate=0.0)
    if args.batch == 1:
        big = sorted(reqs, key=lambda q: -q.side)[:8]
        sp = serve_request_spmv(big, local)
        sp_kernel = ("k_bspmv_dir<U,MINB>" if sp["folded"] else "k_bspmv") + \
            f" (FP32 padded 3x3 block SpMV of one request, the 8 largest of the stream, sides {sp['sides']}, " \
            "launched round-robin from HBM)"
        sp_batch = {k: sp[k] for k in ("neq", "nblocks", "requests")}
    else:
        sp = serve_batch_spmv(reqs[:16], local)
        sp_kernel = "kb_sspmv<4,8> (batched FP32 SpMV of a 16-request batch, all instances active)"
        sp_batch = {k: sp[k] for k in ("neq", "nnz", "instances")}
    hbm, src = peaks()
    ach = sp["bytes"] / (sp["ms"] * 1e-3) / 1e9
    cpu, err_oracle = None, None
    if rank == 0 and world == 1 and not args.no_cpu:
        # the reference algorithm (the oracle running the reference driver:
        # assembly + Jacobi CG to 1e-10 per Newton step) on the first request
        # of the same stream, with all host threads
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from helpers import oracle_newton_driver
        threads = os.cpu_count() or 1
        r0 = reqs[0]
        t0 = time.perf_counter()
        u0, _ = oracle_newton_driver(r0, serve.NEWTON_TOL, serve.MAX_NEWTON, lin_tol=1e-10, nthreads=threads)
        tc = time.perf_counter() - t0
        err_oracle = {m: float(np.linalg.norm(out[m]["u"][r0.rid] - u0) / np.linalg.norm(u0)) for m in arms}
        cpu = {"value": 1.0 / tc, "unit": "requests/s", "cores": threads, "kind": "port",
               "sample": f"request 0 of the stream (side {r0.side}, {3 * (r0.side + 1) ** 3} DOF components, "
                         f"5 load steps) through the oracle's run of the reference driver with Jacobi CG to 1e-10: "
                         f"{tc:.1f} s"}

    def errs_vs_plain(m):
        e = [float(np.linalg.norm(out[m]["u"][rid] - u) / max(np.linalg.norm(u), 1e-300))
             for rid, u in out["plain"]["u"].items()]
        return {"max": max(e), "median": float(np.median(e))}
    mc, pc, ec = out["mixed"]["closed"], out["plain"]["closed"], out["mixed_equal_tol"]["closed"]
    line = {"metric": "served Newton requests/s (closed loop), every request converged by the reference's Newton "
                      "test (||R||/N or ||dU||/N < 1e-12); p50/p99 latency",
            "value": mc["solves_per_s"] * world, "unit": "requests/s", "n_gpus": world, "steps": nreq,
            "warmup": max(3, args.slots), "ms_per_step": 1e3 * mc["wall_s"] / nreq, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded Philox; no dataset)",
            "config": {"workload": "c5 served hex8 neo-Hookean Newton requests, side U{8..48}, mu log-U[0.1,10], "
                                   "kappa = 10 mu, 5 load steps to stretch 1.3",
                       "requests": nreq, "parallelism": "replicas" if world > 1 else "single",
                       "l2": "per-request meshes are set up, assembled and solved from host inputs"},
            "method": (f"native server: one request per batch, {args.slots} at once, each request's FP32 block CG "
                       f"(padded 3x3 node blocks, block Jacobi) on its own stream" if args.batch == 1 else
                       f"native server: batches of up to {args.batch} requests share every launch of a Newton "
                       f"iteration, {args.slots} batches at once, batching window {win} us") +
                      "; FP32 tangent + FP32 CG to 1e-6, FP64 residual; plain: one request per batch, 8 at once, "
                      "FP64 tangent + FP64 point-Jacobi CSR CG to 1e-10",
            "mixed_shared_launches": {"requests_per_s": out["mixed_shared_launches"]["closed"]["solves_per_s"],
                                      "p50": out["mixed_shared_launches"]["closed"]["p50_s"],
                                      "p99": out["mixed_shared_launches"]["closed"]["p99_s"],
                                      "cg_iters": out["mixed_shared_launches"]["closed"]["cg_iters"],
                                      "batches": out["mixed_shared_launches"]["batches"],
                                      "config": "batches of up to 12 requests sharing every launch (batched scalar "
                                                "FP32 CG), 4 at once, batching window 20 ms"},
            "server_host_seconds": {m: out[m]["times"] for m in arms},
            "latency_s": {"mixed_closed": {"p50": mc["p50_s"], "p99": mc["p99_s"]},
                          "plain_closed": {"p50": pc["p50_s"], "p99": pc["p99_s"]},
                          "open_loop_rate_per_s": rate,
                          "mixed_open": {"p50": out["mixed"]["open"]["p50_s"], "p99": out["mixed"]["open"]["p99_s"]},
                          "plain_open": {"p50": out["plain"]["open"]["p50_s"], "p99": out["plain"]["open"]["p99_s"]}},
            "plain_fp64": {"requests_per_s": pc["solves_per_s"], "newton_iters": pc["newton_iters"],
                           "cg_iters": pc["cg_iters"], "batches": out["plain"]["batches"]},
            "mixed": {"newton_iters": mc["newton_iters"], "cg_iters": mc["cg_iters"], "batches": out["mixed"]["batches"],
                      "max_batch": mc["max_batch"]},
            "mixed_equal_lin_tol": {"requests_per_s": ec["solves_per_s"], "p50": ec["p50_s"], "p99": ec["p99_s"],
                                    "newton_iters": ec["newton_iters"], "cg_iters": ec["cg_iters"],
                                    "speedup_vs_plain_fp64": ec["solves_per_s"] / pc["solves_per_s"],
                                    "rel_err_vs_plain_fp64": errs_vs_plain("mixed_equal_tol")},
            "speedup_vs_plain_fp64": mc["solves_per_s"] / pc["solves_per_s"],
            "rel_err_vs_fp64": errs_vs_plain("mixed"), "rel_err_vs_oracle_request0": err_oracle,
            "rel_err_note": "against the plain FP64 server's results: two Newton solutions that both meet the "
                            "reference's stop test differ by about K^-1 R, up to 1e-7 of ||u|| for the softest "
                            "requests at inexact (1e-6) linear solves; at the plain path's linear tolerance "
                            "(mixed_equal_lin_tol) the difference is below 1e-9",
            "converged": all(out[m]["converged"] for m in arms),
            "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                         "traffic": None, "kernel": sp_kernel,
                         "bytes_per_launch": sp["bytes"], "ms_per_launch": sp["ms"], "peak_source": src,
                         "batch": sp_batch},
            "cpu_baseline": cpu,
            "e2e": {"value": mc["solves_per_s"] * world, "unit": "requests/s",
                    "h2d_bytes_per_step": int(out["mixed"]["h2d"] / nreq),
                    "d2h_bytes_per_step": int(out["mixed"]["d2h"] / nreq)},
            "clocks": clocks, "gpu_launches": int(out["mixed"]["launches"])}
    if rank == 0:
        print(json.dumps(line), flush=True)


W_SEED_WARM = 0x15111C0 + 40


def run_heat(args, rank, world, local, pg):
    """heat: nonlinear heat conduction (heat::Static, FenicsTest conductivity
    (1 + u)^3) on the n x n unit square in Q2; n = 200 is the square_200 mesh of
    reference/04-heat/nonlinearHeat.cpp.  One step is the whole Newton run from
    u = 0: assemble the non-symmetric tangent and the residual, BiCGSTAB to
    1e-11, add the increment (4 assemblies, 3 solves)."""
    from insilico_gb300 import _abi as A
    from insilico_gb300 import workloads as W
    from insilico_gb300.system import System
    A.load(build_if_missing=True)
    n = args.n or 200
    X, conn = W.unit_cube("quad", n, n)
    S = System(device=local)
    t0 = time.perf_counter()
    ndofs = W.heat_setup(S, X, conn)
    t_setup = time.perf_counter() - t0
    zeros = np.zeros(S.ndofobj)

    lin = []

    def step():
        S.set_values(zeros)
        lin.clear()
        return W.heat_newton(S, ndofs, lin_iters=lin)
    for _ in range(max(3, args.warmup)):
        rows = step()
    S.sync()
    clk = Clocks(local)
    l0 = S.launch_count()
    S.set_timing(True)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        rows = step()
        S.sync()
        times.append(time.perf_counter() - t0)
    ms, cnt = S.timings()
    S.set_timing(False)
    clocks = clk.stop()
    launches = S.launch_count() - l0
    s_step = max_over_ranks(float(np.median(times)), pg)
    newton = len(rows) - 1
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        import oracle as O
        t0 = time.perf_counter()
        nc, rows_c, _, _ = O.nonlinear_heat(X, conn)
        tc = time.perf_counter() - t0
        cpu = {"value": nc / tc, "unit": "DOF/s", "cores": 1, "kind": "port",
               "sample": f"the whole Newton run on the same {n}x{n} Q2 mesh: oracle assembly (1 thread) + "
                         f"scipy SuperLU of the non-symmetric tangent, {len(rows_c) - 1} iterations, {tc:.1f} s"}
    line = {"metric": "nonlinear heat Newton run (heat::Static, BiCGSTAB) DOF/s", "value": ndofs * world / s_step,
            "unit": "DOF/s", "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup),
            "ms_per_step": s_step * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (unit square; no dataset)",
            "config": {"workload": f"heat: Q2 heat::Static FenicsTest m=3 on the {n}x{n} unit square, u=0 at x=0, "
                                   f"u=1 at x=1, Newton to 1e-8, BiCGSTAB (Jacobi) to 1e-11",
                       "dofs": int(ndofs), "elements": int(len(conn)), "parallelism": "single",
                       "l2": "matrix and vectors resident; per step the DOF values are reset from the host"},
            "newton_iters": newton, "residuals": [r[1] for r in rows], "setup_s": t_setup,
            "bicgstab_iters": list(lin), "bicgstab_spmv": int(S.get_option(A.OPT_BICGSTAB_KIND)),
            "phase_ms_per_step": {"element": ms[A.T_ELEMENT] / args.steps, "gather": ms[A.T_GATHER] / args.steps,
                                  "solve": ms[A.T_SOLVE] / args.steps},
            "cpu_baseline": cpu,
            "e2e": {"value": ndofs * world / s_step, "unit": "DOF/s", "h2d_bytes_per_step": int(zeros.nbytes),
                    "d2h_bytes_per_step": int(2 * newton * ndofs * 8 + ndofs * 8)},
            "clocks": clocks, "gpu_launches": int(launches // max(1, args.steps))}
    S.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


def batch_instances(count, seed):
    """c4 instances: side U{8..256}, degree Q1/Q2 with p = 0.5, per instance
    kappa_e = exp(N(0, 0.5)) and nodal source U[0, 1] (seeded streams)."""
    from insilico_gb300 import workloads as W
    sides = W.rng(seed, 0).integers(8, 257, count)
    degs = np.where(W.rng(seed, 1).uniform(0.0, 1.0, count) < 0.5, 1, 2)
    return [(k, int(sides[k]), int(degs[k])) for k in range(count)]


def batch_groups(inst, pair_budget=1_300_000_000):
    """Contexts of one degree each whose element-pair lists stay within the
    32-bit contribution indices (pairs = elements x local functions^2)."""
    groups = []
    for deg in (1, 2):
        nloc2 = (deg + 1) ** 4
        cur, tot = [], 0
        for k, s, d in inst:
            if d != deg:
                continue
            pairs = s * s * nloc2
            if cur and tot + pairs > pair_budget:
                groups.append((deg, cur))
                cur, tot = [], 0
            cur.append((k, s))
            tot += pairs
        if cur:
            groups.append((deg, cur))
    return groups


def run_batch(args, rank, world, local, pg):
    """c4: batched Q1/Q2 Poisson instances (C1-style data), assembly + per-
    instance CG to 1e-8 (mixed: FP32 CG + FP64 refinement; plain: FP64 CG),
    one context per group of instances, all contexts resident.  The groups'
    assemblies and solves run concurrently: one host thread and one CUDA
    stream per context."""
    import concurrent.futures as cf
    from insilico_gb300 import _abi as A
    from insilico_gb300 import workloads as W
    from insilico_gb300.system import System
    A.load(build_if_missing=True)
    seed = W.SEED_BASE + 3
    inst = batch_instances(args.instances, seed)
    groups = batch_groups(inst)
    systems, coefs = [], []
    t_setup = time.perf_counter()
    for deg, members in groups:
        S = System(device=local)
        meshes, kappa, body = [], [], []
        for k, s in members:
            X, conn = W.unit_cube("quad", s, s)
            meshes.append((X, conn))
            kappa.append(np.exp(W.rng(seed, 16 + 2 * k).normal(0.0, 0.5, len(conn))))
            body.append(W.rng(seed, 17 + 2 * k).uniform(0.0, 1.0, len(X))[:, None])
        S.upload_batch(A.QUAD, meshes)
        S.create_field(deg, 1)
        S.constrain_boundary(lambda x: (np.ones((len(x), 1), dtype=bool), 0.0))
        S.number_dofs()
        S.register_pattern()
        coefs.append((np.concatenate(kappa), 2 * deg))
        S.set_laplace(*coefs[-1])
        S.set_body_force_nodal(np.concatenate(body))
        S.set_option(A.OPT_RELIABLE_DROP, args.reliable_drop)
        del meshes, kappa, body
        systems.append(S)
        log(f"c4 group Q{deg}: {len(members)} instances, {S.nelem} elements, {S.neq} DOFs, {S.nnz} nnz")
    t_setup = time.perf_counter() - t_setup
    neq = sum(S.neq for S in systems)
    nnz = sum(S.nnz for S in systems)
    tol = 1e-8
    pool = cf.ThreadPoolExecutor(max_workers=len(systems))

    def on_all(fn):
        """fn(context index, context) on every context at once (ctypes releases
        the GIL inside the library, so each context drives its own stream)."""
        list(pool.map(lambda kv: fn(*kv), enumerate(systems)))

    def one(mixed, k, S, upload=False, download=False):
        if upload:
            S.set_laplace(*coefs[k])
        S.assemble(A.PREC_MIXED if mixed else A.PREC_FP64)
        S.solve(A.SOLVE_CG_FP32_IR if mixed else A.SOLVE_CG_FP64, tol=tol)
        if download:
            return S.solution()
        S.sync()

    def timed(mixed, steps, **kw):
        for S in systems:
            S.sync()
        t0 = time.perf_counter()
        for _ in range(steps):
            on_all(lambda k, S: one(mixed, k, S, **kw))
        return (time.perf_counter() - t0) / steps

    for _ in range(args.warmup):
        on_all(lambda k, S: one(True, k, S))
    if args.profile:
        # one mixed step inside the profiler range (ncu --profile-from-start off)
        import ctypes
        cudart = ctypes.CDLL("libcudart.so.13")  # already loaded by libisl_gpu.so
        for S in systems:
            S.sync()
        cudart.cudaProfilerStart()
        on_all(lambda k, S: one(True, k, S))
        cudart.cudaProfilerStop()
        for S in systems:
            S.close()
        return
    # accuracy: mixed and plain at the c4 tolerance against a tight FP64 solve
    errs, errs64 = [], []
    for S in systems:
        S.assemble(A.PREC_MIXED)
        S.solve(A.SOLVE_CG_FP64, tol=1e-12)
        xt = S.solution()
        S.solve(A.SOLVE_CG_FP64, tol=tol)
        x64 = S.solution()
        S.solve(A.SOLVE_CG_FP32_IR, tol=tol)
        xm = S.solution()
        eq_off, _ = S.batch_info()
        for k in range(len(eq_off) - 1):
            a, b = eq_off[k], eq_off[k + 1]
            nt = max(np.linalg.norm(xt[a:b]), 1e-300)
            errs.append(float(np.linalg.norm(xm[a:b] - xt[a:b]) / nt))
            errs64.append(float(np.linalg.norm(x64[a:b] - xt[a:b]) / nt))
    l0 = sum(S.launch_count() for S in systems)
    clk = Clocks(local)
    s_mixed = timed(True, args.steps)
    clocks = clk.stop()
    launches = (sum(S.launch_count() for S in systems) - l0) // max(1, args.steps)
    s_plain = timed(False, max(1, args.steps // 2))
    # e2e through the C-ABI with host buffers: per step every group's
    # conductivity table goes up, assembly and solve run, the solutions come back
    e2e_s = timed(True, args.steps, upload=True, download=True)
    h2d = sum(c[0].nbytes for c in coefs)
    # assembly share (one context at a time, CUDA-event phase timers)
    asm_ms = 0.0
    for S in systems:
        S.set_timing(True)
        S.assemble(A.PREC_MIXED)
        S.solve(A.SOLVE_CG_FP32_IR, tol=tol)
        ms, _ = S.timings()
        asm_ms += ms[A.T_ELEMENT] + ms[A.T_GATHER]
        S.set_timing(False)
    iters = np.concatenate([S.batch_stats()[0] for S in systems])
    # dominant kernel: the batched FP32 SpMV with every instance active, per
    # context; achieved = the contexts' algorithmic bytes over their summed times
    hbm, src = peaks()
    sp_ms, sp_bytes, kinds = 0.0, 0, []
    for S in systems:
        sp_ms += S.time_spmv(A.PREC_FP32, 20)
        sp_bytes += spmv_bytes(S.nnz, S.neq, 4, 2 if S.get_option(A.OPT_SHORT_COLUMNS) else 4)
        kinds.append(S.get_option(A.OPT_SPMV32_KIND))
    ach = sp_bytes / (sp_ms * 1e-3) / 1e9
    kname = ", ".join(sorted({("kb_sspmv<%d,%d>" % (k - 100, 8 if k < 108 else 6)) if k >= 100 else
                              f"kb_spmv<float,float,{k}>" for k in kinds}))
    for S in systems:
        S.close()
    pool.shutdown()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = batch_cpu_sample(inst, seed, tol)
    line = {"metric": METRIC, "value": neq * world / s_mixed, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": s_mixed * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded Philox; no dataset)",
            "config": {"workload": f"c4 {args.instances} batched Poisson instances (unit square, side U{{8..256}}, "
                                   "Q1/Q2 p = 0.5, kappa_e = exp(N(0,0.5)), nodal source U[0,1], g = 0), tol 1e-8",
                       "active_dofs": int(neq), "nnz": int(nnz), "contexts": len(systems),
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (FP32 CSR %.1f GB)" % (nnz * 8 / 1e9)},
            "method": "mixed FP32 CG + FP64 reliable updates per instance (when the FP32 r.r has dropped "
                      f"1e{args.reliable_drop}x since the last one); contexts concurrent (one stream each)",
            "assembly_ms": asm_ms, "assembly_gdofs": neq / (asm_ms * 1e-3) / 1e9, "setup_s": t_setup,
            "plain_fp64": {"ms_per_step": s_plain * 1e3, "dofs_per_s": neq / s_plain},
            "speedup_vs_plain_fp64": s_plain / s_mixed,
            "rel_err_vs_fp64": {"max": max(errs), "median": float(np.median(errs)),
                                "plain_fp64_max": max(errs64), "reference": "GPU FP64 CG to 1e-12 per instance"},
            "cg_iters": {"min": int(iters.min()), "median": int(np.median(iters)), "max": int(iters.max())},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                         "traffic": (lambda r: None if r is None else r * sp_bytes)(ncu_traffic_ratio("spmv_fp32_c4")),
                         "kernel": kname + " (batched FP32 SpMV, all instances)",
                         "bytes_per_launch": sp_bytes, "ms_per_launch": sp_ms, "peak_source": src},
            "cpu_baseline": cpu,
            "e2e": {"value": neq * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(neq * 8), "ms_per_step": e2e_s * 1e3},
            "clocks": clocks, "gpu_launches": int(launches)}
    if rank == 0:
        print(json.dumps(line), flush=True)


def batch_cpu_sample(inst, seed, tol, budget_s=20.0):
    """The reference algorithm (oracle) on the first instances of the c4
    stream, in stream order, with all host threads: assembly + Jacobi CG to
    tol per instance, until budget_s is spent."""
    import oracle as O
    from insilico_gb300 import _abi as A
    from insilico_gb300 import workloads as W
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import oracle_problem
    threads = os.cpu_count() or 1
    dofs, t, done = 0, 0.0, []
    for k, side, deg in inst:
        X, conn = W.unit_cube("quad", side, side)
        p = W.Problem("inst", A.QUAD, X, conn, deg, 1, "laplace", 2 * deg,
                      kappa=np.exp(W.rng(seed, 16 + 2 * k).normal(0.0, 0.5, len(conn))),
                      body=W.rng(seed, 17 + 2 * k).uniform(0.0, 1.0, len(X))[:, None],
                      dirichlet=lambda x: (np.ones((len(x), 1), dtype=bool), 0.0))
        P, _ = oracle_problem(p, assemble=False)
        P.pattern()
        t0 = time.perf_counter()
        rp, ci, v, b = P.assemble(incremental=True, nthreads=threads)
        O.cg(rp, ci, v, b, tol=tol, nthreads=threads)
        t += time.perf_counter() - t0
        dofs += P.neq
        done.append(f"Q{deg} side {side}")
        if t >= budget_s:
            break
    return {"value": dofs / t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"oracle assembly + Jacobi CG to {tol:g} of the first {len(done)} instances of the stream "
                      f"({', '.join(done)}; {dofs} DOFs, {t:.1f} s); numbering and pattern outside"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--n", type=int, default=0, help="mesh size (default: the workload's own, 64)")
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5", "heat"],
                    help="c2 (default, the headline): hex8 elasticity 64^3; c1: Q1 Poisson 64^2; c3: tet10 Poisson "
                         "64^3; c4: 4096 batched Q1/Q2 Poisson instances; c5: served neo-Hookean Newton requests; "
                         "heat: nonlinear heat Newton run (heat::Static, BiCGSTAB), square 200")
    ap.add_argument("--requests", type=int, default=48, help="c5: requests per run")
    ap.add_argument("--slots", type=int, default=8, help="c5: batches the mixed server runs at once")
    ap.add_argument("--batch", type=int, default=1, help="c5: requests per batch of the mixed server")
    ap.add_argument("--order", type=int, default=0,
                    help="c5: 1 starts batches from the largest queued request (isl_serve_config.order)")
    ap.add_argument("--reliable-drop", type=int, default=2,
                    help="c4: reliable update after the FP32 r.r drops by 10^value (ISL_OPT_RELIABLE_DROP)")
    ap.add_argument("--persist", type=int, default=0,
                    help="c5: 1 lets single-request batches solve small systems in one launch (ISL_OPT_PERSISTENT)")
    ap.add_argument("--batch-window-us", type=int, default=20000, help="c5: batching window of the mixed server")
    ap.add_argument("--size-ratio", type=float, default=0.0,
                    help="c5: > 1 batches only requests within this element-count factor of the batch's first")
    ap.add_argument("--c5-mixed-only", action="store_true", help="c5: the mixed server's closed loop only (sweeps)")
    ap.add_argument("--instances", type=int, default=4096, help="c4: batched instances")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile", action="store_true",
                    help="profiling run: setup + the mixed steps only (no calibration, plain arm, e2e or CPU legs)")
    ap.add_argument("--tol", type=float, default=1e-10)
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    if args.workload == "c5":
        run_serve(args, rank, world, local, pg)
    elif args.workload == "heat":
        run_heat(args, rank, world, local, pg)
    elif args.workload == "c4":
        run_batch(args, rank, world, local, pg)
    else:
        run_single(args, rank, world, local, pg)
    if pg:
        pg.destroy_process_group()


def run_single(args, rank, world, local, pg):
    """c1 / c2 / c3: one system, assembly + solve per step."""

    from insilico_gb300 import _abi as A
    from insilico_gb300 import workloads as W

    A.load(build_if_missing=True)
    args.n = args.n or 64
    p = W.config(args.workload, n=args.n)
    from insilico_gb300.system import System
    S = W.setup_system(p, System(device=local))
    neq, nnz = S.neq, S.nnz
    log(f"setup neq={neq} nnz={nnz} blocked={S.get_option(A.OPT_BLOCKED)}")
    if args.profile:
        # the profiler range (ncu --profile-from-start off) covers the steps
        # after the warm-up ones, so autotuning and first-touch work stay out
        import ctypes
        cudart = ctypes.CDLL("libcudart.so.13")  # already loaded by libisl_gpu.so
        for k in range(args.warmup + args.steps):
            if k == args.warmup:
                S.sync()
                cudart.cudaProfilerStart()
            S.assemble(A.PREC_MIXED)
            it, rr, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=args.tol)
            log(f"profile step {k}: iters {it} relres {rr:.2e}")
        S.sync()
        cudart.cudaProfilerStop()
        S.close()
        return
    threads = os.cpu_count() or 1
    # the FP64 oracle solution: the reference algorithm on the host cores
    # (rank 0 of a single-GPU run; replicas and --no-cpu fall back to a tight
    # FP64 GPU solve, and say so)
    leg = None
    if rank == 0 and world == 1 and not args.no_cpu:
        t0 = time.perf_counter()
        leg = oracle_leg(p, threads)
        log(f"oracle leg: setup {leg['t_setup']:.1f}s assembly {leg['t_asm']:.2f}s cg {leg['t_cg']:.1f}s "
            f"({leg['iters']} iters) total {time.perf_counter() - t0:.1f}s")
        assert leg["neq"] == neq
    S.assemble(A.PREC_MIXED)
    if leg is not None:
        x_ref, ref_kind = leg["x"], f"oracle FP64 CG to {ORACLE_TOL:g} (reference algorithm, host)"
    else:
        S.solve(A.SOLVE_CG_FP64, tol=1e-13)
        x_ref, ref_kind = S.solution(), "GPU FP64 CG to 1e-13 (no oracle run)"
    tol64, err64, it64 = calibrate(S, A.SOLVE_CG_FP64, x_ref, REF_TOLS)
    tolm, errm, itm = calibrate(S, A.SOLVE_CG_FP32_IR, x_ref, REF_TOLS)

    def step_mixed():
        S.assemble(A.PREC_MIXED)
        return S.solve(A.SOLVE_CG_FP32_IR, tol=tolm)

    def step_plain():
        S.assemble(A.PREC_FP64)
        return S.solve(A.SOLVE_CG_FP64, tol=tol64)

    for _ in range(args.warmup):
        step_mixed()
    # matrix (FP64 + FP32 values, indices), staging and vectors against L2
    working_set = nnz * 16 + p.nelem * 8 * 300 + neq * 8 * 12
    flush_l2 = working_set < 2 * L2_BYTES
    launches0 = S.launch_count()
    clk = Clocks(local)
    if pg:
        pg.barrier()
    S.sync()
    its = []
    if flush_l2:
        # the working set fits in L2: every timed step starts from a flushed
        # L2 and is timed on its own (the flush is outside the timed region)
        ms_total = 0.0
        for _ in range(args.steps):
            l2_flush(local)
            S.mark(0)
            its.append(step_mixed()[0])
            S.mark(1)
            S.sync()
            ms_total += S.elapsed_ms(0, 1)
    else:
        S.mark(0)
        for _ in range(args.steps):
            its.append(step_mixed()[0])
        S.mark(1)
        S.sync()
        ms_total = S.elapsed_ms(0, 1)
    clocks = clk.stop()
    launches = S.launch_count() - launches0
    x_m = S.solution()
    err_m = float(np.linalg.norm(x_m - x_ref) / np.linalg.norm(x_ref))
    ms_total = max_over_ranks(ms_total, pg)
    ms_step = ms_total / args.steps
    value = neq * world / (ms_step / 1e3)
    log(f"timed: {ms_step:.2f} ms/step, inner iters {its}, err {err_m:.3e}")

    # phase split of one mixed step and the plain FP64 path
    S.set_timing(True)
    step_mixed()
    ms, cnt = S.timings()
    S.set_timing(False)
    asm_ms = ms[A.T_ELEMENT] + ms[A.T_GATHER]
    solve_ms_m = ms[A.T_SOLVE]
    S.mark(2)
    for _ in range(2):
        it_plain = step_plain()[0]
    S.mark(3)
    plain_ms = S.elapsed_ms(2, 3) / 2
    x_p = S.solution()
    err_p = float(np.linalg.norm(x_p - x_ref) / np.linalg.norm(x_ref))
    S.set_timing(True)
    step_plain()
    ms64, _ = S.timings()
    S.set_timing(False)
    asm64_ms = ms64[A.T_ELEMENT] + ms64[A.T_GATHER]

    # what the speed-up is made of: the mixed solve with the plain path's
    # point-Jacobi preconditioner and scalar CSR matrix (precision alone),
    # against the node-block format with block Jacobi
    split = None
    if S.get_option(A.OPT_BLOCKED):
        S.set_option(A.OPT_BLOCK_SOLVER, 0)
        S.assemble(A.PREC_MIXED)
        tolq, errq, _ = calibrate(S, A.SOLVE_CG_FP32_IR, x_ref, REF_TOLS)
        step_mixed_point = lambda: (S.assemble(A.PREC_MIXED), S.solve(A.SOLVE_CG_FP32_IR, tol=tolq))[1]  # noqa: E731
        step_mixed_point()
        S.mark(4)
        for _ in range(2):
            it_q = step_mixed_point()[0]
        S.mark(5)
        point_ms = S.elapsed_ms(4, 5) / 2
        S.set_option(A.OPT_BLOCK_SOLVER, 1)
        split = {"mixed_point_jacobi_csr": {"ms_per_step": point_ms, "iters": it_q, "solve_tol": tolq,
                                            "rel_err_vs_fp64": errq},
                 "precision_alone": plain_ms / point_ms,
                 "block_format_and_block_jacobi": point_ms / ms_step,
                 "note": "plain FP64 (point Jacobi, CSR) -> mixed with the same point Jacobi and CSR (precision "
                         "alone) -> mixed with 3x3 node blocks and block Jacobi"}
        # the same block solve with the direction update as its own kernel
        S.assemble(A.PREC_MIXED)
        S.set_option(A.OPT_FOLD_DIRECTION, 0)
        step_mixed()
        S.mark(4)
        for _ in range(2):
            it_s = step_mixed()[0]
        S.mark(5)
        S.set_option(A.OPT_FOLD_DIRECTION, 1)
        sep_ms = S.elapsed_ms(4, 5) / 2
        split["separate_direction_kernel"] = {"ms_per_step": sep_ms, "iters": it_s,
                                              "folded_gain": sep_ms / ms_step}
        log(f"split: {split}")

    # dominant kernel: FP32 SpMV of the inner CG, timed alone (CUDA events)
    S.assemble(A.PREC_MIXED)
    spmv32_ms = S.time_spmv(A.PREC_FP32, 50)
    spmv64_ms = S.time_spmv(A.PREC_FP64, 50)
    kernels = S.time_kernels(30)
    kernels["update_kind"] = (S.get_option(A.OPT_BLOCK_UPDATE) or 1) if S.get_option(A.OPT_BLOCKED) else 0
    log("kernel ms:", {k: round(v, 4) for k, v in kernels.items()})
    hbm, src = peaks()
    blocked = S.get_option(A.OPT_BLOCKED)
    if blocked:
        # 3x3 blocks: 36 B of values + 4 B of column id per block, x and y once;
        # with the direction update folded in, x is formed from z and the
        # previous direction (both read once) and written once
        nblk, nslot = S.get_option(A.OPT_NBLOCKS), S.get_option(A.OPT_NSLOTS)
        bkind = int(kernels["block_kind"])
        folded = bool(S.get_option(A.OPT_FOLD_DIRECTION)) and bkind in BSPMV_DIR_KERNEL
        col_b = 2 if (folded and S.get_option(A.OPT_SHORT_COLUMNS)) else 4  # 16-bit column offsets
        b32 = nblk * (36 + col_b) + (4 if folded else 2) * neq * 4 + 8 * ((neq // 3 + 31) // 32)
        if folded:
            kname = BSPMV_DIR_KERNEL[bkind] + " (sliced-ELL 3x3 FP32 blocks" + \
                (", 16-bit column offsets" if col_b == 2 else "") + \
                ", inner CG SpMV with the block-Jacobi direction update folded in, autotuned variant)"
        else:
            kname = BSPMV_KERNEL.get(bkind, "k_bspmv") + " (sliced-ELL 3x3 FP32 blocks, inner CG SpMV, autotuned variant)"
    else:
        nblk, nslot = 0, S.get_option(A.OPT_SCALAR_SLOTS)
        b32 = spmv_bytes(nnz, neq, 4, 2 if S.get_option(A.OPT_SHORT_COLUMNS) else 4)
        kind = S.get_option(A.OPT_SPMV32_KIND)
        if kind >= 100:
            kname = SSPMV_KERNEL.get(kind, "k_sspmv_batch") + \
                " (scalar sliced-ELL FP32, rows length-sorted in windows of 2048" + \
                (", 16-bit column offsets" if S.get_option(A.OPT_SHORT_COLUMNS) else "") + ", inner CG SpMV, autotuned)"
        else:
            kname = f"k_spmv_pap<float,float,{kind}> (FP32 CSR, {kind} lanes per row, inner CG SpMV, autotuned)"
    ach = b32 / (spmv32_ms * 1e-3) / 1e9
    traffic = ncu_traffic(f"spmv_fp32_{args.workload}")

    # e2e through the C-ABI with host buffers: per step upload the element
    # material table, assemble, solve, download the solution
    if p.kernel == "laplace":
        coef = [p.kappa.copy()]
        upload = lambda: S.set_laplace(coef[0], p.qdeg)  # noqa: E731
    else:
        coef = [p.lam.copy(), p.mu.copy()]
        upload = lambda: S.set_hyperelastic(p.material, coef[0], coef[1], p.qdeg)  # noqa: E731
    upload()
    step_mixed()
    S.solution()
    S.sync()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        upload()
        step_mixed()
        S.solution()
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e = {"value": neq * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(sum(c.nbytes for c in coef)),
           "d2h_bytes_per_step": int(neq * 8), "ms_per_step": e2e_s * 1e3}

    cpu = None
    if leg is not None:
        rate, its_cpu, t_cpu = oracle_rate(leg, tol64)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"the full workload on the oracle: assembly timed ({leg['t_asm']:.2f} s, OpenMP) + Jacobi CG "
                         f"to {ORACLE_TOL:g} timed ({leg['t_cg']:.1f} s, {leg['iters']} iterations), counted at the "
                         f"{its_cpu} iterations of the plain path's tolerance {tol64:g}; numbering and pattern "
                         f"({leg['t_setup']:.1f} s) outside, as on the GPU",
               "assembly_s": leg["t_asm"], "cg_iter_s": leg["t_iter"], "cg_iters": its_cpu, "step_s": t_cpu,
               "one_thread": {"value": neq / (leg["t_asm1"] + leg["t_iter1"] * (its_cpu + 1)), "unit": UNIT,
                              "assembly_s": leg["t_asm1"], "cg_iter_s": leg["t_iter1"],
                              "sample": "assembly of 1/32 of the elements and 8 CG iterations on one thread, "
                                        "scaled to the full step"}}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded Philox; no dataset)",
        "config": workload_config(args.workload, args.n, neq, nnz, p.nelem, world),
        "method": "mixed FP32 CG + FP64 reliable updates" + (", 3x3 node blocks + block Jacobi" if blocked else ""),
        "assembly_gdofs": neq / (asm_ms * 1e-3) / 1e9, "assembly_ms": asm_ms, "solve_ms": solve_ms_m,
        "solve_tol": tolm, "inner_iters_per_step": int(np.median(its)), "rel_err_vs_fp64": err_m,
        "fp64_reference": ref_kind,
        "plain_fp64": {"ms_per_step": plain_ms, "dofs_per_s": neq / (plain_ms * 1e-3), "assembly_ms": asm64_ms,
                       "solve_ms": ms64[A.T_SOLVE], "iters": it_plain, "solve_tol": tol64, "rel_err_vs_fp64": err_p},
        "speedup_vs_plain_fp64": plain_ms / ms_step, "speedup_split": split,
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                     "traffic": traffic, "kernel": kname, "blocks": nblk, "slots": nslot,
                     "bytes_per_launch": b32, "ms_per_launch": spmv32_ms, "peak_source": src,
                     "fp64_spmv": {"ms_per_launch": spmv64_ms,
                                   "achieved": spmv_bytes(nnz, neq, 8) / (spmv64_ms * 1e-3) / 1e9}},
        "assembly_roofline": assembly_roofline(p, S, asm_ms, hbm, src),
        "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks, "gpu_launches": int(launches),
        "kernel_ms": kernels,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    S.close()


if __name__ == "__main__":
    main()
