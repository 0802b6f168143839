"""Shared test helpers: feed one workload to the oracle (CPU) and to the GPU
library (C-ABI), so the two can be compared on identical inputs."""
import numpy as np

import oracle as O
from insilico_gb300 import _abi as A
from insilico_gb300 import workloads as W

SHAPE_TO_ORACLE = {A.QUAD: O.QUAD, A.HEX: O.HEX, A.TET: O.TET}


def oracle_problem(p: W.Problem, assemble=True):
    """Run the reference call sequence for workload p on the oracle."""
    P = O.Problem(SHAPE_TO_ORACLE[p.shape], p.X, p.conn, p.fedeg, p.ncomp)
    if p.dirichlet is not None:
        x, d = P.boundary_points()
        mask, vals = p.dirichlet(x)
        mask = np.asarray(mask, dtype=bool).reshape(len(x), p.ncomp)
        vals = np.broadcast_to(np.asarray(vals, dtype=np.float64), mask.shape)
        r, c = np.nonzero(mask)
        P.constrain(d[r], c, vals[r, c])
    P.number()
    if p.kernel == "laplace":
        P.set_laplace(p.kappa, p.qdeg)
    else:
        P.set_hyperelastic(p.material, p.lam, p.mu, p.qdeg)
    if p.body is not None:
        P.set_body_nodal(p.body)
    if p.neumann_plane is not None:
        e, f = P.boundary_faces()
        axis, value, t = p.neumann_plane
        e, f = W.faces_on_plane(p.shape, p.X, p.conn, e, f, axis, value)
        P.set_neumann("constant", e, f, np.tile(t, (len(e), 1)), 0.0, 2)
    out = None
    if assemble:
        out = P.assemble(incremental=True)
    return P, out


def rel_entry_err(a, b, floor_frac=1e-12):
    """Max entry error relative to max(|b_i|, floor_frac * max|b|)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.maximum(np.abs(b), floor_frac * np.abs(b).max())
    return float(np.max(np.abs(a - b) / scale))


def oracle_newton(req, rtol=1e-10, max_newton=30, lin_tol=1e-12, nthreads=1):
    """The served Newton problem on the oracle: neo-Hookean hex8 cube, x = 0
    clamped, u_x prescribed on x = 1, load steps scaled as
    solid/CompressibleDriver.hpp:165-172, Newton as :180-211."""
    X, conn = W.unit_cube("hex", req.side, req.side, req.side)
    P = O.Problem(O.HEX, X, conn, 1, 3)
    x, d = P.boundary_points()
    first = req.pull / req.load_steps
    dofs, comps, vals = [], [], []
    for xi, di in zip(x, d):
        if abs(xi[0]) < 1e-9:
            for c in range(3):
                dofs.append(di); comps.append(c); vals.append(0.0)
        if abs(xi[0] - 1.0) < 1e-9:
            dofs.append(di); comps.append(0); vals.append(first)
    P.constrain(dofs, comps, vals)
    neq = P.number()
    ne = len(conn)
    P.set_hyperelastic("neohooke", np.full(ne, req.lam), np.full(ne, req.mu), 3)
    norm0 = None
    for step in range(req.load_steps):
        P.scale_constraints(float(step + 1) if step == 0 else (step + 1) / step)
        for it in range(max_newton):
            rp, ci, v, b = P.assemble(incremental=True, with_residual=True, nthreads=nthreads)
            conv1 = np.linalg.norm(b) / neq
            if it == 0:
                norm0 = conv1
            if conv1 <= rtol * norm0 and it > 0:
                break
            xs, _, _ = O.cg(rp, ci, v, b, tol=lin_tol, nthreads=nthreads)
            P.distribute(xs, add=True)
    return P.values()


def csr_entry_err(rowptr, colind, a, b):
    """Max |a_ij - b_ij| / max(|b_ij|, sqrt(|b_ii b_jj|)) over the CSR pattern.

    The diagonal geometric mean bounds |K_ij| of an SPD matrix, so entries that
    are small only through cancellation of element contributions are measured
    against the scale of their row and column instead of their own size."""
    rowptr = np.asarray(rowptr)
    colind = np.asarray(colind)
    n = len(rowptr) - 1
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    diag = np.zeros(n)
    on = rows == colind
    diag[rows[on]] = np.abs(b[on])
    scale = np.maximum(np.abs(b), np.sqrt(diag[rows] * diag[colind]))
    scale = np.maximum(scale, 1e-300)
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)) / scale))


def oracle_newton_driver(req, tol, max_newton, lin_tol=1e-12, nthreads=1):
    """The served request on the oracle with solid/CompressibleDriver.hpp:156-214
    itself: per load step scale the constraints by (k+1)/k, then Newton:
    assemble, stop when ||R||/N < tol, solve, add, stop when ||dU||/N < tol
    or after max_newton iterations.  Returns (values, Newton iterations)."""
    X, conn = W.unit_cube("hex", req.side, req.side, req.side)
    P = O.Problem(O.HEX, X, conn, 1, 3)
    x, d = P.boundary_points()
    first = req.pull / req.load_steps
    dofs, comps, vals = [], [], []
    for xi, di in zip(x, d):
        if abs(xi[0]) < 1e-9:
            for c in range(3):
                dofs.append(di); comps.append(c); vals.append(0.0)
        if abs(xi[0] - 1.0) < 1e-9:
            dofs.append(di); comps.append(0); vals.append(first)
    P.constrain(dofs, comps, vals)
    neq = P.number()
    ne = len(conn)
    P.set_hyperelastic("neohooke", np.full(ne, req.lam), np.full(ne, req.mu), 3)
    newton = 0
    for step in range(req.load_steps):
        P.scale_constraints(float(step + 1) if step == 0 else (step + 1) / step)
        it = 0
        while it < max_newton:
            rp, ci, v, b = P.assemble(incremental=True, with_residual=True, nthreads=nthreads)
            if np.linalg.norm(b) / neq < tol:
                break
            xs, _, _ = O.cg(rp, ci, v, b, tol=lin_tol, nthreads=nthreads)
            P.distribute(xs, add=True)
            it += 1
            newton += 1
            if np.linalg.norm(xs) / neq < tol:
                break
    return P.values(), newton
