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
