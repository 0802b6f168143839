"""Direct block assembly of small-strain elasticity on parallelepipeds
(ISL_PREC_MIXED, isl_blocks.cu): one thread per stored 3x3 block, double-float
arithmetic, no staged element matrices.  Against the oracle and against the
staged FP64 assembly of the same system:

* c2 (clamped x = 0, traction on x = 1): the path is taken; FP64 CSR values and
  right-hand side within 1e-12 of the oracle;
* a sheared parallelepiped mesh with nonzero Dirichlet values (the lift runs on
  the boundary elements) and per-element materials: the same bars;
* both are translates of one element, so their blocks come from tables formed
  once (ISL_OPT_SHARED_GEOMETRY), within 1e-13 of the per-element blocks; a
  graded mesh (boxes of varying width) forms every element's own;
* the mixed solve on the direct assembly is within 1e-8 of the oracle's FP64 CG
  solution, bitwise reproducible over a second assembly, and the scalar
  point-Jacobi path (FP32 CSR values derived from the FP64 ones) agrees.
"""
import numpy as np
import pytest

import oracle as O
from insilico_gb300 import _abi as A
from insilico_gb300 import workloads as W

from helpers import csr_entry_err, oracle_problem

pytestmark = pytest.mark.gpu

SHEAR = np.array([[1.0, 0.2, 0.1], [0.0, 1.0, 0.15], [0.0, 0.0, 0.9]])


def sheared(n):
    """c2-style elasticity on the unit cube mapped by SHEAR (parallelepipeds),
    x_ref = 0 clamped to a nonzero displacement, per-element E and nu."""
    X, conn = W.unit_cube("hex", n, n, n)
    Xs = X @ SHEAR.T
    g = W.rng(77, 0)
    lam, mu = W.lame(10.0 ** g.uniform(3.0, 5.0, len(conn)), g.uniform(0.2, 0.45, len(conn)))
    inv = np.linalg.inv(SHEAR)

    def diri(x):
        xr = x @ inv.T
        m = np.abs(xr[:, 0]) < 1e-9
        v = np.zeros((len(x), 3))
        v[:, 0] = 0.01 * xr[:, 1]
        v[:, 1] = -0.02 * xr[:, 2]
        v[:, 2] = 0.005
        return np.repeat(m[:, None], 3, axis=1), v
    return W.Problem("sheared", A.HEX, Xs, conn, 1, 3, "hyperelastic", 3, lam=lam, mu=mu, material="stvenant",
                     dirichlet=diri)


def graded(n):
    """c2-style elasticity on boxes of varying width along x (x -> x^1.5 of
    the unit-cube nodes): parallelepipeds that are not translates of one
    another, so every element's blocks come from its own Jacobian."""
    p = W.config("c2", n=n)
    X = p.X.copy()
    X[:, 0] = X[:, 0] ** 1.5
    p.X = X
    return p


@pytest.mark.parametrize("case", ["c2", "sheared", "graded"])
def test_direct_blocks_match_oracle_and_staged_fp64(case):
    p = {"c2": lambda: W.config("c2", n=6), "sheared": lambda: sheared(5), "graded": lambda: graded(5)}[case]()
    S = W.setup_system(p)
    assert S.get_option(A.OPT_BLOCKED) == 1
    S.assemble(A.PREC_FP64)
    assert S.get_option(A.OPT_DIRECT_BLOCKS) == 0
    rp, ci, v64s = S.csr()
    b64s = S.rhs()
    S.assemble(A.PREC_MIXED)
    assert S.get_option(A.OPT_DIRECT_BLOCKS) == 1
    _, _, vd = S.csr()
    bd = S.rhs()
    # translates of one element (c2, the sheared cube) share the blocks of
    # the first element's Jacobian; the graded boxes form their own.  The
    # shared blocks agree with the per-element ones to rounding.
    assert S.get_option(A.OPT_SHARED_GEOMETRY) == (0 if case == "graded" else 1)
    S.set_option(A.OPT_SHARED_GEOMETRY, 0)
    S.assemble(A.PREC_MIXED)
    assert S.get_option(A.OPT_SHARED_GEOMETRY) == 0
    _, _, vpe = S.csr()
    assert csr_entry_err(rp, ci, vd, vpe) <= 1e-13
    np.testing.assert_array_equal(S.rhs(), bd)
    S.set_option(A.OPT_SHARED_GEOMETRY, 1)
    S.assemble(A.PREC_MIXED)
    P, (orp, oci, ov, ob) = oracle_problem(p)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    assert csr_entry_err(orp, oci, vd, ov) <= 1e-12
    assert csr_entry_err(orp, oci, v64s, ov) <= 1e-12
    assert csr_entry_err(orp, oci, vd, v64s) <= 1e-12
    scale = np.max(np.abs(ob))
    assert scale > 0
    assert np.max(np.abs(bd - ob)) <= 1e-12 * scale
    assert np.max(np.abs(b64s - ob)) <= 1e-12 * scale
    # solves on the direct assembly: block path, bitwise reproducible, and the
    # scalar point-Jacobi path on derived FP32 CSR values
    xo, _, _ = O.cg(orp, oci, ov, ob, tol=1e-13)
    on = np.linalg.norm(xo)
    S.solve(A.SOLVE_CG_FP32_IR, tol=1e-11)
    x1 = S.solution()
    assert np.linalg.norm(x1 - xo) <= 1e-8 * on
    S.assemble(A.PREC_MIXED)
    S.solve(A.SOLVE_CG_FP32_IR, tol=1e-11)
    np.testing.assert_array_equal(S.solution(), x1)
    S.set_option(A.OPT_BLOCK_SOLVER, 0)
    S.solve(A.SOLVE_CG_FP32_IR, tol=1e-11)
    assert np.linalg.norm(S.solution() - xo) <= 1e-8 * on
    S.close()
