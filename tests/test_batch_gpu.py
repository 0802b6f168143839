"""Batched instances on the GPU: several independent 2-D heat problems of
different sizes in one context.  Each instance's DOF numbering and CSR block
must be bit-identical to solving it alone (the reference numbering of that
mesh), its matrix entries within 1e-12 of the oracle, and its CG solution
(own scalars and convergence) within 1e-8 of the oracle's solution."""
import numpy as np
import pytest

import oracle as O
from insilico_gb300 import _abi as A
from insilico_gb300 import workloads as W
from insilico_gb300.system import System

from helpers import csr_entry_err, oracle_problem

pytestmark = pytest.mark.gpu


def instance(side, deg, seed):
    X, conn = W.unit_cube("quad", side, side)
    g = W.rng(seed, 0)
    kappa = np.exp(g.normal(0.0, 0.5, len(conn)))
    f = W.rng(seed, 1).uniform(0.0, 1.0, len(X))[:, None]
    return W.Problem("inst", A.QUAD, X, conn, deg, 1, "laplace", 2 * deg, kappa=kappa, body=f,
                     dirichlet=lambda x: (np.ones((len(x), 1), dtype=bool), 0.0), tol=1e-10)


@pytest.mark.parametrize("deg", [1, 2])
def test_batch_matches_single_instances(deg):
    probs = [instance(s, deg, 100 + s) for s in (3, 9, 5, 16, 2)]
    S = System()
    S.upload_batch(A.QUAD, [(p.X, p.conn) for p in probs])
    S.create_field(deg, 1)
    S.constrain_boundary(lambda x: (np.ones((len(x), 1), dtype=bool), 0.0))
    S.number_dofs()
    S.register_pattern()
    S.set_laplace(np.concatenate([p.kappa for p in probs]), 2 * deg)
    S.set_body_force_nodal(np.concatenate([p.body for p in probs]))
    eq_off, _ = S.batch_info()
    S.assemble(A.PREC_MIXED)
    rp, ci, v = S.csr()
    b = S.rhs()
    S.solve(A.SOLVE_CG_FP64, tol=1e-12)
    x64 = S.solution()
    it64, _ = S.batch_stats()
    S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
    xm = S.solution()
    for k, p in enumerate(probs):
        P, (orp, oci, ov, ob) = oracle_problem(p)
        r0, r1 = eq_off[k], eq_off[k + 1]
        assert r1 - r0 == P.neq
        lrp = rp[r0:r1 + 1] - rp[r0]
        np.testing.assert_array_equal(lrp, orp)
        np.testing.assert_array_equal(ci[rp[r0]:rp[r1]] - r0, oci)
        assert csr_entry_err(orp, oci, v[rp[r0]:rp[r1]], ov) <= 1e-12
        assert np.max(np.abs(b[r0:r1] - ob)) <= 1e-12 * np.max(np.abs(ob))
        xo, ito, _ = O.cg(orp, oci, ov, ob, tol=1e-13)
        assert np.linalg.norm(x64[r0:r1] - xo) <= 1e-9 * np.linalg.norm(xo)
        assert np.linalg.norm(xm[r0:r1] - xo) <= 1e-8 * np.linalg.norm(xo)
        assert abs(it64[k] - O.cg(orp, oci, ov, ob, tol=1e-12)[1]) <= 2
    S.close()


@pytest.mark.parametrize("deg", [1, 2])
def test_batch_sliced_ell_and_csr_agree(deg):
    """The batched mixed solve on its per-block sliced-ELL copy (each row block
    of an instance sorted by row length into slices of 32) and on the CSR:
    every instance meets the tolerance and agrees with the oracle within 1e-7;
    the three batch depths sum in slot order and give bitwise equal solves.
    (1e-10: the FP32 iteration with FP64 reliable updates attains about 1e-12
    on the largest of these Q2 instances.)"""
    probs = [instance(s, deg, 300 + s) for s in (40, 3, 27, 61, 8)]
    S = System()
    S.upload_batch(A.QUAD, [(p.X, p.conn) for p in probs])
    S.create_field(deg, 1)
    S.constrain_boundary(lambda x: (np.ones((len(x), 1), dtype=bool), 0.0))
    S.number_dofs()
    S.register_pattern()
    S.set_laplace(np.concatenate([p.kappa for p in probs]), 2 * deg)
    S.set_body_force_nodal(np.concatenate([p.body for p in probs]))
    eq_off, _ = S.batch_info()
    S.assemble(A.PREC_MIXED)
    S.solve(A.SOLVE_CG_FP32_IR, tol=1e-10)  # builds the copy, autotunes the SpMV
    assert S.get_option(A.OPT_SPMV32_KIND) in (2, 4, 8, 16, 32, 102, 104, 108)
    assert S.get_option(A.OPT_SCALAR_SLOTS) >= S.nnz
    out = {}
    for kind in (4, 102, 104, 108):
        S.set_option(A.OPT_SPMV32_KIND, kind)
        S.solve(A.SOLVE_CG_FP32_IR, tol=1e-10)
        assert S.get_option(A.OPT_SPMV32_KIND) == kind
        out[kind] = S.solution()
    for kind in (102, 108):
        assert np.array_equal(out[kind], out[104])
    # 16-bit column offsets (on by default where they fit) against 32-bit ones
    assert S.get_option(A.OPT_SHORT_COLUMNS) == 1
    S.set_option(A.OPT_SHORT_COLUMNS, 0)
    S.set_option(A.OPT_SPMV32_KIND, 104)
    S.solve(A.SOLVE_CG_FP32_IR, tol=1e-10)
    assert np.array_equal(S.solution(), out[104])
    S.set_option(A.OPT_SHORT_COLUMNS, 1)
    for k, p in enumerate(probs):
        P, (orp, oci, ov, ob) = oracle_problem(p)
        r0, r1 = eq_off[k], eq_off[k + 1]
        xo, _, _ = O.cg(orp, oci, ov, ob, tol=1e-13)
        for kind in (4, 104):
            assert np.linalg.norm(out[kind][r0:r1] - xo) <= 1e-7 * np.linalg.norm(xo)
    S.close()


@pytest.mark.parametrize("drop", [2, 4])
def test_batch_reliable_update_spacing(drop):
    """ISL_OPT_RELIABLE_DROP spaces the FP64 reliable updates (an update when
    the FP32 r.r has dropped by 10^drop): every instance still reaches the
    tolerance on its true residual and the oracle's solution within 1e-8."""
    probs = [instance(s, 2, 500 + s) for s in (30, 4, 45, 12)]
    S = System()
    S.upload_batch(A.QUAD, [(p.X, p.conn) for p in probs])
    S.create_field(2, 1)
    S.constrain_boundary(lambda x: (np.ones((len(x), 1), dtype=bool), 0.0))
    S.number_dofs()
    S.register_pattern()
    S.set_laplace(np.concatenate([p.kappa for p in probs]), 4)
    S.set_body_force_nodal(np.concatenate([p.body for p in probs]))
    S.set_option(A.OPT_RELIABLE_DROP, drop)
    assert S.get_option(A.OPT_RELIABLE_DROP) == drop
    eq_off, _ = S.batch_info()
    S.assemble(A.PREC_MIXED)
    S.solve(A.SOLVE_CG_FP32_IR, tol=1e-10)
    xm = S.solution()
    _, rel = S.batch_stats()
    assert np.all(np.asarray(rel) <= 1e-10)
    for k, p in enumerate(probs):
        P, (orp, oci, ov, ob) = oracle_problem(p)
        r0, r1 = eq_off[k], eq_off[k + 1]
        xo, _, _ = O.cg(orp, oci, ov, ob, tol=1e-13)
        assert np.linalg.norm(xm[r0:r1] - xo) <= 1e-8 * np.linalg.norm(xo)
    with pytest.raises(A.IslError):
        S.set_option(A.OPT_RELIABLE_DROP, 0)
    S.close()
