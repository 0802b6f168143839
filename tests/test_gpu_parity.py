"""GPU parity against the oracle, through the C-ABI (libisl_gpu.so).

Bars:
  * DOF numbering and CSR pattern: bit-exact.
  * FP64 matrix entries: |K_gpu - K_oracle| <= 1e-12 max(|K_oracle|, sqrt(K_ii K_jj)),
    i.e. 1e-12 relative, with the diagonal scale for entries that cancel.
  * RHS: same bar.
  * FP64 CG solution vs the oracle's CG solution (both to 1e-13): rel L2 <= 1e-9.
  * Mixed FP32-CG + FP64 refinement to 1e-12: rel L2 error vs FP64 <= 1e-8.
  * Assembly and solve are bit-reproducible run to run (no atomics).
"""
import numpy as np
import scipy.sparse as sp
import pytest

import oracle as O
from insilico_gb300 import _abi as A
from insilico_gb300 import workloads as W

from helpers import csr_entry_err, oracle_problem

pytestmark = pytest.mark.gpu

CASES = [("c1", 12), ("c2", 4), ("c3", 3), ("c1", 2), ("c2", 1)]


@pytest.fixture(scope="module")
def systems():
    out = {}
    yield out
    for S in out.values():
        S.close()


def gpu_problem(p):
    S = W.setup_system(p)
    return S


@pytest.mark.parametrize("precision", [A.PREC_FP64, A.PREC_MIXED])
@pytest.mark.parametrize("name,n", CASES)
def test_pattern_values_rhs_match_oracle(name, n, precision):
    """FP64 element kernels (the plain path) and the mixed assembly
    (double-float element arithmetic on the FP32 pipe) both give entries
    and right-hand sides within 1e-12 of the oracle."""
    p = W.config(name, n=n)
    S = gpu_problem(p)
    P, (rp, ci, v, b) = oracle_problem(p)
    assert S.neq == P.neq
    np.testing.assert_array_equal(S.dof_index(), P.eq_index())
    S.assemble(precision)
    grp, gci, gv = S.csr()
    np.testing.assert_array_equal(grp, rp)
    np.testing.assert_array_equal(gci, ci)
    assert csr_entry_err(rp, ci, gv, v) <= 1e-12
    gb = S.rhs()
    assert np.max(np.abs(gb - b)) <= 1e-12 * max(np.max(np.abs(b)), 1e-300)
    S.close()


@pytest.mark.parametrize("name,n", [("c1", 12), ("c2", 4), ("c3", 3)])
def test_cg_fp64_and_mixed_solution(name, n):
    p = W.config(name, n=n)
    S = gpu_problem(p)
    P, (rp, ci, v, b) = oracle_problem(p)
    xo, _, _ = O.cg(rp, ci, v, b, tol=1e-13)
    S.assemble(A.PREC_MIXED)
    it, rr, _ = S.solve(A.SOLVE_CG_FP64, tol=1e-13)
    x64 = S.solution()
    assert np.linalg.norm(x64 - xo) <= 1e-9 * np.linalg.norm(xo)
    it2, rr2, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
    xm = S.solution()
    assert rr2 <= 1e-12
    assert np.linalg.norm(xm - xo) <= 1e-8 * np.linalg.norm(xo)
    S.close()


@pytest.mark.parametrize("name,n", [("c1", 16), ("c2", 5)])
def test_bitwise_reproducible(name, n):
    p = W.config(name, n=n)
    S = gpu_problem(p)
    S.assemble(A.PREC_FP64)
    _, _, v1 = S.csr()
    b1 = S.rhs()
    S.solve(A.SOLVE_CG_FP64, tol=1e-12)
    x1 = S.solution()
    S.assemble(A.PREC_FP64)
    _, _, v2 = S.csr()
    b2 = S.rhs()
    S.solve(A.SOLVE_CG_FP64, tol=1e-12)
    x2 = S.solution()
    assert np.array_equal(v1, v2) and np.array_equal(b1, b2) and np.array_equal(x1, x2)
    S.close()


@pytest.mark.parametrize("name,n", [("c1", 10), ("c2", 3), ("c3", 2)])
def test_fp32_assembly_close_to_fp64(name, n):
    p = W.config(name, n=n)
    S = gpu_problem(p)
    S.assemble(A.PREC_FP64)
    _, _, v64 = S.csr()
    b64 = S.rhs()
    S.assemble(A.PREC_FP32)
    rp, ci, v32 = S.csr()
    assert csr_entry_err(rp, ci, v32, v64) <= 2e-6
    np.testing.assert_allclose(S.rhs(), b64, rtol=0, atol=1e-12 * np.abs(b64).max())
    S.close()


@pytest.mark.parametrize("material", ["stvenant", "neohooke"])
def test_hyperelastic_tangent_and_residual_at_displacement(material):
    p = W.config("c2", n=3)
    p.material = material
    S = gpu_problem(p)
    P, _ = oracle_problem(p, assemble=False)
    rs = np.random.default_rng(7)
    u = 0.02 * rs.standard_normal(S.ndofobj * 3)
    # constrained components carry their constraint value (zero on the clamp)
    eq = S.dof_index()
    u[eq < 0] = 0.0
    S.set_values(u)
    P.set_values(u)
    rp, ci, v, b = P.assemble(incremental=True, with_residual=True)
    S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
    grp, gci, gv = S.csr()
    np.testing.assert_array_equal(gci, ci)
    ek = csr_entry_err(rp, ci, gv, v)
    assert ek <= 1e-12, ek
    gb = S.rhs()
    eb = np.max(np.abs(gb - b)) / np.max(np.abs(b))
    assert eb <= 1e-12, eb
    # FP32 tangent, FP64 residual
    S.assemble(A.PREC_FP32, incremental=True, with_residual=True)
    eb32 = np.max(np.abs(S.rhs() - b)) / np.max(np.abs(b))
    assert eb32 <= 1e-12, eb32
    S.close()


def test_degenerate_element_reports_status():
    X = np.array([[0, 0], [1, 0], [2, 0], [3, 0]], dtype=float)  # collinear: det J = 0
    from insilico_gb300.system import System
    S = System()
    S.upload_mesh(A.QUAD, X, np.array([[0, 1, 2, 3]]))
    S.create_field(1, 1)
    S.number_dofs()
    S.register_pattern()
    S.set_laplace(np.ones(1), 2)
    with pytest.raises(A.IslError) as ei:
        S.assemble(A.PREC_FP64)
    assert ei.value.code == A.ISL_ERR_DEGENERATE
    S.close()


def test_max_iter_reports_not_converged():
    p = W.config("c1", n=16)
    S = gpu_problem(p)
    S.assemble(A.PREC_FP64)
    it, rr, st = S.solve(A.SOLVE_CG_FP64, tol=1e-14, max_iter=3, check=False)
    assert st == A.ISL_ERR_NOT_CONVERGED and it == 3
    S.close()


def test_block_and_scalar_mixed_paths_agree():
    p = W.config("c2", n=4)
    S = gpu_problem(p)
    assert S.get_option(A.OPT_BLOCKED) == 1
    S.assemble(A.PREC_MIXED)
    S.solve(A.SOLVE_CG_FP64, tol=1e-13)
    x64 = S.solution()
    S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
    xb = S.solution()
    S.set_option(A.OPT_BLOCK_SOLVER, 0)
    S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
    xs = S.solution()
    assert np.linalg.norm(xb - x64) <= 1e-8 * np.linalg.norm(x64)
    assert np.linalg.norm(xs - x64) <= 1e-8 * np.linalg.norm(x64)
    S.close()


@pytest.mark.parametrize("n", [3, 10])
def test_persistent_and_graph_block_cg_agree(n):
    """The persistent cooperative CG kernel and the graph of separate kernels
    run the same recurrences: same iteration count, solutions within 1e-8 of
    FP64, and each path bitwise reproducible."""
    p = W.config("c2", n=n)
    S = gpu_problem(p)
    assert S.get_option(A.OPT_PERSISTENT) == 1
    S.assemble(A.PREC_MIXED)
    S.solve(A.SOLVE_CG_FP64, tol=1e-13)
    x64 = S.solution()
    out = {}
    for persist in (2, 0):
        S.set_option(A.OPT_PERSISTENT, persist)
        it, rel, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
        x = S.solution()
        it2, _, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
        assert it2 == it and np.array_equal(S.solution(), x)
        assert rel <= 1e-12
        assert np.linalg.norm(x - x64) <= 1e-8 * np.linalg.norm(x64)
        out[persist] = (it, x)
    assert abs(out[2][0] - out[0][0]) <= max(2, out[0][0] // 50)
    S.close()


def test_folded_direction_update_matches_separate_kernel():
    """The graph path of the block CG (c2 at 32^3: 34,848 block rows, above
    the persistent kernel's limit) with the direction update folded into the
    SpMV and with the separate direction kernel: both reach the tolerance,
    agree with the FP64 solve within 1e-8, are bitwise reproducible, take
    iteration counts within 2 %, and the folded path launches fewer kernels
    (two per iteration instead of three)."""
    p = W.config("c2", n=32)
    S = gpu_problem(p)
    assert S.get_option(A.OPT_FOLD_DIRECTION) == 1
    S.assemble(A.PREC_MIXED)
    S.solve(A.SOLVE_CG_FP64, tol=1e-13)
    x64 = S.solution()
    out = {}
    for fold in (1, 0):
        S.set_option(A.OPT_FOLD_DIRECTION, fold)
        l0 = S.launch_count()
        it, rel, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
        launches = S.launch_count() - l0
        x = S.solution()
        it2, _, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
        assert it2 == it and np.array_equal(S.solution(), x)
        assert rel <= 1e-12
        assert np.linalg.norm(x - x64) <= 1e-8 * np.linalg.norm(x64)
        out[fold] = (it, launches)
    assert abs(out[1][0] - out[0][0]) <= max(2, out[0][0] // 50)
    assert out[1][1] < out[0][1]
    assert S.get_option(A.OPT_BLOCK_UPDATE) == 0
    # every update kernel (one thread per node; shared-memory tiles at 2, 4,
    # 8 blocks per SM) meets the same bars; the per-node arithmetic is the
    # same, only the FP32 partial sums of r.r and r.z group nodes
    # differently, which moves the FP32 recurrence and with it the iteration
    # count by a few percent
    for uk in (1, 2, 4, 8):
        S.set_option(A.OPT_BLOCK_UPDATE, uk)
        it, rel, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
        assert S.get_option(A.OPT_BLOCK_UPDATE) == uk
        assert rel <= 1e-12 and abs(it - out[1][0]) <= max(2, out[1][0] // 10)
        assert np.linalg.norm(S.solution() - x64) <= 1e-8 * np.linalg.norm(x64)
    with pytest.raises(A.IslError):
        S.set_option(A.OPT_BLOCK_UPDATE, 3)
    # 16-bit column offsets (every offset of this matrix is within 1,123
    # block rows) read the same columns: bitwise the same solve
    S.set_option(A.OPT_BLOCK_UPDATE, 1)
    assert S.get_option(A.OPT_SHORT_COLUMNS) == 1
    it16, _, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
    x16 = S.solution()
    S.set_option(A.OPT_SHORT_COLUMNS, 0)
    assert S.get_option(A.OPT_SHORT_COLUMNS) == 0
    it32, _, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
    assert it32 == it16 and np.array_equal(S.solution(), x16)
    # reliable updates after every 10x drop of the FP32 r.r instead of 100x
    S.set_option(A.OPT_SHORT_COLUMNS, 1)
    S.set_option(A.OPT_RELIABLE_DROP, 1)
    itd, reld, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
    assert reld <= 1e-12 and np.linalg.norm(S.solution() - x64) <= 1e-8 * np.linalg.norm(x64)
    S.set_option(A.OPT_RELIABLE_DROP, 2)
    S.close()


@pytest.mark.parametrize("name,n", [("c1", 40), ("c3", 5), ("c1", 1)])
def test_cluster_and_graph_scalar_cg_agree(name, n):
    """Small scalar systems are solved whole by one thread-block cluster; the
    graph of separate kernels runs the same recurrences.  Both meet the
    tolerance and agree within 1e-8, with and without the FP64 matrix."""
    p = W.config(name, n=n)
    S = gpu_problem(p)
    assert S.neq <= 65536
    S.assemble(A.PREC_MIXED)
    S.solve(A.SOLVE_CG_FP64, tol=1e-13)
    x64 = S.solution()
    out = {}
    for persist in (1, 0):
        S.set_option(A.OPT_PERSISTENT, persist)
        it, rel, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
        x = S.solution()
        S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
        assert np.array_equal(S.solution(), x)
        assert rel <= 1e-12
        assert np.linalg.norm(x - x64) <= 1e-8 * np.linalg.norm(x64)
        out[persist] = it
    assert abs(out[1] - out[0]) <= max(2, out[0] // 50)
    # FP32 tangent only: plain FP32 CG on the iterated residual
    S.assemble(A.PREC_FP32)
    res = {}
    for persist in (1, 0):
        S.set_option(A.OPT_PERSISTENT, persist)
        it, rel, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-6)
        res[persist] = (it, S.solution())
        assert rel <= 1e-6
    assert abs(res[1][0] - res[0][0]) <= max(2, res[0][0] // 20)
    assert np.linalg.norm(res[1][1] - res[0][1]) <= 1e-5 * np.linalg.norm(res[0][1])
    S.close()


def test_persistent_option_range():
    S = gpu_problem(W.config("c1", n=4))
    with pytest.raises(A.IslError):
        S.set_option(A.OPT_PERSISTENT, 3)
    S.set_option(A.OPT_PERSISTENT, 2)
    assert S.get_option(A.OPT_PERSISTENT) == 2
    S.close()


@pytest.mark.parametrize("n", [3, 34])
def test_partially_constrained_nodes_use_padded_blocks(n):
    """x = 1 face pulled in u_x only (PulledSheet-style): the DOF objects there
    keep two of three components active, and the block solver runs on padded
    blocks (ISL_OPT_BLOCKED = 2).  n = 3: the persistent block kernel; n = 34
    (41,650 block rows): the graph path with the folded direction update.
    Pattern and RHS match the oracle; the padded mixed solve, the scalar
    mixed solve and the FP64 solve all reach the oracle's FP64 CG solution
    within 1e-8; an FP32-only assembly runs the padded FP32 block CG to its
    recursive tolerance 1e-6, and its true FP64 residual is within 1e-4."""
    p = _pulled_sheet(n)
    S = gpu_problem(p)
    assert S.get_option(A.OPT_BLOCKED) == 2
    P, (rp, ci, v, b) = oracle_problem(p)
    S.assemble(A.PREC_MIXED)
    np.testing.assert_array_equal(S.csr(values=False)[1], ci)
    assert np.max(np.abs(S.rhs() - b)) <= 1e-12 * np.max(np.abs(b))
    xo, _, _ = O.cg(rp, ci, v, b, tol=1e-13, nthreads=8)
    on = np.linalg.norm(xo)
    it_b, rel, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
    xb = S.solution()
    assert rel <= 1e-12 and np.linalg.norm(xb - xo) <= 1e-8 * on
    it_b2, _, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
    assert it_b2 == it_b and np.array_equal(S.solution(), xb)
    S.solve(A.SOLVE_CG_FP64, tol=1e-13)
    assert np.linalg.norm(S.solution() - xo) <= 1e-8 * on
    S.set_option(A.OPT_BLOCK_SOLVER, 0)
    S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
    assert np.linalg.norm(S.solution() - xo) <= 1e-8 * on
    S.set_option(A.OPT_BLOCK_SOLVER, 1)
    S.assemble(A.PREC_FP32)
    it32, rel32, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-6)
    x32 = S.solution()
    K = sp.csr_matrix((v, ci, rp), shape=(len(b), len(b)))
    assert rel32 <= 1e-6 and it32 > 0
    # the FP32 recursion's residual drifts from the true one by the FP32
    # rounding of matrix and iterates times the conditioning (E spans two
    # decades): a wrong padded map would leave an O(1) residual
    assert np.linalg.norm(b - K @ x32) <= 1e-4 * np.linalg.norm(b)
    S.close()


def _pulled_sheet(n):
    """hex8 elasticity with the x = 1 face pulled in u_x only: nodes there are
    partly active (padded node blocks)."""
    p = W.config("c2", n=n)
    base = p.dirichlet

    def diri(x):
        m, v = base(x)
        m = m.copy()
        m[np.abs(x[:, 0] - 1.0) < 1e-9, 0] = True
        vals = np.zeros(m.shape)
        vals[np.abs(x[:, 0] - 1.0) < 1e-9, 0] = 0.01
        return m, vals
    p.dirichlet = diri
    p.neumann_plane = None
    return p


@pytest.mark.parametrize("case", ["c3", "c1"])
def test_scalar_sliced_ell_and_csr_agree(case):
    """The sliced-ELL copy of a scalar (not node-blocked) system holds every
    stored entry once (padding < 10 %); its SpMV sums each row in slot order
    whatever the batch depth, so the three depths give bitwise identical
    solves; CSR and sliced-ELL both meet the tolerance and agree with FP64."""
    p = W.config("c3", n=16) if case == "c3" else W.config("c1", n=160)
    S = gpu_problem(p)
    assert S.get_option(A.OPT_BLOCKED) == 0 and S.neq >= 20000
    S.assemble(A.PREC_MIXED)
    nnz = len(S.csr(values=False)[1])
    slots = S.get_option(A.OPT_SCALAR_SLOTS)
    assert nnz <= slots <= 1.1 * nnz
    S.set_option(A.OPT_PERSISTENT, 0)  # graph path (the cluster path has its own SpMV)
    S.solve(A.SOLVE_CG_FP64, tol=1e-13)
    x64 = S.solution()
    out = {}
    for kind in (4, 102, 104, 108):
        S.set_option(A.OPT_SPMV32_KIND, kind)
        it, rel, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
        assert S.get_option(A.OPT_SPMV32_KIND) == kind
        x = S.solution()
        assert rel <= 1e-12
        assert np.linalg.norm(x - x64) <= 1e-8 * np.linalg.norm(x64)
        out[kind] = (it, x)
    for kind in (102, 108):
        assert out[kind][0] == out[104][0] and np.array_equal(out[kind][1], out[104][1])
    assert abs(out[104][0] - out[4][0]) <= max(2, out[4][0] // 50)
    # 16-bit column offsets from each row (on by default where they fit)
    # read the same columns: the same bits with 32-bit columns
    assert S.get_option(A.OPT_SHORT_COLUMNS) == 1
    S.set_option(A.OPT_SHORT_COLUMNS, 0)
    S.set_option(A.OPT_SPMV32_KIND, 104)
    it32, _, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
    assert it32 == out[104][0] and np.array_equal(S.solution(), out[104][1])
    S.set_option(A.OPT_SHORT_COLUMNS, 1)
    # autotuned choice is one of the candidates and solves to the same bar
    S.set_option(A.OPT_SPMV32_KIND, 0)
    it, rel, _ = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
    assert S.get_option(A.OPT_SPMV32_KIND) in (4, 8, 16, 32, 102, 104, 108)
    assert np.linalg.norm(S.solution() - x64) <= 1e-8 * np.linalg.norm(x64)
    S.close()


def test_spmv32_kind_option_range():
    S = gpu_problem(W.config("c2", n=4))  # node-blocked: no scalar sliced-ELL copy
    assert S.get_option(A.OPT_SCALAR_SLOTS) == 0
    for bad in (3, 104, 116, -1):
        with pytest.raises(A.IslError):
            S.set_option(A.OPT_SPMV32_KIND, bad)
    S.set_option(A.OPT_SPMV32_KIND, 8)
    S.close()


def test_empty_system_every_dof_constrained():
    p = W.config("c1", n=1)  # a single quad: all four nodes on the Dirichlet boundary
    S = gpu_problem(p)
    assert S.neq == 0 and S.nnz == 0
    S.assemble(A.PREC_MIXED)
    it, rr, st = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
    assert it == 0 and st == A.ISL_OK
    S.distribute()
    assert np.all(S.values() == 0.0)
    S.close()


@pytest.mark.parametrize("material", ["stvenant", "neohooke"])
def test_hex8_non_affine_mesh_matches_oracle(material):
    """Distorted hexahedra (no element a parallelepiped) take the quadrature-
    loop kernel; parallelepipeds take the closed-form one.  Both match the
    oracle: pattern bit-exact, entries and RHS to 1e-12, solution to 1e-8."""
    p = W.config("c2", n=4)
    p.material = material
    g = np.random.default_rng(11)
    interior = np.all((p.X > 1e-9) & (p.X < 1 - 1e-9), axis=1)
    p.X = p.X + 0.08 / 4 * g.uniform(-1.0, 1.0, p.X.shape) * interior[:, None]
    S = gpu_problem(p)
    P, (rp, ci, v, b) = oracle_problem(p)
    S.assemble(A.PREC_MIXED)
    grp, gci, gv = S.csr()
    np.testing.assert_array_equal(grp, rp)
    np.testing.assert_array_equal(gci, ci)
    assert csr_entry_err(rp, ci, gv, v) <= 1e-12
    assert np.max(np.abs(S.rhs() - b)) <= 1e-12 * np.max(np.abs(b))
    S.solve(A.SOLVE_CG_FP32_IR, tol=1e-12)
    xo, _, _ = O.cg(rp, ci, v, b, tol=1e-13)
    assert np.linalg.norm(S.solution() - xo) <= 1e-8 * np.linalg.norm(xo)
    S.close()


def test_persistent_barrier_timeout_reports_status():
    """Failure path of the persistent kernel's grid barrier, without a GPU
    fault: the test hook arms the barrier so that it cannot complete, the
    bounded wait runs out, the solve returns ISL_ERR_TIMEOUT, and the context
    then solves normally."""
    p = W.config("c2", n=3)
    S = gpu_problem(p)
    S.assemble(A.PREC_MIXED)
    S.set_option(A.OPT_PERSISTENT, 2)
    it_ok, _, st = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-10)
    assert st == A.ISL_OK
    x_ok = S.solution()
    S.set_option(A.OPT_BARRIER_TEST, 1)
    _, _, st = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-10, check=False)
    assert st == A.ISL_ERR_TIMEOUT
    it, _, st = S.solve(A.SOLVE_CG_FP32_IR, tol=1e-10)
    assert st == A.ISL_OK and it == it_ok
    assert np.array_equal(S.solution(), x_ok)
    S.close()
