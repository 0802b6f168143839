"""heat::Static (nonlinear heat conduction) and BiCGSTAB on the GPU: the
non-symmetric tangent and residual against the oracle, the BiCGSTAB solution
against a direct solve, and the whole Newton run of
reference/04-heat/nonlinearHeat.cpp against its golden output."""
import numpy as np
import pytest

import oracle as O
from insilico_gb300 import _abi as A
from insilico_gb300 import workloads as W
from insilico_gb300.system import System

from helpers import csr_entry_err

pytestmark = pytest.mark.gpu


def _both(kind, shape, deg, sizes, material, seed, qdeg=2):
    """the same heat::Static problem on the GPU and on the oracle, at random
    nonnegative DOF values (u > -1 for the FenicsTest law)"""
    X, conn = W.unit_cube(kind, *sizes)
    rng = np.random.default_rng(seed)
    prm = rng.uniform(1.0, 3.0, len(conn))
    S = System(device=0)
    S.upload_mesh(shape, X, conn)
    S.create_field(deg, 1)
    mask_fun = lambda x: ((np.abs(x[:, 0]) < 1e-9)[:, None], np.full((len(x), 1), 0.25))  # noqa: E731
    S.constrain_boundary(mask_fun)
    S.number_dofs()
    S.register_pattern()
    S.set_heat_static(material, prm, qdeg)
    u = rng.uniform(0.0, 0.5, S.ndofobj)
    S.set_values(u)
    P = O.Problem({A.QUAD: O.QUAD, A.TET: O.TET, A.HEX: O.HEX}[shape], X, conn, deg, 1)
    x, d = P.boundary_points()
    on = np.abs(x[:, 0]) < 1e-9
    P.constrain(d[on], np.zeros(on.sum()), np.full(on.sum(), 0.25))
    P.number()
    P.set_heat_static(material, prm, qdeg)
    P.set_values(u)
    return S, P


@pytest.mark.parametrize("kind,shape,deg,sizes,qdeg", [
    ("quad", A.QUAD, 2, (6, 5), 2), ("quad", A.QUAD, 1, (9, 7), 2), ("tet", A.TET, 2, (3, 2, 2), 2),
    ("hex", A.HEX, 1, (3, 3, 2), 2), ("tet", A.TET, 2, (3, 2, 2), 4),  # 11-point rule (2 x field degree)
])
@pytest.mark.parametrize("material", ["fenics", "constant"])
def test_heat_static_tangent_and_residual_match_oracle(kind, shape, deg, sizes, qdeg, material):
    S, P = _both(kind, shape, deg, sizes, material, 5, qdeg)
    S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
    rp, ci, v, b = P.assemble(incremental=True, with_residual=True)
    srp, sci, sv = S.csr()
    np.testing.assert_array_equal(srp, rp)
    np.testing.assert_array_equal(sci, ci)
    assert csr_entry_err(rp, ci, sv, v) <= 1e-12
    assert np.max(np.abs(S.rhs() - b)) <= 1e-12 * np.max(np.abs(b))
    if material == "fenics":
        # the tangent is not symmetric
        import scipy.sparse as sp
        Am = sp.csr_matrix((sv, sci, srp))
        assert abs(Am - Am.T).max() > 1e-6 * abs(Am).max()
    S.close()


def test_bicgstab_solves_the_nonsymmetric_system():
    import scipy.sparse as sp
    from scipy.sparse.linalg import spsolve
    S, P = _both("quad", A.QUAD, 2, (16, 12), "fenics", 9)
    S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
    rp, ci, v = S.csr()
    b = S.rhs()
    it, rel, _ = S.solve(A.SOLVE_BICGSTAB, tol=1e-13)
    assert 0 < it < len(b) and rel <= 1e-13
    x = S.solution()
    xd = spsolve(sp.csc_matrix(sp.csr_matrix((v, ci, rp))), b)
    assert np.linalg.norm(x - xd) <= 1e-9 * np.linalg.norm(xd)
    # bitwise reproducible, and CG refuses the non-symmetric tangent
    S.solve(A.SOLVE_BICGSTAB, tol=1e-13)
    assert np.array_equal(S.solution(), x)
    with pytest.raises(A.IslError):
        S.solve(A.SOLVE_CG_FP64, tol=1e-10)
    S.close()


def test_nonlinear_heat_matches_reference_golden(pins):
    """reference/04-heat/nonlinearHeat.cpp on square_200.smf (Q2, 159,999
    DOFs): Newton |R| and |x| per iteration, iteration count and L2 error, to
    the 6 digits of nonlinearHeat.ref.dat"""
    ref = pins["nonlinearHeat"]
    X, conn = O.unitcube("quad", 200, 200, round6=True)
    S = System(device=0)
    n, rows, l2 = W.nonlinear_heat(S, X, conn)
    assert n == ref["ndofs"]
    assert len(rows) == len(ref["newton"]) and len(rows) - 1 == ref["iterations"]
    for got, want in zip(rows, ref["newton"]):
        assert got[0] == want[0]
        assert got[1] == pytest.approx(want[1], rel=2e-5)
        if want[2] is None:
            assert got[2] is None
        else:
            assert got[2] == pytest.approx(want[2], rel=2e-5)
    assert l2 == pytest.approx(ref["L2"], rel=2e-5)
    S.close()


def test_bicgstab_sliced_ell_and_csr_agree():
    """a heat::Static tangent above the sliced-ELL threshold: the CSR and the
    sliced-ELL SpMV solve it to the tolerance and agree with the direct solve"""
    import scipy.sparse as sp
    from scipy.sparse.linalg import spsolve
    S, P = _both("quad", A.QUAD, 2, (80, 70), "fenics", 13)
    assert S.neq >= 20000 and S.get_option(A.OPT_SCALAR_SLOTS) >= S.nnz
    S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
    rp, ci, v = S.csr()
    b = S.rhs()
    xd = spsolve(sp.csc_matrix(sp.csr_matrix((v, ci, rp))), b)
    out = {}
    for kind in (4, 104, 108):
        S.set_option(A.OPT_BICGSTAB_KIND, kind)
        it, rel, _ = S.solve(A.SOLVE_BICGSTAB, tol=1e-12)
        assert S.get_option(A.OPT_BICGSTAB_KIND) == kind and rel <= 1e-12
        out[kind] = S.solution()
        assert np.linalg.norm(out[kind] - xd) <= 1e-8 * np.linalg.norm(xd)
    # slot-order sums do not depend on the batch depth
    assert np.array_equal(out[104], out[108])
    S.set_option(A.OPT_BICGSTAB_KIND, 0)
    S.solve(A.SOLVE_BICGSTAB, tol=1e-12)
    assert S.get_option(A.OPT_BICGSTAB_KIND) in (2, 4, 8, 16, 102, 104, 108)
    S.close()


# Adams-Moulton is not A-stable beyond order 2, and the trapezoidal rule
# oscillates at large steps: the heat::Static cases keep u > -1, where
# (1 + u)^m is defined, through their step sizes (checked on the oracle)
@pytest.mark.parametrize("kind,shape,deg,sizes,order,scheme,kernel,dt", [
    ("quad", A.QUAD, 2, (8, 6), 2, "bdf", "laplace", 0.01), ("quad", A.QUAD, 1, (12, 9), 3, "bdf", "laplace", 0.01),
    ("tet", A.TET, 2, (3, 3, 2), 2, "bdf", "laplace", 0.01), ("quad", A.QUAD, 2, (8, 6), 2, "am", "laplace", 0.01),
    ("quad", A.QUAD, 1, (10, 7), 3, "am", "laplace", 0.01), ("quad", A.QUAD, 2, (7, 5), 2, "am", "fenics", 1e-3),
    ("quad", A.QUAD, 2, (7, 5), 3, "am", "fenics", 2e-5), ("quad", A.QUAD, 2, (7, 5), 2, "bdf", "fenics", 0.01),
])
def test_unsteady_heat_multistep_matches_oracle(kind, shape, deg, sizes, order, scheme, kernel, dt):
    """BDF and Adams-Moulton time stepping: the inertia terms of
    base/time/ReactionTerms.hpp (mass matrix into the tangent, weighted DOF
    history into the forces) and, for Adams-Moulton, the residual forces at
    past states (ResidualForceHistory.hpp), with the Laplace kernel and with
    heat::Static (two Newton iterations per step): every step's DOF values
    equal the oracle's to 1e-10.  The reference has no golden output for time
    integration (its users are sandbox apps), so this pins the device to the
    oracle's restatement only."""
    import scipy.sparse as sp
    from scipy.sparse.linalg import spsolve
    X, conn = W.unit_cube(kind, *sizes)
    rng = np.random.default_rng(3)
    kappa = rng.uniform(0.5, 2.0, len(conn))
    rho = rng.uniform(0.5, 1.5, len(conn))
    steps = 5
    S = System(device=0)
    S.upload_mesh(shape, X, conn)
    S.create_field(deg, 1)
    S.constrain_boundary(lambda x: (np.ones((len(x), 1), bool), 0.0))
    S.number_dofs()
    S.register_pattern()
    P = O.Problem({A.QUAD: O.QUAD, A.TET: O.TET, A.HEX: O.HEX}[shape], X, conn, deg, 1)
    x, d = P.boundary_points()
    P.constrain(d, np.zeros(len(d)), np.zeros(len(d)))
    P.number()
    newton = 1
    method = A.SOLVE_CG_FP64
    if kernel == "laplace":
        S.set_laplace(kappa, 2)
        P.set_laplace(kappa, 2)
    else:
        S.set_heat_static("fenics", kappa, 2)
        P.set_heat_static("fenics", kappa, 2)
        newton, method = 2, A.SOLVE_BICGSTAB
    # initial values: random on the free DOFs (the constrained ones are 0)
    u0 = rng.uniform(0.0, 1.0, S.ndofobj) * (S.dof_index() >= 0)
    S.set_values(u0)
    gpu = W.unsteady_heat(S, rho, steps, dt, order=order, scheme=scheme, newton=newton, method=method)
    P.set_values(u0)
    hist = [u0.copy()] + [np.zeros_like(u0)] * (order - 1)
    for k in range(steps):
        mw, w, fw = W.time_weights(scheme, order, k, dt)
        P.set_inertia(rho, mw, w, hist[: max(len(w) - 1, len(fw))], fw)
        for _ in range(newton):
            rp, ci, v, b = P.assemble(incremental=True, with_residual=True)
            xs = spsolve(sp.csc_matrix(sp.csr_matrix((v, ci, rp))), b)
            P.distribute(xs, add=True)
        cur = P.values()
        hist = [cur.copy()] + hist[:-1]
        err = np.linalg.norm(gpu[k] - cur) / np.linalg.norm(cur)
        assert err <= 1e-10, (k, err)
    # the solution decays (no source, zero boundary values)
    assert np.linalg.norm(gpu[-1]) < np.linalg.norm(u0)
    S.close()

