"""Time-integration terms of a vector field on the GPU: HyperElastic
(trilinear hexahedra) with the inertia terms of base/time/ReactionTerms.hpp
(the mass on each displacement component, base/kernel/Mass.hpp:84-86) and
the residual forces at past states (base/time/ResidualForceHistory.hpp),
against the oracle: the assembled system at given histories, and whole BDF /
Adams-Moulton runs step by step.  The reference has no golden output for time
integration (its users are sandbox apps), so this pins the device to the
oracle's restatement only."""
import numpy as np
import pytest

import oracle as O
from insilico_gb300 import _abi as A
from insilico_gb300 import workloads as W
from insilico_gb300.system import System

from helpers import csr_entry_err

pytestmark = pytest.mark.gpu


def _mesh(seed):
    """4 x 3 x 3 hexahedra, interior nodes jittered (non-affine elements)"""
    X, conn = W.unit_cube("hex", 4, 3, 3)
    rng = np.random.default_rng(seed)
    inner = np.all((X > 1e-9) & (X < 1 - 1e-9), axis=1)
    X = X + rng.uniform(-0.03, 0.03, X.shape) * inner[:, None]
    return X, conn, rng


def _both(X, conn, material, lam, mu, value):
    """the same clamped (x = 0) HyperElastic problem on the GPU and on the oracle"""
    S = System(device=0)
    S.upload_mesh(A.HEX, X, conn)
    S.create_field(1, 3)
    S.constrain_boundary(lambda x: (np.repeat((np.abs(x[:, 0]) < 1e-9)[:, None], 3, axis=1), value))
    S.number_dofs()
    S.register_pattern()
    S.set_hyperelastic(material, lam, mu, 2)
    P = O.Problem(O.HEX, X, conn, 1, 3)
    x, d = P.boundary_points()
    on = np.abs(x[:, 0]) < 1e-9
    dd = np.repeat(d[on], 3)
    P.constrain(dd, np.tile(np.arange(3), on.sum()), np.full(len(dd), value))
    P.number()
    P.set_hyperelastic(material, lam, mu, 2)
    return S, P


@pytest.mark.parametrize("material", ["stvenant", "neohooke"])
@pytest.mark.parametrize("nfw", [0, 2])
def test_hyperelastic_inertia_terms_match_oracle(material, nfw):
    """tangent and right-hand side with the mass, the weighted history and
    (nfw > 0) the residual forces at two past states, at a displacement, with
    a nonzero Dirichlet value lifted through the mass"""
    X, conn, rng = _mesh(7)
    lam, mu = rng.uniform(1.0, 2.0, len(conn)), rng.uniform(0.5, 1.0, len(conn))
    rho = rng.uniform(0.5, 1.5, len(conn))
    S, P = _both(X, conn, material, lam, mu, 0.01)
    n3 = 3 * S.ndofobj
    h2, h1, u = (rng.uniform(-0.03, 0.03, n3) for _ in range(3))
    S.set_history(2)
    S.set_values(h2)
    S.push_history()
    S.set_values(h1)
    S.push_history()
    S.set_values(u)
    w, fw = [7.0, -9.0, 2.0], [0.4, -0.1][:nfw]
    S.set_inertia(rho, 12.5, w)
    S.set_force_history(fw)
    S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
    P.set_values(u)
    P.set_inertia(rho, 12.5, w, [h1, h2], fw)
    rp, ci, v, b = P.assemble(incremental=True, with_residual=True)
    srp, sci, sv = S.csr()
    np.testing.assert_array_equal(srp, rp)
    np.testing.assert_array_equal(sci, ci)
    assert csr_entry_err(rp, ci, sv, v) <= 1e-12
    assert np.max(np.abs(S.rhs() - b)) <= 1e-12 * np.max(np.abs(b))
    # the plain assembly afterwards is the plain assembly
    S.set_inertia(None, 0.0, [])
    S.set_force_history([])
    S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
    P.set_inertia(None, 0.0, [], [])
    rp, ci, v, b = P.assemble(incremental=True, with_residual=True)
    assert csr_entry_err(rp, ci, S.csr()[2], v) <= 1e-12
    assert np.max(np.abs(S.rhs() - b)) <= 1e-12 * np.max(np.abs(b))
    S.close()


@pytest.mark.parametrize("scheme,order,material", [
    ("bdf", 2, "neohooke"), ("bdf", 3, "stvenant"), ("am", 2, "neohooke"), ("am", 3, "stvenant"),
])
def test_hyperelastic_multistep_matches_oracle(scheme, order, material):
    """rho du/dt + F_int(u) = 0 from a random initial displacement, clamped
    at x = 0: two Newton iterations per step, every step's DOF values equal
    the oracle's to 1e-10, and the motion decays"""
    import scipy.sparse as sp
    from scipy.sparse.linalg import spsolve
    X, conn, rng = _mesh(11)
    lam, mu = rng.uniform(1.0, 2.0, len(conn)), rng.uniform(0.5, 1.0, len(conn))
    rho = rng.uniform(0.5, 1.5, len(conn))
    dt = 0.01 if scheme == "bdf" else 2e-3
    steps = 4
    S, P = _both(X, conn, material, lam, mu, 0.0)
    u0 = rng.uniform(-0.05, 0.05, 3 * S.ndofobj) * (S.dof_index() >= 0)
    S.set_values(u0)
    gpu = W.unsteady(S, rho, steps, dt, order=order, scheme=scheme, newton=2, method=A.SOLVE_CG_FP64, lin_tol=1e-13)
    P.set_values(u0)
    hist = [u0.copy()] + [np.zeros_like(u0)] * (order - 1)
    for k in range(steps):
        mw, w, fw = W.time_weights(scheme, order, k, dt)
        P.set_inertia(rho, mw, w, hist[: max(len(w) - 1, len(fw))], fw)
        for _ in range(2):
            rp, ci, v, b = P.assemble(incremental=True, with_residual=True)
            P.distribute(spsolve(sp.csc_matrix(sp.csr_matrix((v, ci, rp))), b), add=True)
        cur = P.values()
        hist = [cur.copy()] + hist[:-1]
        err = np.linalg.norm(gpu[k] - cur) / np.linalg.norm(cur)
        assert err <= 1e-10, (k, err)
    assert np.linalg.norm(gpu[-1]) < np.linalg.norm(u0)
    S.close()


def test_history_shrunk_below_the_weights_is_refused():
    """weights set for a longer history than isl_set_history keeps afterwards
    are an argument error at the next assembly, not a read past the history"""
    X, conn, rng = _mesh(3)
    S, _ = _both(X, conn, "stvenant", np.ones(len(conn)), np.ones(len(conn)), 0.0)
    S.set_history(2)
    S.set_inertia(np.ones(len(conn)), 1.0, [1.0, -1.0, 0.5])
    S.set_force_history([0.5, 0.5])
    S.set_history(1)
    with pytest.raises(A.IslError, match="past the stored history"):
        S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
    S.set_force_history([0.5])
    S.set_inertia(np.ones(len(conn)), 1.0, [1.0, -1.0])
    S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
    S.close()
