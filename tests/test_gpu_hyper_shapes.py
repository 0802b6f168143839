"""solid::HyperElastic on tetrahedra (P1, P2) and on trilinear hexahedra with
a 3x3x3 rule, on the GPU (the one-thread-per-element kernel k_hyper_elem of
isl_hyper.cu): tangent and residual at a displacement, with a nodal body
force and lifted Dirichlet values, and the inertia terms, against the
oracle; a Newton solve of a clamped P2 block against the oracle's."""
import numpy as np
import pytest

import oracle as O
from insilico_gb300 import _abi as A
from insilico_gb300 import workloads as W
from insilico_gb300.system import System

from helpers import csr_entry_err

pytestmark = pytest.mark.gpu

SHAPES = {"tet": (A.TET, O.TET), "hex": (A.HEX, O.HEX)}


def _both(kind, sizes, deg, material, qdeg, value, seed):
    """a jittered block clamped at x = 0 to `value`, on the GPU and on the oracle"""
    X, conn = W.unit_cube(kind, *sizes)
    rng = np.random.default_rng(seed)
    inner = np.all((X > 1e-9) & (X < 1 - 1e-9), axis=1)
    X = X + rng.uniform(-0.01, 0.01, X.shape) * inner[:, None]
    lam, mu = rng.uniform(1.0, 2.0, len(conn)), rng.uniform(0.5, 1.0, len(conn))
    ashape, oshape = SHAPES[kind]
    S = System(device=0)
    S.upload_mesh(ashape, X, conn)
    S.create_field(deg, 3)
    S.constrain_boundary(lambda x: (np.repeat((np.abs(x[:, 0]) < 1e-9)[:, None], 3, axis=1), value))
    S.number_dofs()
    S.register_pattern()
    S.set_hyperelastic(material, lam, mu, qdeg)
    P = O.Problem(oshape, X, conn, deg, 3)
    x, d = P.boundary_points()
    on = np.abs(x[:, 0]) < 1e-9
    dd = np.repeat(d[on], 3)
    P.constrain(dd, np.tile(np.arange(3), on.sum()), np.full(len(dd), value))
    P.number()
    P.set_hyperelastic(material, lam, mu, qdeg)
    return S, P, X, rng


def _check(S, P):
    S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
    rp, ci, v, b = P.assemble(incremental=True, with_residual=True)
    srp, sci, sv = S.csr()
    np.testing.assert_array_equal(srp, rp)
    np.testing.assert_array_equal(sci, ci)
    assert csr_entry_err(rp, ci, sv, v) <= 1e-12
    assert np.max(np.abs(S.rhs() - b)) <= 1e-12 * np.max(np.abs(b))


@pytest.mark.parametrize("kind,sizes,deg,qdeg", [
    ("tet", (3, 2, 2), 1, 2), ("tet", (3, 2, 2), 1, 1), ("tet", (2, 2, 1), 2, 2), ("hex", (3, 2, 2), 1, 4),
])
@pytest.mark.parametrize("material", ["stvenant", "neohooke"])
def test_hyperelastic_shapes_match_oracle(kind, sizes, deg, qdeg, material):
    S, P, X, rng = _both(kind, sizes, deg, material, qdeg, 0.01, 3)
    u = rng.uniform(-0.01, 0.01, 3 * S.ndofobj)
    f = rng.uniform(-1.0, 1.0, (len(X), 3))
    S.set_values(u)
    S.set_body_force_nodal(f)
    P.set_values(u)
    P.set_body_nodal(f.reshape(-1))
    _check(S, P)
    S.close()


def test_p2_tet_inertia_terms_match_oracle():
    S, P, X, rng = _both("tet", (2, 2, 1), 2, "neohooke", 2, 0.01, 5)
    rho = rng.uniform(0.5, 1.5, len(P.conn))
    n3 = 3 * S.ndofobj
    h2, h1, u = (rng.uniform(-0.01, 0.01, n3) for _ in range(3))
    S.set_history(2)
    S.set_values(h2)
    S.push_history()
    S.set_values(h1)
    S.push_history()
    S.set_values(u)
    S.set_inertia(rho, 6.0, [4.0, -5.0, 1.0])
    S.set_force_history([0.5, -0.25])
    P.set_values(u)
    P.set_inertia(rho, 6.0, [4.0, -5.0, 1.0], [h1, h2], [0.5, -0.25])
    _check(S, P)
    S.close()


def test_p2_tet_newton_matches_oracle():
    """a NeoHookean P2 block clamped at x = 0 under a nodal body force: three
    Newton iterations (CG on the GPU, a direct solve on the oracle) reach the
    same displacement"""
    import scipy.sparse as sp
    from scipy.sparse.linalg import spsolve
    S, P, X, rng = _both("tet", (3, 2, 2), 2, "neohooke", 2, 0.0, 7)
    f = np.zeros((len(X), 3))
    f[:, 2] = -0.02
    S.set_body_force_nodal(f)
    P.set_body_nodal(f.reshape(-1))
    for _ in range(3):
        S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
        S.solve(A.SOLVE_CG_FP64, tol=1e-13)
        S.distribute(add=True)
        rp, ci, v, b = P.assemble(incremental=True, with_residual=True)
        P.distribute(spsolve(sp.csc_matrix(sp.csr_matrix((v, ci, rp))), b), add=True)
    u, uo = S.values(), P.values()
    assert np.linalg.norm(uo) > 1e-3
    assert np.linalg.norm(u - uo) <= 1e-9 * np.linalg.norm(uo)
    S.close()
