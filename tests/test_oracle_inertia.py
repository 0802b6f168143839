"""Vector-field inertia terms of the oracle (CPU).  The mass of a
displacement field acts on each component (base/kernel/Mass.hpp:84-86,
M[M*d+i][N*d+i]), so what a HyperElastic problem gains from the inertia
terms is the scalar mass of the same mesh once per component, in the matrix
and, times the weighted history, in the forces."""
import numpy as np
import scipy.sparse as sp

import oracle as O
from insilico_gb300 import workloads as W


def _dense(rp, ci, v, n):
    return sp.csr_matrix((v, ci, rp), shape=(n, n)).toarray()


def test_vector_mass_is_the_scalar_mass_per_component():
    X, conn = W.unit_cube("hex", 3, 2, 2)
    rng = np.random.default_rng(4)
    rho = rng.uniform(0.5, 1.5, len(conn))
    # scalar mass: Laplace with and without the inertia terms
    Ps = O.Problem(O.HEX, X, conn, 1, 1)
    Ps.number()
    Ps.set_laplace(np.ones(len(conn)), 2)
    rp, ci, v0, _ = Ps.assemble()
    Ps.set_inertia(rho, 1.0, [1.0], [])
    _, _, v1, _ = Ps.assemble()
    n = Ps.ndofobj
    es = Ps.eq_index()
    Ms = _dense(rp, ci, v1 - v0, n)[np.ix_(es, es)]       # by DOF object
    assert np.allclose(Ms, Ms.T) and Ms.sum() > 0
    # vector field: HyperElastic at a displacement, history x^(0) = u
    Pv = O.Problem(O.HEX, X, conn, 1, 3)
    Pv.number()
    np.testing.assert_array_equal(Pv.elem_dofobj(), Ps.elem_dofobj())
    Pv.set_hyperelastic("neohooke", rng.uniform(1, 2, len(conn)), rng.uniform(0.5, 1, len(conn)), 2)
    u = rng.uniform(-0.02, 0.02, 3 * n)
    Pv.set_values(u)
    rp, ci, w0, b0 = Pv.assemble(incremental=True, with_residual=True)
    Pv.set_inertia(rho, 2.5, [1.0], [])
    _, _, w1, b1 = Pv.assemble(incremental=True, with_residual=True)
    ev = Pv.eq_index()
    Mv = _dense(rp, ci, w1 - w0, 3 * n)[np.ix_(ev, ev)]   # by (DOF object, component)
    np.testing.assert_allclose(Mv, 2.5 * np.kron(Ms, np.eye(3)), atol=1e-14 * np.abs(Ms).max())
    fv = (b1 - b0)[ev]
    np.testing.assert_allclose(fv, np.kron(Ms, np.eye(3)) @ u, atol=1e-14 * np.abs(Ms).max())
