"""Neumann tractions on tetrahedron faces (triangle surface rules of
base/quad/GaussTriangle.hpp), through the GPU assembly against the oracle
(base/asmb/NeumannForce.hpp:36-70 with the surface element of
base/mesh/SurfaceElement.hpp):

* P1 and P2 tetrahedra, heat::Laplace with a flux on the x = 1 faces and
  Dirichlet values on x = 0 only (the c3 mesh: jittered interior, planar
  boundary);
* P2 tetrahedra, HyperElastic<StVenant> with a traction on x = 1;

right-hand sides and matrices within 1e-12 of the oracle, and the FP64 CG
solutions within 1e-9 of the oracle's.
"""
import numpy as np
import pytest

import oracle as O
from insilico_gb300 import _abi as A
from insilico_gb300 import workloads as W

from helpers import csr_entry_err, oracle_problem

pytestmark = pytest.mark.gpu


def _x0(ncomp):
    return lambda x: (np.repeat((np.abs(x[:, 0]) < 1e-9)[:, None], ncomp, axis=1), 0.0)


def tet_laplace(deg):
    p = W.config("c3", n=3)
    p.fedeg = deg
    p.dirichlet = _x0(1)
    p.neumann_plane = (0, 1.0, np.array([2.5]))
    return p


def tet_elastic():
    p = W.config("c3", n=3)
    g = W.rng(91, 0)
    lam, mu = W.lame(10.0 ** g.uniform(3.0, 4.0, len(p.conn)), g.uniform(0.2, 0.4, len(p.conn)))
    return W.Problem("tet-elastic", A.TET, p.X, p.conn, 2, 3, "hyperelastic", 2, lam=lam, mu=mu,
                     material="stvenant", dirichlet=_x0(3), neumann_plane=(0, 1.0, np.array([1.0, 0.3, -0.2])))


@pytest.mark.parametrize("case", ["tet_p1", "tet_p2", "tet_p2_elastic"])
def test_neumann_faces_match_oracle(case):
    p = {"tet_p1": lambda: tet_laplace(1), "tet_p2": lambda: tet_laplace(2),
         "tet_p2_elastic": tet_elastic}[case]()
    S = W.setup_system(p)
    P, (rp, ci, v, b) = oracle_problem(p)
    assert S.neq == P.neq
    S.assemble(A.PREC_FP64)
    grp, gci, gv = S.csr()
    np.testing.assert_array_equal(grp, rp)
    np.testing.assert_array_equal(gci, ci)
    assert csr_entry_err(rp, ci, gv, v) <= 1e-12
    gb = S.rhs()
    scale = np.max(np.abs(b))
    assert scale > 0
    assert np.max(np.abs(gb - b)) <= 1e-12 * scale
    S.solve(A.SOLVE_CG_FP64, tol=1e-13)
    xo, _, _ = O.cg(rp, ci, v, b, tol=1e-13)
    assert np.linalg.norm(S.solution() - xo) <= 1e-9 * np.linalg.norm(xo)
    S.close()
