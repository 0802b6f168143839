"""Conductivity that varies inside the elements (heat/Laplace.hpp:119-120:
conductivityFun_(geomEp, xi) at every quadrature point).

* CPU: the oracle with a per-point table that is constant on each element
  gives exactly the per-element system.
* GPU: isl_set_laplace_qp with kappa(x) = 1 + x0^2 + 3 x1 x_last evaluated at
  the library's quadrature points matches the oracle's per-point assembly
  (entries and right-hand side to 1e-12) on Q1 / Q2 quadrilaterals and P2
  tetrahedra, and differs from the per-element (centroid) tabulation.
"""
import numpy as np
import pytest

import oracle as O
from insilico_gb300 import _abi as A
from insilico_gb300 import workloads as W

from helpers import SHAPE_TO_ORACLE, csr_entry_err


def kappa_fn(x):
    return 1.0 + x[:, 0] ** 2 + 3.0 * x[:, 1] * x[:, -1]


def case(kind, deg, n):
    if kind == "quad":
        X, conn = W.unit_cube("quad", n, n + 1)
        shape = A.QUAD
    else:
        X, conn = W.unit_cube("tet", n, n, n)
        shape = A.TET
    f = W.rng(91, 1).uniform(0.0, 1.0, len(X))[:, None]
    return shape, X, conn, deg, f


def oracle_system(shape, X, conn, deg, f, kq=None, ke=None, qdeg=None):
    P = O.Problem(SHAPE_TO_ORACLE[shape], X, conn, deg, 1)
    x, d = P.boundary_points()
    P.constrain(d, np.zeros(len(d), dtype=np.int32), 0.1 * x[:, 0])
    P.number()
    if kq is not None:
        P.set_laplace_qp(kq, qdeg)
    else:
        P.set_laplace(ke, qdeg)
    P.set_body_nodal(f)
    return P.assemble(incremental=False)


def test_oracle_pointwise_table_constant_per_element_is_the_element_table():
    shape, X, conn, deg, f = case("quad", 2, 5)
    ke = W.rng(5, 0).uniform(0.5, 2.0, len(conn))
    nq = len(O.quadrature(SHAPE_TO_ORACLE[shape], 4)[0])
    a = oracle_system(shape, X, conn, deg, f, ke=ke, qdeg=4)
    b = oracle_system(shape, X, conn, deg, f, kq=np.repeat(ke[:, None], nq, axis=1), qdeg=4)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,deg,qdeg", [("quad", 1, 2), ("quad", 2, 4), ("tet", 2, 2), ("tet", 2, 4)])
def test_pointwise_conductivity_matches_oracle(kind, deg, qdeg):
    from insilico_gb300.system import System
    shape, X, conn, deg, f = case(kind, deg, 4 if kind == "tet" else 7)
    S = System()
    S.upload_mesh(shape, X, conn)
    S.create_field(deg, 1)
    S.constrain_boundary(lambda x: (np.ones((len(x), 1), dtype=bool), 0.1 * x[:, :1]))
    S.number_dofs()
    S.register_pattern()
    xq = S.quadrature_points(qdeg)
    nq = len(A.quadrature_rule(shape, qdeg)[0])
    kq = kappa_fn(xq).reshape(len(conn), nq)
    S.set_laplace_qp(kq, qdeg)
    S.set_body_force_nodal(f)
    S.assemble(A.PREC_FP64, incremental=False)
    rp, ci, v = S.csr()
    b = S.rhs()
    orp, oci, ov, ob = oracle_system(shape, X, conn, deg, f, kq=kq, qdeg=qdeg)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    assert csr_entry_err(orp, oci, v, ov) <= 1e-12
    assert np.max(np.abs(b - ob)) <= 1e-12 * np.max(np.abs(ob))
    # the centroid tabulation is a different operator
    _, _, ovc, _ = oracle_system(shape, X, conn, deg, f, ke=kq.mean(axis=1), qdeg=qdeg)
    assert csr_entry_err(orp, oci, v, ovc) > 1e-6
    S.close()
