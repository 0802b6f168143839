"""Post-processing on the GPU (base/post/ErrorNorm.hpp): the quadrature-point
coordinates and the L2 / H1 error norms, against the reference's golden L2
errors of reference/06-elastic (the whole pipeline on the GPU) and against the
oracle's error norm on the same DOF values."""
import numpy as np
import pytest

import oracle as O
from insilico_gb300 import _abi as A
from insilico_gb300 import workloads as W
from insilico_gb300.system import System

pytestmark = pytest.mark.gpu


def _elastic_params(dim, E=1000.0, nu=0.25):
    """reference/06-elastic/linearElastic.cpp: Kelvin solution, point force
    (0, 1, 0) at (-0.1, -0.1, -0.1)"""
    lam, mu = O.lame(E, nu)
    prm = np.zeros(8)
    prm[0], prm[1] = lam, mu
    prm[2:2 + dim] = -0.1
    prm[6] = 1.0
    return lam, mu, prm


def _gpu_linear_elastic(dim, n):
    X, conn = O.unitcube("quad" if dim == 2 else "hex", *([n] * dim), round6=True)
    lam, mu, prm = _elastic_params(dim)
    S = System(device=0)
    S.upload_mesh(A.QUAD if dim == 2 else A.HEX, X, conn)
    S.create_field(1, dim)
    S.constrain_boundary(lambda x: (np.ones((len(x), dim), bool), O.eval_refsol(0, prm, x)))
    S.number_dofs()
    S.register_pattern()
    S.set_hyperelastic("stvenant", np.full(len(conn), lam), np.full(len(conn), mu), 3)
    S.assemble(A.PREC_FP64)
    S.solve(A.SOLVE_CG_FP64, tol=2.220446049250313e-16)
    S.distribute()
    return S, X, conn, prm


@pytest.mark.parametrize("n", [2, 4, 8, 12])
def test_linear_elastic_l2_error_matches_reference_golden(pins, n):
    """3-D (the device's HyperElastic kernel is the trilinear hexahedron):
    Quadrature<3, HEX> = 2 x 2 x 2 points, as linearElastic.cpp uses"""
    dim = 3
    ref = dict((a, b) for a, b in pins["linearElastic%dD" % dim])[n]
    S, X, conn, prm = _gpu_linear_elastic(dim, n)
    xq = S.quadrature_points(3)
    assert xq.shape == (len(conn) * 2 ** dim, dim)
    err = S.error_norm(0, 3, O.eval_refsol(0, prm, xq))
    assert err == pytest.approx(ref, rel=2e-5)
    # the same DOF values through the oracle's error norm (sequential sum)
    P = O.Problem(O.QUAD if dim == 2 else O.HEX, X, conn, 1, dim)
    P.set_values(S.values())
    assert err == pytest.approx(P.error_norm(0, prm, 0, 3), rel=1e-12)
    again = S.error_norm(0, 3, O.eval_refsol(0, prm, xq))
    assert again == err  # fixed reduction order
    S.close()


def _cos_product(alpha, x):
    """u = prod_d cos(alpha_d x_d) and its gradient (the oracle's reference
    solution kind 1, reference/05-mixedPoisson)"""
    c = np.cos(alpha[None, :] * x)
    s = np.sin(alpha[None, :] * x)
    u = np.prod(c, axis=1)
    g = np.empty_like(x)
    for d in range(x.shape[1]):
        g[:, d] = -alpha[d] * s[:, d] * np.prod(np.delete(c, d, axis=1), axis=1)
    return u, g


@pytest.mark.parametrize("kind,shape,deg,sizes,qdeg", [
    ("quad", A.QUAD, 2, (9, 7), 3), ("quad", A.QUAD, 1, (12, 10), 2), ("tet", A.TET, 2, (3, 4, 2), 2),
    ("hex", A.HEX, 1, (4, 3, 5), 3), ("tet", A.TET, 1, (3, 3, 3), 1),
    ("tet", A.TET, 2, (3, 4, 2), 4),  # the 11-point rule of P2 tetrahedra
])
def test_error_norms_match_oracle(kind, shape, deg, sizes, qdeg):
    """L2 and H1 errors of an arbitrary field against u = prod cos(alpha x):
    the device sum equals the oracle's sequential sum to 1e-12"""
    X, conn = W.unit_cube(kind, *sizes)
    dim = X.shape[1]
    alpha = np.array([3.0, 5.0, 4.0])[:dim]
    prm = np.zeros(3)
    prm[:dim] = alpha
    S = System(device=0)
    S.upload_mesh(shape, X, conn)
    S.create_field(deg, 1)
    rng = np.random.default_rng(11)
    u = rng.standard_normal(S.ndofobj)
    S.set_values(u)
    xq = S.quadrature_points(qdeg)
    uref, gref = _cos_product(alpha, xq)
    l2 = S.error_norm(0, qdeg, uref[:, None])
    h1 = S.error_norm(1, qdeg, gref[:, None, :])
    P = O.Problem({A.QUAD: O.QUAD, A.TET: O.TET, A.HEX: O.HEX}[shape], X, conn, deg, 1)
    P.set_values(u)
    assert l2 == pytest.approx(P.error_norm(1, prm, 0, qdeg), rel=1e-12)
    assert h1 == pytest.approx(P.error_norm(1, prm, 1, qdeg), rel=1e-12)
    S.close()


def test_quadrature_points_are_the_mapped_rule():
    """x_q = sum_i N_i(xi_q) X_i: on the affine unit square grid, the 2x2 rule
    of element e sits at the element's corner + h * (0.211..., 0.788...), in
    the rule's order (first coordinate fastest) when the element's local axes
    follow x and y"""
    X, conn = W.unit_cube("quad", 4, 4)
    S = System(device=0)
    S.upload_mesh(A.QUAD, X, conn)
    S.create_field(1, 1)
    xq = S.quadrature_points(2).reshape(len(conn), 4, 2)
    lo = X[conn].min(axis=1)
    g = np.array([0.788675134594813, 0.211324865405187])
    want = np.array([[g[i], g[j]] for j in range(2) for i in range(2)])  # first coordinate fastest
    np.testing.assert_allclose(xq - lo[:, None, :], np.broadcast_to(0.25 * want, xq.shape), rtol=0, atol=1e-15)
    with pytest.raises(A.IslError):
        S.error_norm(2, 2, np.zeros(len(conn) * 4))
    S.close()
