"""Quadrature rules of the element kernels (CPU, no GPU): the rules the
device library tabulates (isl_quadrature_rule) equal the oracle's bit for
bit, and integrate monomials up to their degree exactly up to the
reference's truncated constants (base/quad/GaussLegendre.hpp:115-134,
base/quad/GaussTetrahedron.hpp:93-175, and the triangle surface rules of
base/quad/GaussTriangle.hpp:97-180)."""
from math import factorial

import numpy as np
import pytest

import oracle as O
from insilico_gb300 import _abi as A


@pytest.mark.parametrize("shape,oshape", [(A.TET, O.TET), (A.QUAD, O.QUAD), (A.HEX, O.HEX), (A.TRI, O.TRI)])
@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5])
def test_rules_match_oracle_and_are_exact(shape, oshape, degree):
    w, x = A.quadrature_rule(shape, degree)
    wo, xo = O.quadrature(oshape, degree)
    assert np.array_equal(w, wo) and np.array_equal(x, xo)
    dim = x.shape[1]
    worst = 0.0
    for p in np.ndindex(*([degree + 1] * dim)):
        if shape in (A.TET, A.TRI):  # simplex: exact for total degree up to the rule's
            if sum(p) > degree:
                continue
            exact = np.prod([factorial(k) for k in p]) / factorial(sum(p) + dim)
        else:  # tensor rule on [0,1]^dim: exact per coordinate up to the degree
            exact = np.prod([1.0 / (k + 1) for k in p])
        got = np.sum(w * np.prod(x ** np.array(p), axis=1))
        worst = max(worst, abs(got - exact) / exact)
    assert worst <= 5e-14


def test_tet_rule_sizes_and_limits():
    """1, 4, 5, 11 and 15 points for degrees 1 to 5 (the 5-point rule has a
    negative centroid weight); no rule above degree 5"""
    sizes = [len(A.quadrature_rule(A.TET, d)[0]) for d in range(1, 6)]
    assert sizes == [1, 4, 5, 11, 15]
    assert A.quadrature_rule(A.TET, 3)[0][0] < 0
    for bad in (6, 0, -1):
        with pytest.raises(A.IslError):
            A.quadrature_rule(A.TET, bad)
    for shape in (A.QUAD, A.HEX):
        for bad in (0, 6):
            with pytest.raises(A.IslError):
                A.quadrature_rule(shape, bad)
    assert O.quadrature(O.TET, 6) is None


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5])
def test_oracle_triangle_rules_are_exact(degree):
    """the oracle's surface rules on triangles (base/quad/GaussTriangle.hpp,
    degrees 1-5, truncated constants): 1, 3, 4, 6, 7 points, exact for
    monomials up to their degree"""
    w, x = O.quadrature(O.TRI, degree)
    assert len(w) == [1, 3, 4, 6, 7][degree - 1]
    for a in range(degree + 1):
        for b in range(degree + 1 - a):
            exact = factorial(a) * factorial(b) / factorial(a + b + 2)
            got = np.sum(w * x[:, 0] ** a * x[:, 1] ** b)
            assert abs(got - exact) <= 5e-14 * max(exact, 1e-3) + 2e-15, (a, b, got, exact)
