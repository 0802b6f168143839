"""Pin the CPU oracle to the reference's own golden files.

The pins come from tests/golden/reference_pins.json (written by
tests/golden/make_fixtures.py from the reference's *.ref.dat / ref / *.smf):
  * DOF-object numbering + sparsity for Q1/Q2/Q3 on the 20x20 square —
    bit-exact against reference/03-doFHandler/sparsity.{1,2,3}.ref.dat;
  * the unit-cube meshes the reference ships (canonical hash);
  * linear elasticity L2 errors (reference/06-elastic/linearElastic{2,3}D.ref.dat);
  * compressible neo-Hookean Newton histories (reference/06-elastic/compRefOut{D,N}.dat);
  * mixed Poisson (reference/05-mixedPoisson/ref).
The reference prints 6 significant digits; values are compared at 2e-5
relative, and residuals at round-off level (< 1e-11 of the first residual of
the load step) only for being at round-off level.
"""
import sys

import numpy as np
import pytest

import oracle as O

sys.path.insert(0, __import__("os").path.join(__import__("os").path.dirname(__file__), "golden"))
from make_fixtures import lines_hash, mesh_hash  # noqa: E402


def _pad3(X):
    Y = np.zeros((len(X), 3))
    Y[:, : X.shape[1]] = X
    return Y


def test_square20_mesh_matches_reference(pins):
    X, conn = O.unitcube("quad", 20, 20, round6=True)
    assert mesh_hash(_pad3(X), conn) == pins["meshes"]["reference/03-doFHandler/square_20.smf"]["sha256"]


@pytest.mark.parametrize("degree", [1, 2, 3])
def test_sparsity_bit_exact(pins, degree):
    X, conn = O.unitcube("quad", 20, 20, round6=True)
    lines = O.sparsity_lines(degree, X, conn)
    p = pins["sparsity"][str(degree)]
    assert len(lines) == p["lines"]
    assert lines[:12] == p["head"] and lines[-6:] == p["tail"]
    assert lines_hash(lines) == p["sha256"]


@pytest.mark.parametrize("n", [2, 5, 10, 20, 40])
def test_linear_elastic_2d(pins, n):
    ref = dict((a, b) for a, b in pins["linearElastic2D"])[n]
    X, conn = O.unitcube("quad", n, n, round6=True)
    assert mesh_hash(_pad3(X), conn) == pins["meshes"]["reference/06-elastic/quad.%03d.smf" % n]["sha256"]
    assert O.linear_elastic(2, X, conn) == pytest.approx(ref, rel=2e-5)


@pytest.mark.parametrize("n", [2, 4, 8, 12, 16])
def test_linear_elastic_3d(pins, n):
    ref = dict((a, b) for a, b in pins["linearElastic3D"])[n]
    X, conn = O.unitcube("hex", n, n, n, round6=True)
    assert mesh_hash(X, conn) == pins["meshes"]["reference/06-elastic/cube.%03d.smf" % n]["sha256"]
    assert O.linear_elastic(3, X, conn) == pytest.approx(ref, rel=2e-5)


@pytest.mark.parametrize("tag,disp,trac", [("D", True, 1000.0), ("N", False, 300.0)])
def test_compressible_newton_history(pins, tag, disp, trac):
    ref = pins["compRefOut" + tag]
    X, conn = O.unitcube("quad", 20, 20, round6=True)
    n, rows = O.compressible(X, conn, traction=trac, disp_controlled=disp)
    assert n == ref["ndofs"]
    assert len(rows) == len(ref["rows"])
    first = {}
    for got, want in zip(rows, ref["rows"]):
        assert got[:2] == tuple(want[:2])
        first.setdefault(got[0], want[2])
        if want[2] > 1e-11 * first[got[0]]:
            assert got[2] == pytest.approx(want[2], rel=2e-5)
        else:
            assert got[2] < 1e-11 * first[got[0]] * 10
        if len(want) > 3:
            assert got[3] == pytest.approx(want[3], rel=2e-5)


def test_mixed_poisson(pins):
    ref = pins["mixedPoisson"]
    X, conn = O.unitcube("quad", 20, 20, round6=True)
    n, l2, h1 = O.mixed_poisson(X, conn)
    assert n == ref["ndofs"]
    assert l2 == pytest.approx(ref["L2"], rel=2e-5)
    assert h1 == pytest.approx(ref["H1"], rel=2e-5)


def test_nonlinear_heat(pins):
    """reference/04-heat/nonlinearHeat.cpp on square_200.smf: Q2 heat::Static
    with FenicsTest conductivity, Newton with a direct solve of the
    non-symmetric tangent"""
    ref = pins["nonlinearHeat"]
    X, conn = O.unitcube("quad", 200, 200, round6=True)
    assert mesh_hash(_pad3(X), conn) == pins["meshes"]["reference/04-heat/square_200.smf"]["sha256"]
    n, rows, l2, _ = O.nonlinear_heat(X, conn)
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
