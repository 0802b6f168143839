"""solid::HyperElastic in 2-D (plane strain) on the GPU: Q1 / Q2
quadrilaterals, tangent and residual against the oracle, tractions given at
face vertices, the inertia terms, and the whole Newton runs of
reference/06-elastic/compressible.cpp against its golden output
(compRefOut{D,N}.dat)."""
import numpy as np
import pytest

import oracle as O
from insilico_gb300 import _abi as A
from insilico_gb300 import workloads as W
from insilico_gb300.system import System

from helpers import csr_entry_err

pytestmark = pytest.mark.gpu


def _sheet(nx, ny, seed):
    """unit square of nx x ny quadrilaterals, interior nodes jittered"""
    X, conn = W.unit_cube("quad", nx, ny)
    rng = np.random.default_rng(seed)
    inner = np.all((X > 1e-9) & (X < 1 - 1e-9), axis=1)
    return X + rng.uniform(-0.04, 0.04, X.shape) * inner[:, None], conn, rng


def _both(X, conn, deg, material, lam, mu, qdeg, value):
    """the same sheet, clamped at x = 0 to `value`, on the GPU and on the oracle"""
    S = System(device=0)
    S.upload_mesh(A.QUAD, X, conn)
    S.create_field(deg, 2)
    S.constrain_boundary(lambda x: (np.repeat((np.abs(x[:, 0]) < 1e-9)[:, None], 2, axis=1), value))
    S.number_dofs()
    S.register_pattern()
    S.set_hyperelastic(material, lam, mu, qdeg)
    P = O.Problem(O.QUAD, X, conn, deg, 2)
    x, d = P.boundary_points()
    on = np.abs(x[:, 0]) < 1e-9
    dd = np.repeat(d[on], 2)
    P.constrain(dd, np.tile(np.arange(2), on.sum()), np.full(len(dd), value))
    P.number()
    P.set_hyperelastic(material, lam, mu, qdeg)
    return S, P


def _check(S, P):
    S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
    rp, ci, v, b = P.assemble(incremental=True, with_residual=True)
    srp, sci, sv = S.csr()
    np.testing.assert_array_equal(srp, rp)
    np.testing.assert_array_equal(sci, ci)
    assert csr_entry_err(rp, ci, sv, v) <= 1e-12
    assert np.max(np.abs(S.rhs() - b)) <= 1e-12 * np.max(np.abs(b))


@pytest.mark.parametrize("deg", [1, 2])
@pytest.mark.parametrize("qdeg", [3, 5])
@pytest.mark.parametrize("material", ["stvenant", "neohooke"])
def test_quad_hyperelastic_tangent_and_residual_match_oracle(deg, qdeg, material):
    """at a displacement, with a nodal body force and a nonzero Dirichlet
    value lifted into the right-hand side"""
    X, conn, rng = _sheet(5, 4, 3)
    lam, mu = rng.uniform(1.0, 2.0, len(conn)), rng.uniform(0.5, 1.0, len(conn))
    S, P = _both(X, conn, deg, material, lam, mu, qdeg, 0.01)
    u = rng.uniform(-0.02, 0.02, 2 * S.ndofobj)
    f = rng.uniform(-1.0, 1.0, (len(X), 2))
    S.set_values(u)
    S.set_body_force_nodal(f)
    P.set_values(u)
    P.set_body_nodal(f.reshape(-1))
    _check(S, P)
    S.close()


def test_vertex_traction_matches_pulled_sheet():
    """the traction (value (y - 1/2), 0) on x = 1 of PulledSheet.hpp, evaluated
    at the surface points by the oracle and interpolated from the face
    vertices on the GPU, gives the same forces; a traction that is the same
    at both vertices equals the constant-per-face path"""
    X, conn, rng = _sheet(6, 5, 5)
    lam, mu = np.full(len(conn), 1.5), np.full(len(conn), 0.8)
    S, P = _both(X, conn, 2, "neohooke", lam, mu, 3, 0.0)
    fe, ff, fy = W.pulled_sheet_faces(S, X, conn)
    assert len(fe) == 5
    t = np.zeros((len(fe), 2, 2))
    t[:, :, 0] = 300.0 * (fy - 0.5)
    S.set_neumann_vertex(fe, ff, t, 3)
    be, bf = P.boundary_faces()
    P.set_neumann("pulledsheet", be, bf, None, 300.0, 3)
    _check(S, P)
    S.set_neumann_vertex(fe, ff, np.array([2.0, -1.0]), 3)
    S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
    b_vertex = S.rhs()
    S.set_neumann(fe, ff, np.array([2.0, -1.0]), 3)
    S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
    # the face functions sum to 1 up to rounding at the surface points
    assert np.max(np.abs(S.rhs() - b_vertex)) <= 1e-14 * np.max(np.abs(b_vertex))
    S.close()


@pytest.mark.parametrize("deg,nfw", [(2, 0), (1, 2)])
def test_quad_inertia_terms_match_oracle(deg, nfw):
    """mass per component, weighted history and residual forces at past
    states on quadrilaterals"""
    X, conn, rng = _sheet(4, 4, 9)
    lam, mu = rng.uniform(1.0, 2.0, len(conn)), rng.uniform(0.5, 1.0, len(conn))
    rho = rng.uniform(0.5, 1.5, len(conn))
    S, P = _both(X, conn, deg, "neohooke", lam, mu, 3, 0.01)
    n2 = 2 * S.ndofobj
    h2, h1, u = (rng.uniform(-0.02, 0.02, n2) for _ in range(3))
    S.set_history(2)
    S.set_values(h2)
    S.push_history()
    S.set_values(h1)
    S.push_history()
    S.set_values(u)
    w, fw = [5.0, -6.0, 1.0], [0.5, -0.25][:nfw]
    S.set_inertia(rho, 9.0, w)
    S.set_force_history(fw)
    P.set_values(u)
    P.set_inertia(rho, 9.0, w, [h1, h2], fw)
    _check(S, P)
    S.close()


@pytest.mark.parametrize("tag,disp,trac", [("D", True, 1000.0), ("N", False, 300.0)])
def test_compressible_matches_reference_golden(pins, tag, disp, trac):
    """reference/06-elastic/compressible.cpp on quad.020.smf (Q2,
    NeoHookeanCompressible, five load steps): the Newton history |R|, |x| per
    iteration, to the 6 digits of compRefOut{D,N}.dat, on the GPU"""
    ref = pins["compRefOut" + tag]
    X, conn = O.unitcube("quad", 20, 20, round6=True)
    S = System(device=0)
    n, rows = W.compressible(S, X, conn, traction=trac, disp_controlled=disp)
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
    S.close()
