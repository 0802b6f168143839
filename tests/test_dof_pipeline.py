"""The product's host DOF pipeline (host-only isl_ctx, no GPU) against the
oracle and the reference's golden sparsity files: DOF-object ids, boundary
support points and numbering must be bit-exact."""
import sys

import numpy as np
import pytest

import oracle as O
from insilico_gb300 import _abi as A
from insilico_gb300 import workloads as W
from insilico_gb300.system import System

sys.path.insert(0, __import__("os").path.join(__import__("os").path.dirname(__file__), "golden"))
from make_fixtures import lines_hash  # noqa: E402
from helpers import SHAPE_TO_ORACLE, oracle_problem  # noqa: E402


def host_system(shape, X, conn, deg, ncomp):
    S = System(device=-1)
    S.upload_mesh(shape, X, conn)
    S.create_field(deg, ncomp)
    return S


@pytest.mark.parametrize("degree", [1, 2, 3])
def test_product_sparsity_matches_reference_golden(pins, degree):
    X, conn = O.unitcube("quad", 20, 20, round6=True)
    S = host_system(A.QUAD, X, conn, degree, 1)
    ed = S.elem_dofobj()
    pairs = set()
    n = S.ndofobj
    nf = ed.shape[1]
    r = np.repeat(ed, nf, axis=1).ravel()
    c = np.tile(ed, (1, nf)).ravel()
    key = np.unique(r * n + c)
    lines = [f"{k // n} {k % n}" for k in key.tolist()]
    p = pins["sparsity"][str(degree)]
    assert len(lines) == p["lines"]
    assert lines_hash(lines) == p["sha256"]


@pytest.mark.parametrize("kind,shape,deg,ncomp,args", [
    ("quad", A.QUAD, 1, 1, (7, 5)), ("quad", A.QUAD, 2, 1, (6, 4)), ("quad", A.QUAD, 3, 1, (3, 3)),
    ("quad", A.QUAD, 2, 2, (4, 5)), ("hex", A.HEX, 1, 3, (3, 4, 2)), ("hex", A.HEX, 2, 1, (2, 2, 3)),
    ("tet", A.TET, 2, 1, (3, 2, 2)), ("tet", A.TET, 1, 1, (2, 2, 2)),
])
def test_dofobj_ids_and_boundary_match_oracle(kind, shape, deg, ncomp, args):
    X, conn = W.unit_cube(kind, *args)
    S = host_system(shape, X, conn, deg, ncomp)
    P = O.Problem(SHAPE_TO_ORACLE[shape], X, conn, deg, ncomp)
    assert S.ndofobj == P.ndofobj
    np.testing.assert_array_equal(S.elem_dofobj(), P.elem_dofobj())
    e1, f1 = S.boundary_faces()
    e2, f2 = P.boundary_faces()
    np.testing.assert_array_equal(e1, e2)
    np.testing.assert_array_equal(f1, f2)
    x1, d1 = S.boundary_points()
    x2, d2 = P.boundary_points()
    # same (dof object, point) pairs; the order within a face may differ
    k1 = sorted(zip(d1.tolist(), np.round(x1, 12).tolist()))
    k2 = sorted(zip(d2.tolist(), np.round(x2, 12).tolist()))
    assert k1 == k2


@pytest.mark.parametrize("name,n", [("c1", 9), ("c2", 4), ("c3", 3)])
def test_numbering_matches_oracle(name, n):
    p = W.config(name, n=n)
    S = System(device=-1)
    S.upload_mesh(p.shape, p.X, p.conn)
    S.create_field(p.fedeg, p.ncomp)
    S.constrain_boundary(p.dirichlet)
    neq = S.number_dofs()
    P, _ = oracle_problem(p, assemble=False)
    assert neq == P.neq
    np.testing.assert_array_equal(S.dof_index(), P.eq_index())


def test_jittered_tets_are_positive():
    p = W.config("c3", n=6)
    X, conn = p.X, p.conn
    a, b, c, d = (X[conn[:, i]] for i in range(4))
    det = np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a)
    assert (det > 0).all()


def _pins():
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fullsize_hashes.json")) as f:
        return json.load(f)


def _h64(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i8").tobytes()).hexdigest()


@pytest.mark.parametrize("deg", [1, 2])
def test_oracle_reproduces_c4_instance_pins(deg):
    """The committed full-size pins are the oracle's own: the c4 instances are
    recomputed here (the c2 / c3 pins take the same code path at 64^3)."""
    pins = _pins()["c4_instances"]
    for side in (8, 131, 256):
        X, conn = W.unit_cube("quad", side, side)
        P = O.Problem(O.QUAD, X, conn, deg, 1)
        x, d = P.boundary_points()
        P.constrain(d, np.zeros(len(d), dtype=np.int32), np.zeros(len(d)))
        P.number()
        rp, ci = P.pattern()
        pin = pins[f"Q{deg}_side{side}"]
        assert (P.neq, len(ci)) == (pin["neq"], pin["nnz"])
        assert _h64(P.elem_dofobj()) == pin["elem_dofobj_sha256"]
        assert _h64(P.eq_index()) == pin["eq_index_sha256"]
        assert _h64(rp) == pin["rowptr_sha256"] and _h64(ci) == pin["colind_sha256"]


@pytest.mark.parametrize("name", ["c2", "c3"])
def test_host_pipeline_matches_full_size_pins(name):
    """The product's host DOF pipeline at the full c2 / c3 sizes: DOF-object ids
    and equation indices against the oracle's pins (the GPU tests check the
    device pipeline and the CSR pattern against the same pins)."""
    p = W.config(name)
    pin = _pins()["configs"][name]
    S = System(device=-1)
    S.upload_mesh(p.shape, p.X, p.conn)
    S.create_field(p.fedeg, p.ncomp)
    S.constrain_boundary(p.dirichlet)
    assert S.number_dofs() == pin["neq"]
    assert S.ndofobj == pin["n_dofobj"]
    assert _h64(S.elem_dofobj()) == pin["elem_dofobj_sha256"]
    assert _h64(S.dof_index()) == pin["eq_index_sha256"]
    S.close()
