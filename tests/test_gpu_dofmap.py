"""The DOF-object numbering and boundary detection on the GPU (sorts and scans)
against the host pipeline and the reference's golden sparsity files: the ids,
the boundary face order, the support points, the equation numbering and the
CSR pattern must be identical, bit for bit."""
import sys

import numpy as np
import pytest

from insilico_gb300 import _abi as A
from insilico_gb300 import workloads as W
from insilico_gb300.system import System

import oracle as O

sys.path.insert(0, __import__("os").path.join(__import__("os").path.dirname(__file__), "golden"))
from make_fixtures import lines_hash  # noqa: E402

pytestmark = pytest.mark.gpu


def setup(shape, meshes, deg, ncomp, host):
    S = System(device=0)
    S.set_option(A.OPT_HOST_SETUP, 1 if host else 0)
    if len(meshes) == 1:
        S.upload_mesh(shape, *meshes[0])
    else:
        S.upload_batch(shape, meshes)
    S.create_field(deg, ncomp)
    return S


@pytest.mark.parametrize("degree", [2, 3])
def test_device_sparsity_matches_reference_golden(pins, degree):
    X, conn = O.unitcube("quad", 20, 20, round6=True)
    S = setup(A.QUAD, [(X, conn)], degree, 1, host=False)
    ed = S.elem_dofobj()
    n = S.ndofobj
    nf = ed.shape[1]
    key = np.unique(np.repeat(ed, nf, axis=1).ravel() * n + np.tile(ed, (1, nf)).ravel())
    lines = [f"{k // n} {k % n}" for k in key.tolist()]
    p = pins["sparsity"][str(degree)]
    assert len(lines) == p["lines"]
    assert lines_hash(lines) == p["sha256"]
    S.close()


def _permuted(kind, sizes, seed):
    """unit-cube meshes with their nodes renumbered at random, so first-visit
    order and node order differ"""
    rng = np.random.default_rng(seed)
    out = []
    for sz in sizes:
        X, conn = W.unit_cube(kind, *sz)
        perm = rng.permutation(len(X))
        inv = np.argsort(perm)
        out.append((X[perm], inv[conn]))
    return out


CASES = [
    ("quad", A.QUAD, 2, 1, [(6, 4)], False), ("quad", A.QUAD, 3, 1, [(5, 3)], True),
    ("quad", A.QUAD, 2, 2, [(40, 33)], True), ("hex", A.HEX, 2, 1, [(3, 4, 2)], True),
    ("hex", A.HEX, 2, 3, [(9, 8, 7)], False), ("tet", A.TET, 2, 1, [(3, 2, 2)], True),
    ("tet", A.TET, 2, 1, [(14, 12, 13)], False),
    ("quad", A.QUAD, 2, 1, [(4, 4), (3, 5), (7, 2), (30, 41)], True),
    ("tet", A.TET, 2, 1, [(2, 2, 2), (3, 2, 1), (5, 6, 4)], True),
]


@pytest.mark.parametrize("kind,shape,deg,ncomp,sizes,permute", CASES)
def test_device_and_host_setup_agree(kind, shape, deg, ncomp, sizes, permute):
    meshes = _permuted(kind, sizes, 7) if permute else [W.unit_cube(kind, *sz) for sz in sizes]
    Sd = setup(shape, meshes, deg, ncomp, host=False)
    Sh = setup(shape, meshes, deg, ncomp, host=True)
    assert Sd.get_option(A.OPT_HOST_SETUP) == 0 and Sh.get_option(A.OPT_HOST_SETUP) == 1
    assert Sd.ndofobj == Sh.ndofobj
    np.testing.assert_array_equal(Sd.elem_dofobj(), Sh.elem_dofobj())
    for a, b in zip(Sd.boundary_faces(), Sh.boundary_faces()):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(Sd.boundary_points(), Sh.boundary_points()):
        np.testing.assert_array_equal(a, b)
    if len(meshes) > 1:
        for a, b in zip(Sd.batch_info(), Sh.batch_info()):
            np.testing.assert_array_equal(a, b)
    for S in (Sd, Sh):
        S.constrain_boundary(lambda x: (np.ones((len(x), ncomp), bool), 0.0))
    assert Sd.number_dofs() == Sh.number_dofs()
    np.testing.assert_array_equal(Sd.dof_index(), Sh.dof_index())
    if len(meshes) == 1 and Sd.neq > 0:
        Sd.register_pattern()
        Sh.register_pattern()
        for a, b in zip(Sd.csr(values=False)[:2], Sh.csr(values=False)[:2]):
            np.testing.assert_array_equal(a, b)
    Sd.close()
    Sh.close()


def test_device_setup_c3_matches_oracle_numbering():
    """tet10 Poisson workload (jittered cube) through the device path: equation
    numbering and CSR pattern equal to the oracle's"""
    from helpers import oracle_problem
    p = W.config("c3", n=5)
    S = W.setup_system(p)
    assert S.get_option(A.OPT_HOST_SETUP) == 0
    P, (rp, ci, _, _) = oracle_problem(p)
    np.testing.assert_array_equal(S.dof_index(), P.eq_index())
    srp, sci, _ = S.csr(values=False)
    np.testing.assert_array_equal(srp, rp)
    np.testing.assert_array_equal(sci, ci)
    S.close()
