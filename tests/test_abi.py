"""The C-ABI library builds, loads without a GPU and exports every entry point
declared in include/isl_gpu.h; host-only contexts run the DOF pipeline."""
import os
import re

import numpy as np

from insilico_gb300 import _abi as A
from insilico_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    with open(os.path.join(ROOT, "include", "isl_gpu.h")) as f:
        txt = f.read()
    return sorted(set(re.findall(r"^(?:int|const char\*)\s+(isl_\w+)\s*\(", txt, re.M)))


def test_library_builds_and_exports_all_symbols():
    B.build()
    L = A.load()
    syms = declared_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(L, s), s
    assert sorted(A.EXPORTED) == syms


def test_every_declaration_cites_the_reference():
    with open(os.path.join(ROOT, "include", "isl_gpu.h")) as f:
        txt = f.read()
    # each block of declarations is preceded by a comment; the file cites reference files
    assert txt.count(".hpp:") >= 15


def test_host_only_context_rejects_device_work():
    from insilico_gb300.system import System
    S = System(device=-1)
    X = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], dtype=float)
    S.upload_mesh(A.QUAD, X, np.array([[0, 1, 2, 3]]))
    S.create_field(1, 1)
    S.number_dofs()
    try:
        S.register_pattern()
        raise AssertionError("expected failure")
    except A.IslError as e:
        assert e.code == A.ISL_ERR_ARG


def test_host_only_argument_checks():
    """argument checks of the newer entry points on a host-only context: the
    time-integration and post-processing calls that need a device refuse with
    ISL_ERR_ARG, and option values out of range, inertia weights beyond the
    stored history and Neumann faces out of range are refused"""
    import pytest
    from insilico_gb300.system import System
    S = System(device=-1)
    X = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], dtype=float)
    S.upload_mesh(A.QUAD, X, np.array([[0, 1, 2, 3]]))
    S.create_field(1, 1)
    for call in (lambda: S.set_history(1), lambda: S.quadrature_points(2),
                 lambda: S.error_norm(0, 2, np.zeros(4)), lambda: S.set_force_history([1.0]),
                 lambda: S.set_option(A.OPT_BICGSTAB_KIND, 104), lambda: S.set_option(A.OPT_SPMV32_KIND, 3),
                 lambda: S.set_option(A.OPT_PERSISTENT, 7),
                 lambda: S.set_inertia(np.ones(1), 1.0, [1.0, -1.0]),
                 lambda: S.set_neumann_vertex([0], [4], np.zeros((1, 2, 1))),
                 lambda: S.set_neumann_vertex([1], [0], np.zeros((1, 2, 1)))):
        with pytest.raises(A.IslError) as ei:
            call()
        assert ei.value.code == A.ISL_ERR_ARG
    # host-only values round trip (the I/O path reads them)
    S.set_values(np.arange(4.0))
    assert np.array_equal(S.values(), np.arange(4.0))
    S.set_option(A.OPT_HOST_SETUP, 1)
    assert S.get_option(A.OPT_HOST_SETUP) == 1
