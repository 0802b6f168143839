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
