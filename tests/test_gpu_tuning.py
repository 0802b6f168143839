"""The tuning cache (isl_tune_cache): the first context of a problem class
times the candidates of its autotunes (element kernel launch shape, FP32 and
FP64 SpMV formats) and records the choices; a second context, and a fresh
load of the cache file (as a new process would read it), take the same
variants without timing anything."""
import ctypes as C

import numpy as np
import pytest

from insilico_gb300 import _abi as A
from insilico_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def run_once():
    p = W.config("c1", n=300)  # 90,000 Q1 elements, 89,401 equations: large enough to tune, above the one-cluster solve
    S = W.setup_system(p)
    S.assemble(A.PREC_MIXED)
    S.solve(A.SOLVE_CG_FP32_IR, tol=1e-10)
    S.assemble(A.PREC_FP64)
    S.solve(A.SOLVE_CG_FP64, tol=1e-10)
    out = (S.get_option(A.OPT_TUNE_RUNS), S.get_option(A.OPT_ELEM_VARIANT), S.get_option(A.OPT_SPMV32_KIND),
           S.solution())
    S.close()
    return out


def test_second_run_takes_the_cached_variants(tmp_path):
    L = A.load()
    path = tmp_path / "tune.txt"
    assert L.isl_tune_cache(str(path).encode()) == A.ISL_OK
    try:
        runs1, elem1, spmv1, x1 = run_once()
        assert runs1 >= 2 and elem1 in (32, 64, 128) and spmv1 > 0
        lines = path.read_text().split("\n")
        assert any(l.startswith("elem_laplace") for l in lines) and any(l.startswith("spmv32") for l in lines)
        runs2, elem2, spmv2, x2 = run_once()
        assert runs2 == 0 and (elem2, spmv2) == (elem1, spmv1)
        np.testing.assert_array_equal(x1, x2)
        # a new process reads the file
        assert L.isl_tune_cache(str(path).encode()) == A.ISL_OK
        runs3, elem3, spmv3, _ = run_once()
        assert runs3 == 0 and (elem3, spmv3) == (elem1, spmv1)
    finally:
        L.isl_tune_cache(None)
