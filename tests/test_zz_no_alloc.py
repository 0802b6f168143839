"""isl_cg_solve_noalloc (FP64 Jacobi CG on caller-owned device buffers, work
vectors in the library's fixed device scratch array) against the context
solver isl_solve(ISL_SOLVE_CG_FP64) on the same assembled system.

Two calls in a row on the same inputs: both must match the context solver
(relative L2 <= 1e-9, the FP64 CG bar of the parity tests) and each other bit
for bit, so the second call does not depend on what the first left in the
shared scratch array.  The device buffers are made by the test (torch); the
entry point itself allocates nothing: the device's free memory is the same
before and after the second call (the first may still load the library's
device code, which the CUDA runtime does lazily).
"""
import ctypes as C

import numpy as np
import pytest

from insilico_gb300 import _abi as A
from insilico_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-12
REL = 1e-9


def context_solve(name, n):
    S = W.setup_system(W.config(name, n=n))
    try:
        S.assemble(A.PREC_FP64)
        b = S.rhs()
        rp, ci, v = S.csr()
        it, _, _ = S.solve(A.SOLVE_CG_FP64, tol=TOL)
        x = S.solution()
    finally:
        S.close()
    return rp, ci, v, b, x, it


def device_free(L):
    f, t = C.c_int64(), C.c_int64()
    assert L.isl_device_memory(0, C.byref(f), C.byref(t)) == A.ISL_OK
    return f.value


def noalloc_solve(L, torch, dev, x, n):
    it, rel = C.c_int64(), C.c_double()
    stream = torch.cuda.current_stream().cuda_stream
    st = L.isl_cg_solve_noalloc(0, stream, n, dev["rp"].data_ptr(), dev["ci"].data_ptr(), dev["v"].data_ptr(),
                                dev["b"].data_ptr(), x.data_ptr(), TOL, 0, C.byref(it), C.byref(rel))
    return st, x.cpu().numpy(), it.value, rel.value


@pytest.mark.parametrize("name,n", [("c2", 16), ("c1", 120)])
def test_noalloc_cg_matches_context_solver_twice(name, n):
    torch = pytest.importorskip("torch")
    L = A.load()
    rp, ci, v, b, xref, itref = context_solve(name, n)
    neq = len(b)
    assert 0 < neq <= A.NOALLOC_MAX_N
    dev = {
        "rp": torch.from_numpy(rp.astype(np.int32)).to("cuda:0"),
        "ci": torch.from_numpy(ci.astype(np.int32)).to("cuda:0"),
        "v": torch.from_numpy(v).to("cuda:0"),
        "b": torch.from_numpy(b).to("cuda:0"),
    }
    outs = []
    for k in range(2):
        x = torch.full((neq,), float("nan"), dtype=torch.float64, device="cuda:0")
        torch.cuda.synchronize()
        free0 = device_free(L)
        st, x, it, rel = noalloc_solve(L, torch, dev, x, neq)
        if k == 1:
            assert device_free(L) == free0, "the no-allocation solve changed the device's free memory"
        assert st == A.ISL_OK, st
        assert np.all(np.isfinite(x))
        assert rel <= TOL
        assert abs(it - itref) <= 2, (it, itref)
        err = np.linalg.norm(x - xref) / np.linalg.norm(xref)
        assert err <= REL, err
        outs.append(x)
    np.testing.assert_array_equal(outs[0], outs[1])


def test_noalloc_rejects_sizes_beyond_the_scratch_array():
    L = A.load()
    it, rel = C.c_int64(-1), C.c_double(-1.0)
    # rejected on the host before any device work: the pointers are never read
    st = L.isl_cg_solve_noalloc(0, None, A.NOALLOC_MAX_N + 1, 16, 16, 16, 16, 16, TOL, 0, C.byref(it), C.byref(rel))
    assert st == A.ISL_ERR_CAPACITY
    st = L.isl_cg_solve_noalloc(0, None, 0, None, None, None, None, None, TOL, 0, C.byref(it), C.byref(rel))
    assert st == A.ISL_OK and it.value == 0
