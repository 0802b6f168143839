"""ctypes binding of the C-ABI in include/isl_gpu.h (libisl_gpu.so).

There is no fallback: if the shared library is missing or fails to load, the
import of the GPU path raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

(ISL_OK, ISL_ERR_ARG, ISL_ERR_NOMEM, ISL_ERR_DEGENERATE, ISL_ERR_NOT_CONVERGED, ISL_ERR_TIMEOUT, ISL_ERR_CUDA, ISL_ERR_NAN,
 ISL_ERR_CAPACITY) = range(9)
NOALLOC_MAX_N = 65536  # ISL_NOALLOC_MAX_N
QUAD, TET, HEX = 3, 4, 5
TRI = 2  # tetrahedron faces: isl_quadrature_rule only
KERNEL_LAPLACE, KERNEL_HYPERELASTIC, KERNEL_HEAT_STATIC = 0, 1, 2
MAT_STVENANT, MAT_NEOHOOKE = 0, 1
THERMAL_CONSTANT, THERMAL_FENICS = 0, 1
PREC_FP64, PREC_FP32, PREC_MIXED = 0, 1, 2
SOLVE_CG_FP64, SOLVE_CG_FP32_IR, SOLVE_BICGSTAB = 0, 1, 2
T_ELEMENT, T_GATHER, T_SOLVE, T_SPMV, T_PATTERN, NTIMERS = 0, 1, 2, 3, 4, 8

_STATUS = {
    ISL_ERR_ARG: "invalid argument",
    ISL_ERR_NOMEM: "out of memory",
    ISL_ERR_DEGENERATE: "degenerate element",
    ISL_ERR_NOT_CONVERGED: "not converged",
    ISL_ERR_TIMEOUT: "timeout",
    ISL_ERR_CUDA: "CUDA error",
    ISL_ERR_NAN: "non-finite value",
    ISL_ERR_CAPACITY: "larger than a fixed capacity",
}

EXPORTED = [
    "isl_ctx_create", "isl_ctx_destroy", "isl_last_error", "isl_mesh_upload", "isl_field_create",
    "isl_field_elem_dofobj", "isl_boundary_faces", "isl_boundary_points", "isl_constrain",
    "isl_scale_constraints", "isl_number_dofs", "isl_dof_index", "isl_register_pattern", "isl_set_laplace",
    "isl_set_hyperelastic", "isl_set_body_force_nodal", "isl_set_neumann", "isl_set_neumann_vertex", "isl_quadrature_rule", "isl_set_values", "isl_get_values",
    "isl_assemble", "isl_solve", "isl_get_solution", "isl_get_rhs", "isl_norm", "isl_distribute", "isl_get_csr",
    "isl_sync", "isl_set_timing", "isl_timings", "isl_time_spmv", "isl_mark", "isl_elapsed", "isl_launch_count",
    "isl_set_option", "isl_get_option", "isl_device_memory", "isl_batch_mesh_upload", "isl_batch_info",
    "isl_batch_solve_stats", "isl_time_kernels", "isl_cg_solve_noalloc", "isl_quadrature_points",
    "isl_error_norm", "isl_mesh_read_smf", "isl_mesh_get", "isl_mesh_write_smf", "isl_write_vtk",
    "isl_set_heat_static", "isl_set_history", "isl_push_history", "isl_set_inertia", "isl_set_force_history",
    "isl_batch_norms", "isl_batch_scale_constraints", "isl_batch_set_mask",
    "isl_serve_create", "isl_serve_submit", "isl_serve_poll", "isl_serve_wait", "isl_serve_result", "isl_serve_error",
    "isl_serve_release", "isl_serve_destroy", "isl_serve_counters", "isl_tune_cache", "isl_set_laplace_qp",
    "isl_serve_times",
]
(OPT_BLOCK_SOLVER, OPT_BLOCKED, OPT_NBLOCKS, OPT_NSLOTS, OPT_PERSISTENT, OPT_BARRIER_TEST, OPT_SPMV32_KIND,
 OPT_SCALAR_SLOTS, OPT_HOST_SETUP, OPT_BICGSTAB_KIND, OPT_BATCHED_SOLVE, OPT_DIRECT_BLOCKS, OPT_TUNE_RUNS,
 OPT_ELEM_VARIANT, OPT_FOLD_DIRECTION, OPT_BLOCK_UPDATE, OPT_SHORT_COLUMNS,
 OPT_RELIABLE_DROP, OPT_SHARED_GEOMETRY) = range(19)


class ServeConfig(C.Structure):
    """isl_serve_config"""
    _fields_ = [("max_batch", C.c_int), ("max_batches", C.c_int), ("precision", C.c_int),
                ("reserve_bytes", C.c_int64), ("max_pairs", C.c_int64), ("test_budget_bytes", C.c_int64),
                ("test_fake_us_per_elem", C.c_double), ("batch_window_us", C.c_int64), ("size_ratio", C.c_double),
                ("persistent", C.c_int), ("order", C.c_int)]


class ServeRequest(C.Structure):
    """isl_serve_request"""
    _fields_ = [("shape", C.c_int), ("n_nodes", C.c_int64), ("coords", C.POINTER(C.c_double)), ("n_elem", C.c_int64),
                ("conn", C.POINTER(C.c_int64)), ("ncomp", C.c_int), ("kernel", C.c_int), ("material", C.c_int),
                ("quad_degree", C.c_int), ("coef0", C.POINTER(C.c_double)), ("coef1", C.POINTER(C.c_double)),
                ("body", C.POINTER(C.c_double)), ("n_fixed", C.c_int64), ("fixed_node", C.POINTER(C.c_int64)),
                ("fixed_comp", C.POINTER(C.c_int)), ("fixed_value", C.POINTER(C.c_double)), ("load_steps", C.c_int),
                ("max_newton", C.c_int), ("tolerance", C.c_double), ("lin_tol", C.c_double)]


class ServeStats(C.Structure):
    """isl_serve_stats"""
    _fields_ = [("newton_iters", C.c_int64), ("cg_iters", C.c_int64), ("load_steps_done", C.c_int64),
                ("converged", C.c_int), ("status", C.c_int), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_finish", C.c_double), ("batch_id", C.c_int64), ("batch_size", C.c_int)]


class IslError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_STATUS.get(code, code)}: {msg}")
        self.code = code


_lib = None
_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_I32 = C.POINTER(C.c_int)


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load libisl_gpu.so; raise if it is not there (no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError(f"{path} is missing: run insilico_gb300.build.build() (or __graft_entry__.build())")
        _build.build()
    L = C.CDLL(path)
    i = C.c_int
    L.isl_ctx_create.argtypes = [C.POINTER(_P), i, _P]
    L.isl_ctx_destroy.argtypes = [_P]
    L.isl_last_error.argtypes = [_P]
    L.isl_last_error.restype = C.c_char_p
    L.isl_mesh_upload.argtypes = [_P, i, i, C.c_int64, _D, C.c_int64, _I64]
    L.isl_field_create.argtypes = [_P, i, i, _I64, _I32]
    L.isl_field_elem_dofobj.argtypes = [_P, _I64]
    L.isl_boundary_faces.argtypes = [_P, _I64, _I64, _I32]
    L.isl_boundary_points.argtypes = [_P, _I64, _D, _I64]
    L.isl_constrain.argtypes = [_P, C.c_int64, _I64, _I32, _D]
    L.isl_scale_constraints.argtypes = [_P, C.c_double]
    L.isl_number_dofs.argtypes = [_P, _I64]
    L.isl_dof_index.argtypes = [_P, _I64]
    L.isl_register_pattern.argtypes = [_P, _I64]
    L.isl_set_laplace.argtypes = [_P, _D, i]
    L.isl_set_hyperelastic.argtypes = [_P, i, _D, _D, i]
    L.isl_set_body_force_nodal.argtypes = [_P, _D]
    L.isl_set_neumann.argtypes = [_P, C.c_int64, _I64, _I32, _D, i]
    L.isl_set_neumann_vertex.argtypes = [_P, C.c_int64, _I64, _I32, _D, i]
    L.isl_quadrature_rule.argtypes = [i, i, C.POINTER(C.c_int), _D, _D]
    L.isl_set_values.argtypes = [_P, _D]
    L.isl_get_values.argtypes = [_P, _D]
    L.isl_assemble.argtypes = [_P, i, i, i]
    L.isl_solve.argtypes = [_P, i, C.c_double, C.c_int64, _I64, _D]
    L.isl_get_solution.argtypes = [_P, _D]
    L.isl_get_rhs.argtypes = [_P, _D]
    L.isl_norm.argtypes = [_P, _D]
    L.isl_distribute.argtypes = [_P, i]
    L.isl_quadrature_points.argtypes = [_P, i, _I64, _D]
    L.isl_error_norm.argtypes = [_P, i, i, _D, _D]
    L.isl_mesh_read_smf.argtypes = [_P, C.c_char_p, i]
    L.isl_set_heat_static.argtypes = [_P, i, _D, i]
    L.isl_set_history.argtypes = [_P, i]
    L.isl_push_history.argtypes = [_P]
    L.isl_set_inertia.argtypes = [_P, _D, C.c_double, i, _D]
    L.isl_set_force_history.argtypes = [_P, i, _D]
    L.isl_mesh_get.argtypes = [_P, _I64, _I64, _D, _I64]
    L.isl_mesh_write_smf.argtypes = [_P, C.c_char_p]
    L.isl_write_vtk.argtypes = [_P, C.c_char_p, C.c_char_p, C.c_char_p, i, i, _D]
    L.isl_get_csr.argtypes = [_P, _I64, _I64, _D]
    L.isl_sync.argtypes = [_P]
    L.isl_set_timing.argtypes = [_P, i]
    L.isl_timings.argtypes = [_P, _D, _I64]
    L.isl_time_spmv.argtypes = [_P, i, i, _D]
    L.isl_mark.argtypes = [_P, i]
    L.isl_elapsed.argtypes = [_P, i, i, _D]
    L.isl_launch_count.argtypes = [_P, _I64]
    L.isl_set_option.argtypes = [_P, i, C.c_int64]
    L.isl_get_option.argtypes = [_P, i, _I64]
    L.isl_device_memory.argtypes = [i, _I64, _I64]
    L.isl_batch_mesh_upload.argtypes = [_P, i, i, C.c_int64, _I64, _D, _I64, _I64]
    L.isl_batch_info.argtypes = [_P, _I64, _I64, _I64]
    L.isl_batch_solve_stats.argtypes = [_P, _I64, _D]
    L.isl_time_kernels.argtypes = [_P, i, _D]
    # device pointers are passed as integers (c_void_p)
    L.isl_cg_solve_noalloc.argtypes = [i, _P, i, _P, _P, _P, _P, _P, C.c_double, C.c_int64, _I64, _D]
    L.isl_batch_norms.argtypes = [_P, _D]
    L.isl_batch_scale_constraints.argtypes = [_P, _D]
    L.isl_batch_set_mask.argtypes = [_P, C.POINTER(C.c_uint8)]
    L.isl_serve_create.argtypes = [C.POINTER(_P), i, C.POINTER(ServeConfig)]
    L.isl_serve_submit.argtypes = [_P, C.POINTER(ServeRequest), _I64]
    L.isl_serve_poll.argtypes = [_P, C.c_int64, C.POINTER(C.c_int)]
    L.isl_serve_wait.argtypes = [_P, C.c_int64, C.c_double, C.POINTER(C.c_int)]
    L.isl_serve_result.argtypes = [_P, C.c_int64, _D, C.POINTER(ServeStats)]
    L.isl_serve_error.argtypes = [_P, C.c_int64]
    L.isl_serve_error.restype = C.c_char_p
    L.isl_serve_release.argtypes = [_P, C.c_int64]
    L.isl_serve_destroy.argtypes = [_P]
    L.isl_serve_counters.argtypes = [_P, _I64, _I64]
    L.isl_serve_times.argtypes = [_P, _D, _D, _D, _D, _I64]
    L.isl_tune_cache.argtypes = [C.c_char_p]
    L.isl_set_laplace_qp.argtypes = [_P, _D, i]
    for name in EXPORTED:
        f = getattr(L, name)
        if name not in ("isl_last_error", "isl_serve_error"):
            f.restype = C.c_int
    _lib = L
    return L


def d(a):
    return a.ctypes.data_as(_D)


def i64(a):
    return a.ctypes.data_as(_I64)


def i32(a):
    return a.ctypes.data_as(_I32)


def quadrature_rule(shape: int, degree: int):
    """(weights [n], reference points [n, dim]) of the rule the element
    kernels use for a shape and polynomial degree (isl_quadrature_rule)."""
    import numpy as np
    L = load()
    n = C.c_int()
    st = L.isl_quadrature_rule(shape, degree, C.byref(n), None, None)
    if st != ISL_OK:
        raise IslError(st, f"isl_quadrature_rule: no rule for shape {shape}, degree {degree}")
    dim = 2 if shape in (QUAD, TRI) else 3
    w = np.zeros(n.value)
    x = np.zeros(n.value * dim)
    L.isl_quadrature_rule(shape, degree, C.byref(n), d(w), d(x))
    return w, x.reshape(n.value, dim)
