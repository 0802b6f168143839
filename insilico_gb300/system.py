"""Host-side mirror of the reference's assembly/solver call surface over the C-ABI.

The reference drives one boundary value problem as (reference/06-elastic/
linearElastic.cpp:80-216, heat/PoissonDriver.hpp:153-210,
solid/CompressibleDriver.hpp:156-214):

    dof::generate -> MeshBoundary::create -> constrainBoundary ->
    numberDoFsConsecutively -> Eigen3 solver(N) -> registerFields ->
    stiffnessMatrixComputation / computeResidualForces / bodyForceComputation /
    neumannForceComputation -> finishAssembly -> cgSolve -> setDoFsFromSolver

:class:`System` exposes the same steps, each a call into libisl_gpu.so; the
device keeps mesh, pattern, matrix and iterate resident between calls.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, Optional

import numpy as np

from . import _abi as A
from ._abi import IslError


class System:
    """One mesh + field + assembled system on one GPU (an isl_ctx)."""

    def __init__(self, device: int = 0, stream: Optional[int] = None):
        self.L = A.load()
        h = C.c_void_p()
        st = self.L.isl_ctx_create(C.byref(h), device, C.c_void_p(stream) if stream else None)
        if st != A.ISL_OK:
            raise IslError(st, "isl_ctx_create failed")
        self.h = h
        self.neq = 0
        self.nnz = 0

    def close(self):
        if getattr(self, "h", None):
            self.L.isl_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, st, what=""):
        if st != A.ISL_OK:
            msg = self.L.isl_last_error(self.h)
            raise IslError(st, f"{what}: {msg.decode() if msg else ''}")

    # -- mesh / field / DOFs ------------------------------------------------
    def upload_mesh(self, shape: int, X: np.ndarray, conn: np.ndarray):
        self.X = np.ascontiguousarray(X, dtype=np.float64)
        self.conn = np.ascontiguousarray(conn, dtype=np.int64)
        self.shape, self.dim = shape, self.X.shape[1]
        self.nnodes, self.nelem = len(self.X), len(self.conn)
        self._chk(self.L.isl_mesh_upload(self.h, shape, self.dim, self.nnodes, A.d(self.X), self.nelem, A.i64(self.conn)),
                  "isl_mesh_upload")

    def create_field(self, fe_degree: int, ncomp: int):
        n = C.c_int64()
        nf = C.c_int()
        self._chk(self.L.isl_field_create(self.h, fe_degree, ncomp, C.byref(n), C.byref(nf)), "isl_field_create")
        self.fedeg, self.ncomp, self.ndofobj, self.nfun = fe_degree, ncomp, n.value, nf.value
        return self.ndofobj

    def elem_dofobj(self):
        out = np.zeros((self.nelem, self.nfun), dtype=np.int64)
        self._chk(self.L.isl_field_elem_dofobj(self.h, A.i64(out)))
        return out

    def boundary_faces(self):
        n = C.c_int64()
        self._chk(self.L.isl_boundary_faces(self.h, C.byref(n), None, None))
        e = np.zeros(n.value, dtype=np.int64)
        f = np.zeros(n.value, dtype=np.int32)
        self._chk(self.L.isl_boundary_faces(self.h, C.byref(n), A.i64(e), A.i32(f)))
        return e, f

    def boundary_points(self):
        n = C.c_int64()
        self._chk(self.L.isl_boundary_points(self.h, C.byref(n), None, None))
        x = np.zeros((n.value, self.dim))
        dof = np.zeros(n.value, dtype=np.int64)
        self._chk(self.L.isl_boundary_points(self.h, C.byref(n), A.d(x), A.i64(dof)))
        return x, dof

    def constrain(self, dofobj, comp, value):
        dofobj = np.ascontiguousarray(dofobj, dtype=np.int64)
        comp = np.ascontiguousarray(comp, dtype=np.int32)
        value = np.ascontiguousarray(value, dtype=np.float64)
        self._chk(self.L.isl_constrain(self.h, len(dofobj), A.i64(dofobj), A.i32(comp), A.d(value)), "isl_constrain")

    def constrain_boundary(self, fun: Callable[[np.ndarray], tuple]):
        """constrainBoundary: fun(x [n,dim]) -> (mask [n, ncomp] bool, values [n, ncomp])."""
        x, dof = self.boundary_points()
        mask, vals = fun(x)
        mask = np.asarray(mask, dtype=bool).reshape(len(x), self.ncomp)
        vals = np.broadcast_to(np.asarray(vals, dtype=np.float64), mask.shape)
        rows, comps = np.nonzero(mask)
        self.constrain(dof[rows], comps, vals[rows, comps])

    def scale_constraints(self, factor: float):
        self._chk(self.L.isl_scale_constraints(self.h, factor))

    def number_dofs(self):
        n = C.c_int64()
        self._chk(self.L.isl_number_dofs(self.h, C.byref(n)), "isl_number_dofs")
        self.neq = n.value
        return self.neq

    def dof_index(self):
        out = np.zeros(self.ndofobj * self.ncomp, dtype=np.int64)
        self._chk(self.L.isl_dof_index(self.h, A.i64(out)))
        return out

    def register_pattern(self):
        n = C.c_int64()
        self._chk(self.L.isl_register_pattern(self.h, C.byref(n)), "isl_register_pattern")
        self.nnz = n.value
        return self.nnz

    # -- kernels / forces ----------------------------------------------------
    def set_laplace(self, kappa, quad_degree: int):
        self._kappa = np.ascontiguousarray(kappa, dtype=np.float64)
        self._chk(self.L.isl_set_laplace(self.h, A.d(self._kappa), quad_degree), "isl_set_laplace")

    def set_laplace_qp(self, kappa, quad_degree: int):
        """Conductivity at every quadrature point, [nelem, nq] (isl_set_laplace_qp)."""
        self._kqp = np.ascontiguousarray(kappa, dtype=np.float64)
        self._chk(self.L.isl_set_laplace_qp(self.h, A.d(self._kqp), quad_degree), "isl_set_laplace_qp")

    def set_heat_static(self, material: str, param, quad_degree: int):
        """heat::Static with mat::thermal IsotropicConstant ("constant", param =
        conductivity) or FenicsTest ("fenics", param = m), per element."""
        m = {"constant": A.THERMAL_CONSTANT, "fenics": A.THERMAL_FENICS}[material]
        self._thermal = np.ascontiguousarray(param, dtype=np.float64)
        self._chk(self.L.isl_set_heat_static(self.h, m, A.d(self._thermal), quad_degree), "isl_set_heat_static")

    # -- time integration (base/time/ReactionTerms.hpp) -------------------------
    def set_history(self, nhist: int):
        self._chk(self.L.isl_set_history(self.h, nhist), "isl_set_history")

    def push_history(self):
        self._chk(self.L.isl_push_history(self.h), "isl_push_history")

    def set_inertia(self, density, lhs_weight: float, weights):
        """computeInertiaTerms: lhs_weight * M into the matrix, M (sum_s w_s x^(s))
        into the right-hand side; density None turns them off."""
        if density is None:
            self._chk(self.L.isl_set_inertia(self.h, None, 0.0, 0, None), "isl_set_inertia")
            return
        self._rho = np.ascontiguousarray(density, dtype=np.float64)
        self._hw = np.ascontiguousarray(weights, dtype=np.float64)
        self._chk(self.L.isl_set_inertia(self.h, A.d(self._rho), float(lhs_weight), len(self._hw), A.d(self._hw)),
                  "isl_set_inertia")

    def set_force_history(self, weights):
        """computeResidualForceHistory: -sum_s w[s-1] F(x^(s)) into the forces."""
        self._fw = np.ascontiguousarray(weights, dtype=np.float64) if len(weights) else np.zeros(1)
        self._chk(self.L.isl_set_force_history(self.h, len(weights), A.d(self._fw)), "isl_set_force_history")

    def set_hyperelastic(self, material: str, lam, mu, quad_degree: int):
        m = {"stvenant": A.MAT_STVENANT, "neohooke": A.MAT_NEOHOOKE}[material]
        self._lam = np.ascontiguousarray(lam, dtype=np.float64)
        self._mu = np.ascontiguousarray(mu, dtype=np.float64)
        self._chk(self.L.isl_set_hyperelastic(self.h, m, A.d(self._lam), A.d(self._mu), quad_degree), "isl_set_hyperelastic")

    def set_body_force_nodal(self, f):
        if f is None:
            self._chk(self.L.isl_set_body_force_nodal(self.h, None))
            return
        self._f = np.ascontiguousarray(f, dtype=np.float64)
        self._chk(self.L.isl_set_body_force_nodal(self.h, A.d(self._f)), "isl_set_body_force_nodal")

    def set_neumann(self, elem, face, traction, squad_degree: int = 2):
        e = np.ascontiguousarray(elem, dtype=np.int64)
        f = np.ascontiguousarray(face, dtype=np.int32)
        t = np.ascontiguousarray(np.broadcast_to(traction, (len(e), self.ncomp)), dtype=np.float64)
        self._chk(self.L.isl_set_neumann(self.h, len(e), A.i64(e), A.i32(f), A.d(t), squad_degree), "isl_set_neumann")

    def set_neumann_vertex(self, elem, face, traction, squad_degree: int = 2):
        """traction per face vertex [n, nfv, ncomp], interpolated along each face"""
        e = np.ascontiguousarray(elem, dtype=np.int64)
        f = np.ascontiguousarray(face, dtype=np.int32)
        nfv = 2 if self.shape == A.QUAD else 4
        t = np.ascontiguousarray(np.broadcast_to(traction, (len(e), nfv, self.ncomp)), dtype=np.float64)
        self._chk(self.L.isl_set_neumann_vertex(self.h, len(e), A.i64(e), A.i32(f), A.d(t), squad_degree),
                  "isl_set_neumann_vertex")

    def set_values(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        self._chk(self.L.isl_set_values(self.h, A.d(u)))

    def values(self):
        out = np.zeros(self.ndofobj * self.ncomp)
        self._chk(self.L.isl_get_values(self.h, A.d(out)))
        return out

    # -- assembly / solve ------------------------------------------------------
    def assemble(self, precision: int = A.PREC_FP64, incremental: bool = True, with_residual: bool = False):
        self._chk(self.L.isl_assemble(self.h, precision, int(incremental), int(with_residual)), "isl_assemble")

    def solve(self, method: int = A.SOLVE_CG_FP64, tol: float = 1e-10, max_iter: int = 0, check: bool = True):
        it = C.c_int64()
        rr = C.c_double()
        st = self.L.isl_solve(self.h, method, tol, max_iter, C.byref(it), C.byref(rr))
        if check:
            self._chk(st, "isl_solve")
        return it.value, rr.value, st

    def solution(self):
        x = np.zeros(self.neq)
        self._chk(self.L.isl_get_solution(self.h, A.d(x)))
        return x

    def rhs(self):
        b = np.zeros(self.neq)
        self._chk(self.L.isl_get_rhs(self.h, A.d(b)))
        return b

    def norm(self):
        v = C.c_double()
        self._chk(self.L.isl_norm(self.h, C.byref(v)))
        return v.value

    def batch_norms(self):
        """||v_k|| / N_k of every instance (isl_batch_norms)."""
        n = C.c_int64()
        self._chk(self.L.isl_batch_info(self.h, C.byref(n), None, None))
        out = np.zeros(n.value)
        self._chk(self.L.isl_batch_norms(self.h, A.d(out)), "isl_batch_norms")
        return out

    def batch_scale_constraints(self, factors):
        f = np.ascontiguousarray(factors, dtype=np.float64)
        self._chk(self.L.isl_batch_scale_constraints(self.h, A.d(f)), "isl_batch_scale_constraints")

    def batch_set_mask(self, keep):
        if keep is None:
            self._chk(self.L.isl_batch_set_mask(self.h, None), "isl_batch_set_mask")
            return
        m = np.ascontiguousarray(np.asarray(keep, dtype=bool).astype(np.uint8))
        self._chk(self.L.isl_batch_set_mask(self.h, m.ctypes.data_as(C.POINTER(C.c_uint8))), "isl_batch_set_mask")

    def distribute(self, add: bool = False):
        self._chk(self.L.isl_distribute(self.h, int(add)), "isl_distribute")

    # -- mesh / field I/O (base/io/smf, base/io/vtk) ---------------------------
    def read_smf(self, path: str, shape: int):
        """smf::readMesh into the context (replaces upload_mesh)."""
        self._chk(self.L.isl_mesh_read_smf(self.h, str(path).encode(), shape), "isl_mesh_read_smf")
        nn, ne = C.c_int64(), C.c_int64()
        self._chk(self.L.isl_mesh_get(self.h, C.byref(nn), C.byref(ne), None, None), "isl_mesh_get")
        dim = 2 if shape == A.QUAD else 3
        X = np.zeros((nn.value, dim))
        conn = np.zeros((ne.value, 8 if shape == A.HEX else 4), dtype=np.int64)
        self._chk(self.L.isl_mesh_get(self.h, None, None, A.d(X), A.i64(conn)), "isl_mesh_get")
        self.X, self.conn, self.shape, self.dim = X, conn, shape, dim
        return X, conn

    def write_smf(self, path: str):
        self._chk(self.L.isl_mesh_write_smf(self.h, str(path).encode()), "isl_mesh_write_smf")

    def write_vtk(self, path: str, point_name=None, cell_name=None, cell_values=None):
        """LegacyWriter: grid, the field's values at the nodes (point_name), and
        per-cell data: [ncells] plain scalars or [ncells, r, c] matrices."""
        rows = cols = 0
        cv = None
        if cell_name is not None:
            cv = np.ascontiguousarray(cell_values, dtype=np.float64)
            if cv.ndim == 3:
                rows, cols = cv.shape[1], cv.shape[2]
        self._chk(self.L.isl_write_vtk(self.h, str(path).encode(), point_name.encode() if point_name else None,
                                       cell_name.encode() if cell_name else None, rows, cols,
                                       A.d(cv) if cv is not None else None), "isl_write_vtk")

    # -- post-processing (base/post/ErrorNorm.hpp) -----------------------------
    def quadrature_points(self, quad_degree: int) -> np.ndarray:
        """Physical coordinates of the quadrature points, [nelem * nq, dim]."""
        n = C.c_int64()
        self._chk(self.L.isl_quadrature_points(self.h, quad_degree, C.byref(n), None), "isl_quadrature_points")
        x = np.zeros((n.value, self.dim))
        self._chk(self.L.isl_quadrature_points(self.h, quad_degree, C.byref(n), A.d(x)), "isl_quadrature_points")
        return x

    def error_norm(self, order: int, quad_degree: int, ref) -> float:
        """errorComputation<order> against ref tabulated at quadrature_points():
        order 0 [npoints, ncomp] values, order 1 [npoints, ncomp, dim] gradients."""
        r = np.ascontiguousarray(ref, dtype=np.float64)
        v = C.c_double()
        self._chk(self.L.isl_error_norm(self.h, order, quad_degree, A.d(r), C.byref(v)), "isl_error_norm")
        return v.value

    def csr(self, values: bool = True):
        rp = np.zeros(self.neq + 1, dtype=np.int64)
        ci = np.zeros(self.nnz, dtype=np.int64)
        v = np.zeros(self.nnz) if values else None
        self._chk(self.L.isl_get_csr(self.h, A.i64(rp), A.i64(ci), A.d(v) if values else None), "isl_get_csr")
        return rp, ci, v

    def sync(self):
        self._chk(self.L.isl_sync(self.h))

    def set_timing(self, on: bool):
        self._chk(self.L.isl_set_timing(self.h, int(on)))

    def timings(self):
        ms = np.zeros(A.NTIMERS)
        cnt = np.zeros(A.NTIMERS, dtype=np.int64)
        self._chk(self.L.isl_timings(self.h, A.d(ms), A.i64(cnt)))
        return ms, cnt

    def time_spmv(self, precision: int, nrep: int = 20) -> float:
        v = C.c_double()
        self._chk(self.L.isl_time_spmv(self.h, precision, nrep, C.byref(v)), "isl_time_spmv")
        return v.value

    def mark(self, slot: int):
        self._chk(self.L.isl_mark(self.h, slot))

    def elapsed_ms(self, a: int, b: int) -> float:
        v = C.c_double()
        self._chk(self.L.isl_elapsed(self.h, a, b, C.byref(v)))
        return v.value

    def launch_count(self) -> int:
        v = C.c_int64()
        self._chk(self.L.isl_launch_count(self.h, C.byref(v)))
        return v.value

    def set_option(self, key: int, value: int):
        self._chk(self.L.isl_set_option(self.h, key, value), "isl_set_option")

    def get_option(self, key: int) -> int:
        v = C.c_int64()
        self._chk(self.L.isl_get_option(self.h, key, C.byref(v)), "isl_get_option")
        return v.value

    # -- batches of independent meshes -----------------------------------------
    def upload_batch(self, shape: int, meshes):
        """meshes: list of (X [n_i, dim], conn [E_i, nv] with local node ids)."""
        node_off = np.zeros(len(meshes) + 1, dtype=np.int64)
        elem_off = np.zeros(len(meshes) + 1, dtype=np.int64)
        for k, (X, conn) in enumerate(meshes):
            node_off[k + 1] = node_off[k] + len(X)
            elem_off[k + 1] = elem_off[k] + len(conn)
        self.X = np.ascontiguousarray(np.concatenate([m[0] for m in meshes]), dtype=np.float64)
        self.conn = np.ascontiguousarray(np.concatenate([m[1] + node_off[k] for k, m in enumerate(meshes)]), dtype=np.int64)
        self.shape, self.dim = shape, self.X.shape[1]
        self.nnodes, self.nelem = len(self.X), len(self.conn)
        self.node_off, self.elem_off = node_off, elem_off
        self._chk(self.L.isl_batch_mesh_upload(self.h, shape, self.dim, len(meshes), A.i64(node_off), A.d(self.X),
                                               A.i64(elem_off), A.i64(self.conn)), "isl_batch_mesh_upload")

    def batch_info(self):
        n = C.c_int64()
        self._chk(self.L.isl_batch_info(self.h, C.byref(n), None, None))
        eq = np.zeros(n.value + 1, dtype=np.int64)
        do = np.zeros(n.value + 1, dtype=np.int64)
        self._chk(self.L.isl_batch_info(self.h, C.byref(n), A.i64(eq) if self.neq else None, A.i64(do)))
        return eq, do

    def batch_stats(self):
        n = C.c_int64()
        self._chk(self.L.isl_batch_info(self.h, C.byref(n), None, None))
        it = np.zeros(n.value, dtype=np.int64)
        rr = np.zeros(n.value)
        self._chk(self.L.isl_batch_solve_stats(self.h, A.i64(it), A.d(rr)))
        return it, rr

    def time_kernels(self, nrep: int = 20):
        ms = np.zeros(8)
        self._chk(self.L.isl_time_kernels(self.h, nrep, A.d(ms)), "isl_time_kernels")
        keys = ["block_spmv32", "update_b3", "dir_b3", "spmv64", "update64", "dir64", "residual64", "block_kind"]
        return dict(zip(keys, ms.tolist()))
