"""ORACLE — test infrastructure only.

ctypes wrapper around ``oracle/_build/libisl_oracle.so``, the CPU restatement
of the inSilico assembly + CG path.  Only ``tests/``, ``__graft_entry__.smoke``
and the CPU-baseline leg of ``bench.py`` import this module; the product
package ``insilico_gb300`` never does.

The drivers below re-run the reference's golden applications on the oracle:

* :func:`sparsity_lines` — reference/03-doFHandler/doFHandler.cpp:47-132
* :func:`linear_elastic` — reference/06-elastic/linearElastic.cpp:80-216
* :func:`compressible` — reference/06-elastic/compressible.cpp:104-340
* :func:`mixed_poisson` — reference/05-mixedPoisson/mixedPoisson.cpp:100-230
* :func:`nonlinear_heat` — reference/04-heat/nonlinearHeat.cpp:88-237
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libisl_oracle.so")
_lib = None

# element shapes (oracle/isl_oracle.cpp enum Shape)
LINE, TRI, QUAD, TET, HEX = 1, 2, 3, 4, 5
_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_I32 = C.POINTER(C.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle shared library (make in oracle/)."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "isl_oracle.cpp"))
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.orc_create.restype = _P
        L.orc_create.argtypes = [C.c_int, C.c_int, C.c_int64, _D, C.c_int64, _I64, C.c_int, C.c_int]
        L.orc_destroy.argtypes = [_P]
        L.orc_num_dofobj.restype = C.c_int64
        L.orc_num_dofobj.argtypes = [_P]
        L.orc_nfun.restype = C.c_int
        L.orc_nfun.argtypes = [_P]
        L.orc_elem_dofobj.argtypes = [_P, _I64]
        L.orc_dofobj_sparsity.restype = C.c_int64
        L.orc_dofobj_sparsity.argtypes = [_P, _I64, _I64]
        L.orc_boundary_points.restype = C.c_int64
        L.orc_boundary_points.argtypes = [_P, _D, _I64]
        L.orc_boundary_faces.restype = C.c_int64
        L.orc_boundary_faces.argtypes = [_P, _I64, _I32]
        L.orc_constrain.argtypes = [_P, C.c_int64, _I64, _I32, _D]
        L.orc_scale_constraints.argtypes = [_P, C.c_double]
        L.orc_number.restype = C.c_int64
        L.orc_number.argtypes = [_P]
        L.orc_eq_index.argtypes = [_P, _I64]
        L.orc_set_laplace.argtypes = [_P, _D, C.c_int]
        L.orc_set_laplace_qp.argtypes = [_P, _D, C.c_int]
        L.orc_set_hyperelastic.argtypes = [_P, C.c_int, _D, _D, C.c_int]
        L.orc_set_heat_static.argtypes = [_P, C.c_int, _D, C.c_int]
        L.orc_set_inertia.argtypes = [_P, _D, C.c_double, C.c_int, _D, C.c_int, _D, C.c_int, _D]
        L.orc_quadrature.argtypes = [C.c_int, C.c_int, _D, _D]
        L.orc_quadrature.restype = C.c_int
        L.orc_set_body_nodal.argtypes = [_P, _D]
        L.orc_set_body_cosproduct.argtypes = [_P, _D]
        L.orc_set_neumann.argtypes = [_P, C.c_int, C.c_int64, _I64, _I32, _D, C.c_double, C.c_int]
        L.orc_set_values.argtypes = [_P, _D]
        L.orc_get_values.argtypes = [_P, _D]
        L.orc_assemble.restype = C.c_int64
        L.orc_assemble.argtypes = [_P, C.c_int, C.c_int, C.c_int]
        L.orc_get_csr.argtypes = [_P, _I64, _I64, _D, _D]
        L.orc_build_pattern.restype = C.c_int64
        L.orc_build_pattern.argtypes = [_P]
        L.orc_set_element_range.argtypes = [_P, C.c_int64, C.c_int64]
        L.orc_element_matrices.argtypes = [_P, C.c_int64, C.c_int64, _D]
        L.orc_cg.restype = C.c_int64
        L.orc_cg.argtypes = [C.c_int64, _I64, _I64, _D, _D, C.c_double, C.c_int64, _D, _D, C.c_int]
        L.orc_cg_hist.restype = C.c_int64
        L.orc_cg_hist.argtypes = [C.c_int64, _I64, _I64, _D, _D, C.c_double, C.c_int64, _D, _D, C.c_int, _D]
        L.orc_distribute.argtypes = [_P, _D, C.c_int]
        L.orc_eval_refsol.argtypes = [C.c_int, _D, C.c_int, C.c_int64, _D, _D]
        L.orc_error_norm.restype = C.c_double
        L.orc_error_norm.argtypes = [_P, C.c_int, _D, C.c_int, C.c_int]
        L.orc_unitcube.restype = C.c_int64
        L.orc_unitcube.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _D, _I64, _I64]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_D)


def _i64(a):
    return a.ctypes.data_as(_I64)


def _i32(a):
    return a.ctypes.data_as(_I32)


def unitcube(kind: str, e1: int, e2: int, e3: int = 0, round6: bool = False):
    """Structured unit-cube mesh (tools/meshGeneration/unitCube/unitCube.hpp:180-263).

    kind: 'quad' | 'hex' | 'tet'.  Returns (X [n, dim] float64, conn [E, nv] int64)."""
    k = {"quad": 0, "hex": 1, "tet": 2}[kind]
    dim = 2 if k == 0 else 3
    L = lib()
    ne = C.c_int64(0)
    nn = L.orc_unitcube(k, e1, e2, e3, int(round6), None, None, C.byref(ne))
    X = np.zeros((nn, dim))
    nv = {0: 4, 1: 8, 2: 4}[k]
    conn = np.zeros((ne.value, nv), dtype=np.int64)
    L.orc_unitcube(k, e1, e2, e3, int(round6), _d(X), _i64(conn), C.byref(ne))
    return X, conn


def read_smf_text(text: str):
    """SMF reader semantics (base/io/smf/Reader.hpp:275-307): node and element
    IDs are their order in the file."""
    lines = [l for l in text.splitlines() if l.strip() and not l.startswith("#") and not l.startswith("!")]
    nn, ne = (int(t) for t in lines[0].split()[:2])
    X = np.array([[float(t) for t in l.split()] for l in lines[1:1 + nn]])
    conn = np.array([[int(t) for t in l.split()] for l in lines[1 + nn:1 + nn + ne]], dtype=np.int64)
    return X, conn


class Problem:
    """One mesh + field on the oracle (geometry degree 1)."""

    def __init__(self, shape: int, X: np.ndarray, conn: np.ndarray, fedeg: int, ncomp: int):
        self.L = lib()
        self.shape, self.dim = shape, X.shape[1]
        self.X = np.ascontiguousarray(X, dtype=np.float64)
        self.conn = np.ascontiguousarray(conn, dtype=np.int64)
        self.ncomp = ncomp
        self.h = self.L.orc_create(shape, self.dim, len(X), _d(self.X), len(conn), _i64(self.conn), fedeg, ncomp)
        self.ndofobj = self.L.orc_num_dofobj(self.h)
        self.nfun = self.L.orc_nfun(self.h)
        self.neq = None

    def __del__(self):
        try:
            self.L.orc_destroy(self.h)
        except Exception:
            pass

    def elem_dofobj(self):
        out = np.zeros((len(self.conn), self.nfun), dtype=np.int64)
        self.L.orc_elem_dofobj(self.h, _i64(out))
        return out

    def dofobj_sparsity(self):
        n = self.L.orc_dofobj_sparsity(self.h, None, None)
        r = np.zeros(n, dtype=np.int64)
        c = np.zeros(n, dtype=np.int64)
        self.L.orc_dofobj_sparsity(self.h, _i64(r), _i64(c))
        return r, c

    def boundary_points(self):
        n = self.L.orc_boundary_points(self.h, None, None)
        x = np.zeros((n, self.dim))
        d = np.zeros(n, dtype=np.int64)
        self.L.orc_boundary_points(self.h, _d(x), _i64(d))
        return x, d

    def boundary_faces(self):
        n = self.L.orc_boundary_faces(self.h, None, None)
        e = np.zeros(n, dtype=np.int64)
        f = np.zeros(n, dtype=np.int32)
        self.L.orc_boundary_faces(self.h, _i64(e), _i32(f))
        return e, f

    def constrain(self, dofobj, comp, value):
        dofobj = np.ascontiguousarray(dofobj, dtype=np.int64)
        comp = np.ascontiguousarray(comp, dtype=np.int32)
        value = np.ascontiguousarray(value, dtype=np.float64)
        self.L.orc_constrain(self.h, len(dofobj), _i64(dofobj), _i32(comp), _d(value))

    def scale_constraints(self, f):
        self.L.orc_scale_constraints(self.h, f)

    def number(self):
        self.neq = self.L.orc_number(self.h)
        return self.neq

    def eq_index(self):
        out = np.zeros(self.ndofobj * self.ncomp, dtype=np.int64)
        self.L.orc_eq_index(self.h, _i64(out))
        return out

    def set_laplace(self, kappa, qdeg):
        self._kappa = np.ascontiguousarray(kappa, dtype=np.float64)
        self.L.orc_set_laplace(self.h, _d(self._kappa), qdeg)

    def set_laplace_qp(self, kappa, qdeg):
        """heat::Laplace with the conductivity at every quadrature point, [nelem, nq]."""
        self._kappa = np.ascontiguousarray(kappa, dtype=np.float64)
        self.L.orc_set_laplace_qp(self.h, _d(self._kappa), qdeg)

    def set_hyperelastic(self, material, lam, mu, qdeg):
        self._lam = np.ascontiguousarray(lam, dtype=np.float64)
        self._mu = np.ascontiguousarray(mu, dtype=np.float64)
        self.L.orc_set_hyperelastic(self.h, {"stvenant": 0, "neohooke": 1}[material], _d(self._lam), _d(self._mu), qdeg)

    def set_heat_static(self, material, param, qdeg):
        """heat::Static with mat::thermal::IsotropicConstant ("constant", param =
        conductivity) or FenicsTest ("fenics", param = exponent m), per element."""
        self._thermal = np.ascontiguousarray(param, dtype=np.float64)
        self.L.orc_set_heat_static(self.h, {"constant": 0, "fenics": 1}[material], _d(self._thermal), qdeg)

    def set_inertia(self, rho, mass_w, weights, history, force_weights=()):
        """ReactionTerms (base/time/ReactionTerms.hpp): mass_w * M into the
        matrix, M (sum_s weights[s] x^(s)) into the forces; x^(0) the current
        values, history = [x^(1), x^(2), ...]; force_weights[s-1] weighs the
        residual force at x^(s) (ResidualForceHistory.hpp); rho None turns
        them off."""
        if rho is None:
            self.L.orc_set_inertia(self.h, None, 0.0, 0, None, 0, None, 0, None)
            return
        self._rho = np.ascontiguousarray(rho, dtype=np.float64)
        self._hw = np.ascontiguousarray(weights, dtype=np.float64)
        self._fw = np.ascontiguousarray(force_weights, dtype=np.float64) if len(force_weights) else np.zeros(1)
        self._hist = np.ascontiguousarray(np.array(history, dtype=np.float64).reshape(-1)) if len(history) else np.zeros(1)
        self.L.orc_set_inertia(self.h, _d(self._rho), float(mass_w), len(self._hw), _d(self._hw), len(history),
                               _d(self._hist), len(force_weights), _d(self._fw))

    def set_body_nodal(self, f):
        self._f = np.ascontiguousarray(f, dtype=np.float64)
        self.L.orc_set_body_nodal(self.h, _d(self._f))

    def set_body_cosproduct(self, alpha):
        a = np.zeros(3)
        a[: len(alpha)] = alpha
        self._alpha = a
        self.L.orc_set_body_cosproduct(self.h, _d(self._alpha))

    def set_neumann(self, kind, elem, face, traction=None, value=0.0, sqdeg=2):
        self._ne = np.ascontiguousarray(elem, dtype=np.int64)
        self._nf = np.ascontiguousarray(face, dtype=np.int32)
        self._nt = None if traction is None else np.ascontiguousarray(traction, dtype=np.float64)
        kinds = {"constant": 1, "cosproduct": 2, "pulledsheet": 3}
        self.L.orc_set_neumann(self.h, kinds[kind], len(self._ne), _i64(self._ne), _i32(self._nf),
                               None if self._nt is None else _d(self._nt), value, sqdeg)

    def set_values(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        self.L.orc_set_values(self.h, _d(u))

    def values(self):
        out = np.zeros(self.ndofobj * self.ncomp)
        self.L.orc_get_values(self.h, _d(out))
        return out

    def assemble(self, incremental=False, with_residual=False, nthreads=1):
        nnz = self.L.orc_assemble(self.h, int(incremental), int(with_residual), nthreads)
        rp = np.zeros(self.neq + 1, dtype=np.int64)
        ci = np.zeros(nnz, dtype=np.int64)
        v = np.zeros(nnz)
        b = np.zeros(self.neq)
        self.L.orc_get_csr(self.h, _i64(rp), _i64(ci), _d(v), _d(b))
        return rp, ci, v, b

    def element_range(self, e0=0, e1=-1):
        """Limit later assemblies to elements [e0, e1) (timing samples); e1 < 0: all."""
        self.L.orc_set_element_range(self.h, e0, e1)

    def pattern(self):
        """CSR rowptr / colind of the current numbering (no assembly)."""
        nnz = self.L.orc_build_pattern(self.h)
        rp = np.zeros(self.neq + 1, dtype=np.int64)
        ci = np.zeros(nnz, dtype=np.int64)
        self.L.orc_get_csr(self.h, _i64(rp), _i64(ci), None, None)
        return rp, ci

    def element_matrices(self, e0, ne):
        nloc = self.nfun * self.ncomp
        out = np.zeros((ne, nloc, nloc))
        self.L.orc_element_matrices(self.h, e0, ne, _d(out))
        return out

    def distribute(self, x, add=False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        self.L.orc_distribute(self.h, _d(x), int(add))

    def error_norm(self, kind, params, order, qdeg):
        p = np.ascontiguousarray(params, dtype=np.float64)
        return self.L.orc_error_norm(self.h, kind, _d(p), order, qdeg)


def quadrature(shape: int, degree: int):
    """(weights [n], points [n, dim]) of the oracle's rule for a shape
    (LINE/TRI/QUAD/TET/HEX) and polynomial degree; None without such a rule."""
    L = lib()
    n = L.orc_quadrature(shape, degree, None, None)
    if n < 0:
        return None
    dim = {LINE: 1, TRI: 2, QUAD: 2, TET: 3, HEX: 3}[shape]
    w = np.zeros(n)
    x = np.zeros(n * dim)
    L.orc_quadrature(shape, degree, _d(w), _d(x))
    return w, x.reshape(n, dim)


def cg(rowptr, colind, val, b, tol=2.220446049250313e-16, max_iter=None, nthreads=1, history=False):
    """Eigen-3.2 ConjugateGradient semantics (Jacobi preconditioner, x0 = 0).

    Returns (x, iterations, relative residual); with history=True also the
    array of ||r||^2 / ||b||^2 after every iteration (see iters_to)."""
    n = len(b)
    if max_iter is None:
        max_iter = 2 * n
    rp = np.ascontiguousarray(rowptr, dtype=np.int64)
    ci = np.ascontiguousarray(colind, dtype=np.int64)
    v = np.ascontiguousarray(val, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(n)
    rr = C.c_double(0.0)
    if not history:
        it = lib().orc_cg(n, _i64(rp), _i64(ci), _d(v), _d(bb), tol, max_iter, _d(x), C.byref(rr), nthreads)
        return x, int(it), rr.value
    hist = np.full(max(1, max_iter), np.inf)
    it = lib().orc_cg_hist(n, _i64(rp), _i64(ci), _d(v), _d(bb), tol, max_iter, _d(x), C.byref(rr), nthreads, _d(hist))
    return x, int(it), rr.value, hist[:min(len(hist), int(it) + 1)]


def iters_to(history, tol):
    """Iterations Eigen's CG takes to ||r|| < tol ||b||, from a cg(...,
    history=True) residual history of a solve to a tighter tolerance."""
    hit = np.nonzero(np.asarray(history) < tol * tol)[0]
    return int(hit[0]) if len(hit) else None


def eval_refsol(kind, params, x):
    p = np.ascontiguousarray(params, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    dim = x.shape[1]
    nc = dim if kind == 0 else 1
    out = np.zeros((len(x), nc))
    lib().orc_eval_refsol(kind, _d(p), dim, len(x), _d(x), _d(out))
    return out


# ---------------------------------------------------------------------------
# Golden drivers
# ---------------------------------------------------------------------------
def sparsity_lines(degree: int, X, conn):
    """DOF-object sparsity of a Q<degree> field on a quad mesh, in the text
    format of reference/03-doFHandler/doFHandler.cpp:95-104 (data lines only)."""
    P = Problem(QUAD, X, conn, degree, 1)
    r, c = P.dofobj_sparsity()
    return [f"{a} {b}" for a, b in zip(r.tolist(), c.tolist())]


def lame(E, nu):
    """mat/Lame.hpp:28-49"""
    return E * nu / (1.0 + nu) / (1.0 - 2.0 * nu), E / 2.0 / (1.0 + nu)


def linear_elastic(dim: int, X, conn, E=1000.0, nu=0.25):
    """L2 error of reference/06-elastic/linearElastic.cpp on the given mesh."""
    shape = QUAD if dim == 2 else HEX
    lam, mu = lame(E, nu)
    P = Problem(shape, X, conn, 1, dim)
    prm = np.zeros(8)
    prm[0], prm[1] = lam, mu
    prm[2:2 + dim] = -0.1
    prm[5 + 1] = 1.0  # dir = (0, 1, 0)
    x, d = P.boundary_points()
    U = eval_refsol(0, prm, x)
    P.constrain(np.repeat(d, dim), np.tile(np.arange(dim), len(d)), U.reshape(-1))
    P.number()
    ne = len(conn)
    P.set_hyperelastic("stvenant", np.full(ne, lam), np.full(ne, mu), 3)
    rp, ci, v, b = P.assemble(incremental=True)
    xs, it, rr = cg(rp, ci, v, b)
    P.distribute(xs)
    return P.error_norm(0, prm, 0, 3)


def compressible(X, conn, E=1000.0, nu=0.3, max_iter=30, load_steps=5, pull=3.0, traction=1000.0,
                 disp_controlled=True, tolerance=1e-12, return_values=False):
    """Newton history of reference/06-elastic/compressible.cpp (2-D, Q2,
    NeoHookeanCompressible, PulledSheet boundary conditions); with
    return_values, also the final DOF values [ndofobj * 2]."""
    lam, mu = lame(E, nu)
    P = Problem(QUAD, X, conn, 2, 2)
    first_pull = pull / load_steps
    x, d = P.boundary_points()
    dofs, comps, vals = [], [], []
    for xi, di in zip(x, d):
        # reference/06-elastic/PulledSheet.hpp:35-58 (constrainValue keeps the latest value)
        if abs(xi[0]) < 1e-6:
            for c in range(2):
                dofs.append(di); comps.append(c); vals.append(0.0)
        if abs(xi[0] - 1.0) < 1e-6 and disp_controlled:
            dofs.append(di); comps.append(0); vals.append(first_pull)
    P.constrain(dofs, comps, vals)
    neq = P.number()
    ne = len(conn)
    P.set_hyperelastic("neohooke", np.full(ne, lam), np.full(ne, mu), 3)
    if not disp_controlled:
        be, bf = P.boundary_faces()
    rows = []
    for step in range(load_steps):
        factor = float(step + 1) if step == 0 else (step + 1) / step
        P.scale_constraints(factor)
        it = 0
        while it < max_iter:
            if not disp_controlled:
                P.set_neumann("pulledsheet", be, bf, None, traction * (step + 1) / load_steps, 3)
            rp, ci, v, b = P.assemble(incremental=True, with_residual=True)
            conv1 = np.linalg.norm(b) / neq
            if conv1 < tolerance * E:
                rows.append((step, it, conv1, None))
                break
            xs, _, _ = cg(rp, ci, v, b)
            P.distribute(xs, add=True)
            conv2 = np.linalg.norm(xs) / neq
            rows.append((step, it, conv1, conv2))
            it += 1
            if conv2 < tolerance:
                break
    if return_values:
        return neq, rows, P.values()
    return neq, rows


def nonlinear_heat(X, conn, m=3.0, max_iter=10, tolerance=1e-8, qdeg=5):
    """reference/04-heat/nonlinearHeat.cpp: Q2 heat::Static with FenicsTest
    conductivity (1 + u)^m, u = 0 at x = 0 and u = 1 at x = 1, Newton with a
    direct solve of the non-symmetric tangent (SuperLU there, scipy's SuperLU
    here).  Returns (ndofs, [(iter, |R|, |x| or None)], L2 error)."""
    from scipy.sparse import csr_matrix
    from scipy.sparse.linalg import splu
    P = Problem(QUAD, X, conn, 2, 1)
    x, d = P.boundary_points()
    left = np.abs(x[:, 0]) < 1e-5
    right = np.abs(x[:, 0] - 1.0) < 1e-5
    sel = left | right
    P.constrain(d[sel], np.zeros(sel.sum()), np.where(right[sel], 1.0, 0.0))
    n = P.number()
    P.set_heat_static("fenics", np.full(len(conn), m), qdeg)
    rows = []
    it = 0
    while it < max_iter:
        rp, ci, v, b = P.assemble(incremental=True, with_residual=True)
        rn = np.linalg.norm(b) / n
        if rn < tolerance:
            rows.append((it, rn, None))
            break
        xs = splu(csr_matrix((v, ci, rp), shape=(n, n)).tocsc()).solve(b)
        xn = np.linalg.norm(xs) / n
        if xn < tolerance:
            rows.append((it, rn, xn))
            break
        rows.append((it, rn, xn))
        P.distribute(xs, add=True)
        it += 1
    prm = np.array([m])
    return n, rows, P.error_norm(2, prm, 0, qdeg), P


def mixed_poisson(X, conn, alpha=(3.0, 5.0, 4.0)):
    """reference/05-mixedPoisson/mixedPoisson.cpp: Q2 Poisson with Dirichlet on
    x_d = 0, co-normal Neumann data elsewhere; returns (ndofs, L2, H1)."""
    P = Problem(QUAD, X, conn, 2, 1)
    prm = np.zeros(3)
    prm[:2] = alpha[:2]
    x, d = P.boundary_points()
    u = eval_refsol(1, prm, x)[:, 0]
    on = (np.abs(x) < 1e-5).any(axis=1)
    P.constrain(d[on], np.zeros(on.sum()), u[on])
    n = P.number()
    P.set_body_cosproduct(prm[:2])
    be, bf = P.boundary_faces()
    P.set_neumann("cosproduct", be, bf, None, 0.0, 3)
    P.set_laplace(np.ones(len(conn)), 3)
    rp, ci, v, b = P.assemble(incremental=False)
    xs, _, _ = cg(rp, ci, v, b)
    P.distribute(xs)
    return n, P.error_norm(1, prm, 0, 3), P.error_norm(1, prm, 1, 3)
