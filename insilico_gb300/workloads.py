"""Seeded synthetic workloads with the shapes of the benchmark configurations.

Meshes follow the reference's unit-cube generator connectivity
(tools/meshGeneration/unitCube/unitCube.hpp:85-263): nodes numbered with the
first coordinate fastest, element corners in hierarchic order, hexahedra split
into six tetrahedra by base/cut/DecomposeHyperCube.hpp:81-90.  Random fields
come from a counter-based Philox generator, one stream per field, seeded by
one 64-bit value per configuration.

Configurations (sizes can be scaled down for tests with ``n=``):
  c1  2-D Poisson (heat::Laplace), Q1 quads 64x64, kappa = exp(N(0, 0.5)) per
      element, nodal source U[0,1], homogeneous Dirichlet on all edges, 2x2 Gauss
  c2  3-D linear elasticity (HyperElastic at u = 0), hex8 64^3, E log-uniform
      [1e3, 1e5], nu U[0.2, 0.45] per element, x = 0 clamped, traction
      (1, 0, 0) on x = 1, 2x2x2 Gauss
  c3  3-D Poisson, tet10 on 64^3 cubes split into 6 tets, interior nodes
      jittered by U[-0.2h, 0.2h], kappa lognormal (sigma = 1), nodal source
      U[0,1], Dirichlet on all faces, 4-point Gauss
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np

from . import _abi as A

SEED_BASE = 0x15111C0

HEX_FACES = np.array([[0, 3, 2, 1], [4, 5, 6, 7], [0, 1, 5, 4], [1, 2, 6, 5], [2, 3, 7, 6], [3, 0, 4, 7]])
QUAD_EDGES = np.array([[0, 1], [1, 2], [2, 3], [3, 0]])
TET_FACES = np.array([[0, 2, 1], [0, 1, 3], [1, 2, 3], [2, 0, 3]])  # base/mesh/ElementFaces.hpp
TET_SPLIT = np.array([[0, 1, 3, 4], [1, 3, 4, 5], [3, 4, 5, 7], [1, 3, 5, 2], [3, 5, 2, 7], [5, 2, 7, 6]])
HEX_LEX_OF_HIER = np.array([0, 1, 3, 2, 4, 5, 7, 6])


def rng(seed: int, stream: int) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(np.random.SeedSequence([seed, stream])))


def unit_cube(kind: str, n1: int, n2: int, n3: int = 0):
    """Structured unit square / cube mesh; kind in {'quad', 'hex', 'tet'}."""
    if kind == "quad":
        xs, ys = np.linspace(0, 1, n1 + 1), np.linspace(0, 1, n2 + 1)
        xs = np.arange(n1 + 1) * (1.0 / n1)
        ys = np.arange(n2 + 1) * (1.0 / n2)
        Y, Xg = np.meshgrid(ys, xs, indexing="ij")
        X = np.stack([Xg.ravel(), Y.ravel()], axis=1)
        j, i = np.meshgrid(np.arange(n2), np.arange(n1), indexing="ij")
        base = (i + j * (n1 + 1)).ravel()
        conn = np.stack([base, base + 1, base + 1 + (n1 + 1), base + (n1 + 1)], axis=1)
        return X, conn.astype(np.int64)
    xs = np.arange(n1 + 1) * (1.0 / n1)
    ys = np.arange(n2 + 1) * (1.0 / n2)
    zs = np.arange(n3 + 1) * (1.0 / n3)
    Z, Y, Xg = np.meshgrid(zs, ys, xs, indexing="ij")
    X = np.stack([Xg.ravel(), Y.ravel(), Z.ravel()], axis=1)
    k, j, i = np.meshgrid(np.arange(n3), np.arange(n2), np.arange(n1), indexing="ij")
    b = (i + (n1 + 1) * (j + (n2 + 1) * k)).ravel()
    sx, sy = 1, n1 + 1
    sz = (n1 + 1) * (n2 + 1)
    lex = np.stack([b, b + sx, b + sy, b + sx + sy, b + sz, b + sx + sz, b + sy + sz, b + sx + sy + sz], axis=1)
    if kind == "hex":
        conn = lex[:, [0, 1, 3, 2, 4, 5, 7, 6]]
        return X, conn.astype(np.int64)
    # the split table numbers corners hierarchically; map to lexicographic corners
    conn = lex[:, HEX_LEX_OF_HIER[TET_SPLIT]].reshape(-1, 4)
    return X, conn.astype(np.int64)


def faces_on_plane(shape: int, X, conn, elem, face, axis: int, value: float, tol: float = 1e-9):
    """Select boundary faces whose vertices all lie on x[axis] == value."""
    table = HEX_FACES if shape == A.HEX else (TET_FACES if shape == A.TET else QUAD_EDGES)
    verts = conn[elem[:, None], table[face]]
    on = np.all(np.abs(X[verts, axis] - value) < tol, axis=1)
    return elem[on], face[on]


@dataclass
class Problem:
    name: str
    shape: int
    X: np.ndarray
    conn: np.ndarray
    fedeg: int
    ncomp: int
    kernel: str                       # 'laplace' | 'hyperelastic'
    qdeg: int
    kappa: Optional[np.ndarray] = None
    lam: Optional[np.ndarray] = None
    mu: Optional[np.ndarray] = None
    material: str = "stvenant"
    body: Optional[np.ndarray] = None  # nodal [nnodes, ncomp]
    dirichlet: Optional[Callable] = None  # x -> (mask [n, ncomp], values)
    neumann_plane: Optional[tuple] = None  # (axis, value, traction vector)
    tol: float = 1e-10
    meta: dict = field(default_factory=dict)

    @property
    def nelem(self):
        return len(self.conn)


def _all_boundary(ncomp):
    def f(x):
        return np.ones((len(x), ncomp), dtype=bool), 0.0
    return f


def _clamp_x0(ncomp):
    def f(x):
        m = np.abs(x[:, 0]) < 1e-9
        return np.repeat(m[:, None], ncomp, axis=1), 0.0
    return f


def lame(E, nu):
    """mat/Lame.hpp:28-49"""
    return E * nu / (1.0 + nu) / (1.0 - 2.0 * nu), E / 2.0 / (1.0 + nu)


def config(name: str, n: Optional[int] = None, seed: Optional[int] = None) -> Problem:
    idx = {"c1": 0, "c2": 1, "c3": 2}[name]
    s = SEED_BASE + idx if seed is None else seed
    if name == "c1":
        n = n or 64
        X, conn = unit_cube("quad", n, n)
        kappa = np.exp(rng(s, 0).normal(0.0, 0.5, len(conn)))
        f = rng(s, 1).uniform(0.0, 1.0, len(X))[:, None]
        return Problem("c1", A.QUAD, X, conn, 1, 1, "laplace", 2, kappa=kappa, body=f,
                       dirichlet=_all_boundary(1), tol=1e-10, meta={"n": n})
    if name == "c2":
        n = n or 64
        X, conn = unit_cube("hex", n, n, n)
        E = 10.0 ** rng(s, 0).uniform(3.0, 5.0, len(conn))
        nu = rng(s, 1).uniform(0.2, 0.45, len(conn))
        lam, mu = lame(E, nu)
        return Problem("c2", A.HEX, X, conn, 1, 3, "hyperelastic", 3, lam=lam, mu=mu, material="stvenant",
                       dirichlet=_clamp_x0(3), neumann_plane=(0, 1.0, np.array([1.0, 0.0, 0.0])), tol=1e-10,
                       meta={"n": n})
    n = n or 64
    X, conn = unit_cube("tet", n, n, n)
    h = 1.0 / n
    interior = np.all((X > 1e-9) & (X < 1 - 1e-9), axis=1)
    jit = rng(s, 2).uniform(-0.2 * h, 0.2 * h, X.shape) * interior[:, None]
    # a jitter of 0.2h per coordinate can invert a few of the slim tets; the
    # vertices of an inverted tet go back to their grid position (repeat until
    # every tet has positive volume)
    for _ in range(20):
        Y = X + jit
        a, b, c, d = (Y[conn[:, i]] for i in range(4))
        bad = np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a) <= 0.0
        if not bad.any():
            break
        jit[np.unique(conn[bad])] = 0.0
    X = X + jit
    kappa = np.exp(rng(s, 0).normal(0.0, 1.0, len(conn)))
    f = rng(s, 1).uniform(0.0, 1.0, len(X))[:, None]
    return Problem("c3", A.TET, X, conn, 2, 1, "laplace", 2, kappa=kappa, body=f, dirichlet=_all_boundary(1),
                   tol=1e-10, meta={"n": n})


def setup_system(p: Problem, sys=None):
    """Drive the C-ABI through the reference's setup sequence for problem p."""
    from .system import System
    S = sys or System()
    S.upload_mesh(p.shape, p.X, p.conn)
    S.create_field(p.fedeg, p.ncomp)
    if p.dirichlet is not None:
        S.constrain_boundary(p.dirichlet)
    S.number_dofs()
    S.register_pattern()
    if p.kernel == "laplace":
        S.set_laplace(p.kappa, p.qdeg)
    else:
        S.set_hyperelastic(p.material, p.lam, p.mu, p.qdeg)
    if p.body is not None:
        S.set_body_force_nodal(p.body)
    if p.neumann_plane is not None:
        e, f = S.boundary_faces()
        axis, value, t = p.neumann_plane
        e, f = faces_on_plane(p.shape, p.X, p.conn, e, f, axis, value)
        S.set_neumann(e, f, t, 2)
    return S


# ---------------------------------------------------------------------------
# Nonlinear heat conduction (heat::Static), reference/04-heat/nonlinearHeat.cpp
def heat_reference_solution(x, m):
    """u = ((2^(m+1) - 1) x + 1)^(1/(m+1)) - 1 (nonlinearHeat.cpp:37-44) and its
    gradient, at points x [n, dim]."""
    fac = 2.0 ** (m + 1.0)
    mant = (fac - 1.0) * x[:, 0] + 1.0
    u = mant ** (1.0 / (m + 1.0)) - 1.0
    g = np.zeros_like(x)
    g[:, 0] = (fac - 1.0) / (m + 1.0) * mant ** (1.0 / (m + 1.0) - 1.0)
    return u, g


def nonlinear_heat(S, X, conn, m=3.0, max_iter=10, tolerance=1e-8, qdeg=5, lin_tol=1e-11, method=None):
    """The Newton loop of reference/04-heat/nonlinearHeat.cpp:166-211 through the
    C-ABI: Q2 heat::Static with FenicsTest conductivity (1 + u)^m, u = 0 at
    x = 0 and u = 1 at x = 1 (simpleBC :48-61); per iteration assemble the
    tangent and the residual, stop when |R| = ||b|| / N < tolerance, solve the
    non-symmetric system (BiCGSTAB to lin_tol on the GPU, far below what the
    6 printed digits of the Newton history resolve; SuperLU there), stop
    when |x| < tolerance, add the increment to the DOFs.  Returns
    (ndofs, [(iter, |R|, |x| or None)], L2 error of errorComputation<0>)."""
    n = heat_setup(S, X, conn, m, qdeg)
    rows = heat_newton(S, n, max_iter, tolerance, lin_tol, method)
    xq = S.quadrature_points(qdeg)
    u, _ = heat_reference_solution(xq, m)
    return n, rows, S.error_norm(0, qdeg, u[:, None])


def heat_setup(S, X, conn, m=3.0, qdeg=5):
    """mesh, Q2 field, simpleBC constraints (nonlinearHeat.cpp:48-61), numbering,
    pattern and the FenicsTest heat::Static kernel; returns the DOF count"""
    S.upload_mesh(A.QUAD, X, conn)
    S.create_field(2, 1)

    def bc(x):
        left = np.abs(x[:, 0]) < 1e-5
        right = np.abs(x[:, 0] - 1.0) < 1e-5
        return (left | right)[:, None], np.where(right, 1.0, 0.0)[:, None]
    S.constrain_boundary(bc)
    n = S.number_dofs()
    S.register_pattern()
    S.set_heat_static("fenics", np.full(len(conn), m), qdeg)
    return n


def heat_newton(S, n, max_iter=10, tolerance=1e-8, lin_tol=1e-11, method=None, lin_iters=None):
    """Newton iterations of nonlinearHeat.cpp:166-207 from the context's current
    DOF values; returns [(iter, |R|, |x| or None)] and appends the linear
    iteration counts to lin_iters when given"""
    if method is None:
        method = A.SOLVE_BICGSTAB
    rows = []
    it = 0
    while it < max_iter:
        S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
        rn = S.norm()
        if rn < tolerance:
            rows.append((it, rn, None))
            break
        li, _, _ = S.solve(method, tol=lin_tol)
        if lin_iters is not None:
            lin_iters.append(li)
        xn = S.norm()
        if xn < tolerance:
            rows.append((it, rn, xn))
            break
        rows.append((it, rn, xn))
        S.distribute(add=True)
        it += 1
    return rows


def pulled_sheet_faces(S, X, conn):
    """boundary faces on x = 1 and the y coordinate of their two vertices
    (face vertex order of QUAD_EDGES)"""
    e, f = S.boundary_faces()
    e, f = faces_on_plane(A.QUAD, X, conn, e, f, 0, 1.0, tol=1e-5)
    y = X[conn[e[:, None], QUAD_EDGES[f]], 1]
    return e, f, y


def compressible(S, X, conn, E=1000.0, nu=0.3, max_iter=30, load_steps=5, pull=3.0, traction=1000.0,
                 disp_controlled=True, tolerance=1e-12, lin_tol=1e-12, method=None):
    """reference/06-elastic/compressible.cpp through the C-ABI: a Q2 sheet of
    NeoHookeanCompressible material (E, nu), clamped at x = 0 and pulled at
    x = 1 (PulledSheet.hpp:35-75): by the displacement pull in x
    (disp_controlled) or by the traction value (y - 1/2) in x, raised in
    load_steps equal steps.  Per load step (compressible.cpp:245-330) the
    Dirichlet values are scaled up (scaleConstraints, :254), then Newton:
    assemble the tangent and residual, stop when |R| = ||b|| / N < tolerance E
    (:298-302), solve (cgSolve there, CG to lin_tol here), stop when
    |x| < tolerance (:315-321), add the increment.  The traction is
    tabulated at the vertices of the x = 1 faces (isl_set_neumann_vertex),
    exact for this linear profile.  Returns (ndofs, [(step, iter, |R|, |x| or
    None)])."""
    if method is None:
        method = A.SOLVE_CG_FP64
    lam, mu = lame(E, nu)
    S.upload_mesh(A.QUAD, X, conn)
    S.create_field(2, 2)
    first_pull = pull / load_steps

    def bc(x):
        left = np.abs(x[:, 0]) < 1e-6
        right = np.abs(x[:, 0] - 1.0) < 1e-6
        mask = np.zeros((len(x), 2), dtype=bool)
        vals = np.zeros((len(x), 2))
        mask[left, :] = True
        if disp_controlled:
            mask[right, 0] = True
            vals[right, 0] = first_pull
        return mask, vals
    S.constrain_boundary(bc)
    n = S.number_dofs()
    S.register_pattern()
    S.set_hyperelastic("neohooke", np.full(len(conn), lam), np.full(len(conn), mu), 3)
    if not disp_controlled:
        fe, ff, fy = pulled_sheet_faces(S, X, conn)
    rows = []
    for step in range(load_steps):
        S.scale_constraints(float(step + 1) if step == 0 else (step + 1) / step)
        it = 0
        while it < max_iter:
            if not disp_controlled:
                t = np.zeros((len(fe), 2, 2))
                t[:, :, 0] = traction * (step + 1) / load_steps * (fy - 0.5)
                S.set_neumann_vertex(fe, ff, t, 3)
            S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
            conv1 = S.norm()
            if conv1 < tolerance * E:
                rows.append((step, it, conv1, None))
                break
            S.solve(method, tol=lin_tol)
            conv2 = S.norm()
            S.distribute(add=True)
            rows.append((step, it, conv1, conv2))
            it += 1
            if conv2 < tolerance:
                break
    return n, rows


# ---------------------------------------------------------------------------
# Linear multi-step time integration (base/time/BDF.hpp, MultiStep.hpp)
# BDF LHS weights a_0..a_q as base/time/BDF.hpp:95-104 defines them (its
# 4th-order row carries +4/3 where the table in its comment has -4/3; the
# coded values are the reference's behaviour).
BDF_WEIGHTS = {1: [1.0, -1.0], 2: [1.5, -2.0, 0.5], 3: [11.0 / 6.0, -3.0, 1.5, -1.0 / 3.0],
               4: [25.0 / 12.0, -4.0, 3.0, 4.0 / 3.0, 1.0 / 4.0]}


def bdf_weights(order: int, step: int):
    """systemMassWeight(step) and reactionWeights(step) of BDF<order>
    (base/time/MultiStep.hpp:104-127): the order ramps up over the first steps,
    q = order while step + 2 >= q + 1, else one lower (LHSWeights :28-44)."""
    q = order
    while q > 1 and step + 2 < q + 1:
        q -= 1
    a = BDF_WEIGHTS[q]
    return a[0], list(a)


def inertia_weights(order: int, step: int, dt: float, incremental: bool = True):
    """lhs weight and history weights of isl_set_inertia for BDF<order> at a
    step (ReactionTerms.hpp:214-248): a0 / dt and -a_s / dt, the current values'
    weight dropped when not incremental"""
    a0, a = bdf_weights(order, step)
    w = [-x / dt for x in a]
    if not incremental:
        w[0] = 0.0
    return a0 / dt, w


# Adams-Moulton RHS weights b_0..b_{q-1} (base/time/AdamsMoulton.hpp:70-84);
# its LHS weights are always (1, -1)
AM_WEIGHTS = {1: [1.0], 2: [0.5, 0.5], 3: [5.0 / 12.0, 2.0 / 3.0, -1.0 / 12.0],
              4: [3.0 / 8.0, 19.0 / 24.0, -5.0 / 24.0, 1.0 / 24.0]}


def multistep_weights(method: str, order: int, step: int):
    """LHS and RHS weights of BDF<order> or AdamsMoulton<order> at a step, with
    the ramp-up of base/time/MultiStep.hpp:28-62 (a lower order while the step
    count cannot feed the full formula)."""
    if method == "bdf":
        return bdf_weights(order, step)[1], [1.0]
    q = order
    while q > 1 and step + 2 < q:
        q -= 1
    return [1.0, -1.0], list(AM_WEIGHTS[q])


def time_weights(method: str, order: int, step: int, dt: float, incremental: bool = True):
    """The arguments of isl_set_inertia and isl_set_force_history for a step:
    systemMassWeight / dt, -reactionWeights / dt (MultiStep.hpp:104-127) and the
    forceWeights b_s / b_0, s >= 1 (:129-137)."""
    a, b = multistep_weights(method, order, step)
    w = [-(x / b[0]) / dt for x in a]
    if not incremental:
        w[0] = 0.0
    return a[0] / b[0] / dt, w, [x / b[0] for x in b[1:]]


def unsteady(S, rho, steps, dt, order=2, lin_tol=1e-12, method=None, scheme="bdf", newton=1):
    """Implicit multi-step time stepping (BDF or Adams-Moulton) of
    rho du/dt + F_int(u) = f on the context's problem (kernel already set,
    initial values in the DOFs): rho du/dt - div(k grad u) = f for Laplace and
    heat::Static, the same first-order inertia on each displacement component
    for HyperElastic.  Per step `newton` Newton iterations from the current
    values (one suffices for Laplace, which is linear in u), then
    pushHistory.  Returns the DOF values after every step."""
    if method is None:
        method = A.SOLVE_CG_FP64
    out = []
    S.set_history(order)
    S.push_history()
    for k in range(steps):
        mw, w, fw = time_weights(scheme, order, k, dt)
        S.set_inertia(rho, mw, w)
        S.set_force_history(fw)
        for _ in range(newton):
            S.assemble(A.PREC_FP64, incremental=True, with_residual=True)
            S.solve(method, tol=lin_tol)
            S.distribute(add=True)
        S.push_history()
        out.append(S.values())
    return out


# the heat equation's name for the driver
unsteady_heat = unsteady
