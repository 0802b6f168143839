"""The C++ SOLVER adapter (include/isl_gpu_solver.hpp) on the GPU: a C++
program compiled against it runs the reference's linear-elastic call
sequence (reference/06-elastic/linearElastic.cpp:131-200) on a hex8 cube:
mesh -> field -> constrainBoundary -> numberDoFs -> registerFields ->
HyperElastic<StVenant> with per-element materials + a Neumann traction on
x = 1 -> assemble -> norm() -> cgSolve -> getValue / norm(); then the served
path (Gb300Server) on two neo-Hookean requests.  Compared with the oracle:

* norm() after the assembly and before the solve is ||b|| / N, the value
  solid/CompressibleDriver.hpp:190-197 tests for convergence (1e-12);
* getValue over all DOFs is the oracle's FP64 CG solution (1e-9), and norm()
  after the solve is ||x|| / N;
* the served requests reproduce the oracle's run of the reference driver (1e-8).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from insilico_gb300 import _abi as A
from insilico_gb300 import build as B
from insilico_gb300 import serve
from insilico_gb300 import workloads as W

from helpers import oracle_newton_driver, oracle_problem
import oracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N = 5

PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "isl_gpu_solver.hpp"

// unit-cube hex8 mesh: nodes with the first coordinate fastest, corners in
// hierarchic order (0,1,3,2,4,5,7,6 of the lexicographic corners)
static void cube(int n, std::vector<double>& X, std::vector<int64_t>& conn) {
    const int m = n + 1;
    for (int k = 0; k < m; ++k) for (int j = 0; j < m; ++j) for (int i = 0; i < m; ++i) {
        X.push_back(double(i) / n); X.push_back(double(j) / n); X.push_back(double(k) / n);
    }
    const int lex2h[8] = {0, 1, 3, 2, 4, 5, 7, 6};
    for (int k = 0; k < n; ++k) for (int j = 0; j < n; ++j) for (int i = 0; i < n; ++i) {
        const int64_t b = i + m * (j + m * k);
        const int64_t lex[8] = {b, b + 1, b + m, b + 1 + m, b + m * m, b + 1 + m * m, b + m + m * m, b + 1 + m + m * m};
        for (int a = 0; a < 8; ++a) conn.push_back(lex[lex2h[a]]);
    }
}

int main(int argc, char** argv) {
    const int n = atoi(argv[1]);
    std::vector<double> X;
    std::vector<int64_t> conn;
    cube(n, X, conn);
    const size_t ne = conn.size() / 8;
    // linear elasticity: per-element Lame parameters (mat/Lame.hpp:28-49)
    std::vector<double> lam(ne), mu(ne);
    for (size_t e = 0; e < ne; ++e) {
        const double E = 1e3 * (1.0 + double(e % 7)), nu = 0.2 + 0.03 * double(e % 5);
        lam[e] = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu);
        mu[e] = E / 2.0 / (1.0 + nu);
    }
    isl::Gb300Solver s(0);
    s.mesh(ISL_HEX, 3, X, conn, 8);
    s.field(1, 3);
    s.constrainBoundary(3, [](const double* x, int, double& v) { v = 0.0; return x[0] < 1e-9; });
    const size_t neq = s.numberDoFs();
    s.registerFields();
    s.hyperElastic(ISL_MAT_STVENANT, lam, mu, 3);
    std::vector<int64_t> be;
    std::vector<int> bf;
    s.boundaryFaces(be, bf);
    const int faces[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};
    std::vector<int64_t> ne_;
    std::vector<int> nf_;
    std::vector<double> tr;
    for (size_t i = 0; i < be.size(); ++i) {
        bool on = true;
        for (int a = 0; a < 4; ++a) on = on && X[3 * conn[8 * be[i] + faces[bf[i]][a]]] > 1.0 - 1e-9;
        if (on) { ne_.push_back(be[i]); nf_.push_back(bf[i]); tr.push_back(1.0); tr.push_back(0.0); tr.push_back(0.0); }
    }
    s.neumann(ne_, nf_, tr, 2);
    s.assemble(ISL_PREC_FP64, true, false);
    s.finishAssembly();
    std::printf("%zu %.17g\n", neq, s.norm());
    const int it = s.cgSolve(1e-12);
    std::printf("%d %.17g\n", it, s.norm());
    for (size_t i = 0; i < neq; ++i) std::printf("%.17g\n", s.getValue(i));

    // served path: two neo-Hookean cubes of sides 3 and 4 (PulledSheet
    // conditions, 5 load steps), one batch
    isl::Gb300Server srv(0, ISL_PREC_FP32, 8, 1, 0, 200000);  // requests submitted together: one batch
    const int sides[2] = {3, 4};
    const double mus[2] = {1.7, 0.4};
    std::vector<int64_t> tickets;
    std::vector<std::vector<double>> Xs(2), c0(2), c1(2), fv(2);
    std::vector<std::vector<int64_t>> cs(2), fn(2);
    std::vector<std::vector<int>> fc(2);
    for (int r = 0; r < 2; ++r) {
        cube(sides[r], Xs[r], cs[r]);
        const size_t ner = cs[r].size() / 8, nn = Xs[r].size() / 3;
        c0[r].assign(ner, 10.0 * mus[r] - 2.0 * mus[r] / 3.0);
        c1[r].assign(ner, mus[r]);
        for (size_t i = 0; i < nn; ++i) {
            if (Xs[r][3 * i] < 1e-9) for (int c = 0; c < 3; ++c) { fn[r].push_back(i); fc[r].push_back(c); fv[r].push_back(0.0); }
            if (Xs[r][3 * i] > 1.0 - 1e-9) { fn[r].push_back(i); fc[r].push_back(0); fv[r].push_back(0.3 / 5); }
        }
        isl_serve_request q{};
        q.shape = ISL_HEX; q.n_nodes = nn; q.coords = Xs[r].data(); q.n_elem = ner; q.conn = cs[r].data();
        q.ncomp = 3; q.kernel = ISL_KERNEL_HYPERELASTIC; q.material = ISL_MAT_NEOHOOKE; q.quad_degree = 3;
        q.coef0 = c0[r].data(); q.coef1 = c1[r].data(); q.body = nullptr;
        q.n_fixed = fn[r].size(); q.fixed_node = fn[r].data(); q.fixed_comp = fc[r].data(); q.fixed_value = fv[r].data();
        q.load_steps = 5; q.max_newton = 12; q.tolerance = 1e-12; q.lin_tol = 1e-6;
        tickets.push_back(srv.submit(q));
    }
    for (int r = 0; r < 2; ++r) {
        isl_serve_stats st{};
        const std::vector<double> u = srv.result(tickets[r], Xs[r].size(), &st);
        std::printf("served %d %lld %d\n", r, (long long)st.newton_iters, st.batch_size);
        for (double v : u) std::printf("%.17g\n", v);
    }
    return 0;
}
"""


def materials(ne):
    e = np.arange(ne)
    E = 1e3 * (1.0 + (e % 7))
    nu = 0.2 + 0.03 * (e % 5)
    return W.lame(E, nu)


def test_cpp_adapter_pipeline_and_server_on_gpu(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    lib = B.build()
    src = tmp_path / "prog.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "prog"
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O1", str(src), "-I", os.path.join(ROOT, "include"), "-L", libdir,
                    "-lisl_gpu", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(N)], check=True, capture_output=True, text=True, timeout=600).stdout.split("\n")
    neq, norm_b = int(out[0].split()[0]), float(out[0].split()[1])
    it, norm_x = int(out[1].split()[0]), float(out[1].split()[1])
    x = np.array([float(v) for v in out[2:2 + neq]])
    # the same problem on the oracle
    X, conn = W.unit_cube("hex", N, N, N)
    lam, mu = materials(len(conn))
    p = W.Problem("cpp", A.HEX, X, conn, 1, 3, "hyperelastic", 3, lam=lam, mu=mu, material="stvenant",
                  dirichlet=lambda x: (np.repeat((np.abs(x[:, 0]) < 1e-9)[:, None], 3, axis=1), 0.0),
                  neumann_plane=(0, 1.0, np.array([1.0, 0.0, 0.0])))
    P, (rp, ci, v, b) = oracle_problem(p)
    assert neq == P.neq
    assert abs(norm_b - np.linalg.norm(b) / neq) <= 1e-12 * np.linalg.norm(b) / neq
    xo, ito, _ = O.cg(rp, ci, v, b, tol=1e-13)
    assert np.linalg.norm(x - xo) <= 1e-9 * np.linalg.norm(xo)
    assert abs(norm_x - np.linalg.norm(x) / neq) <= 1e-12 * norm_x
    assert it > 0
    # served requests
    pos = 2 + neq
    for r, (side, m) in enumerate(((3, 1.7), (4, 0.4))):
        head = out[pos].split()
        assert head[0] == "served" and int(head[1]) == r and int(head[3]) == 2
        nd = 3 * (side + 1) ** 3
        u = np.array([float(t) for t in out[pos + 1:pos + 1 + nd]])
        pos += 1 + nd
        uo, _ = oracle_newton_driver(serve.Request(r, side, m), serve.NEWTON_TOL, serve.MAX_NEWTON)
        assert np.linalg.norm(u - uo) <= 1e-8 * np.linalg.norm(uo)
