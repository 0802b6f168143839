"""The header-only C++ SOLVER adapter (include/isl_gpu_solver.hpp) compiles
against the C-ABI, links with libisl_gpu.so and drives the host-side steps of
the pipeline on a host-only context (no GPU): SMF write and read, the DOF
pipeline and the constraints, with the counts the Python binding gets."""
import os
import shutil
import subprocess

import pytest

from insilico_gb300 import _abi as A
from insilico_gb300 import build as B
from insilico_gb300 import workloads as W
from insilico_gb300.system import System

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <cstdio>
#include "isl_gpu_solver.hpp"
int main(int argc, char** argv) {
    isl::Gb300Solver s(-1);
    s.readSMF(argv[1], ISL_QUAD);
    s.writeSMF(argv[2]);
    const long long ndofobj = (long long)s.field(2, 1);
    s.constrainBoundary(2, [](const double* x, int, double& v) { v = x[0]; return x[0] < 1e-9 || x[0] > 1 - 1e-9; });
    const long long n = (long long)s.numberDoFs();
    std::printf("%lld %lld\n", ndofobj, n);
    try { s.registerFields(); } catch (const isl::gpu_error& e) { std::printf("device-only %d\n", e.code); }
    const isl::QuadratureRule q = isl::quadratureRule(ISL_TET, 4);
    double sum = 0.0;
    for (double w : q.w) sum += w;
    std::printf("%zu %.17g\n", q.w.size(), sum);
    return 0;
}
"""


def test_cpp_adapter_builds_and_runs_host_steps(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    lib = B.build()
    src = tmp_path / "prog.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "prog"
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O1", str(src), "-I", os.path.join(ROOT, "include"), "-L", libdir,
                    "-lisl_gpu", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    X, conn = W.unit_cube("quad", 7, 5)
    S = System(device=-1)
    S.upload_mesh(A.QUAD, X, conn)
    S.write_smf(tmp_path / "in.smf")
    out = subprocess.run([str(exe), str(tmp_path / "in.smf"), str(tmp_path / "out.smf")], check=True,
                         capture_output=True, text=True).stdout.split("\n")
    ndofobj, n = (int(t) for t in out[0].split())
    assert out[1].startswith("device-only")
    nq, wsum = out[2].split()
    w, _ = A.quadrature_rule(A.TET, 4)
    assert int(nq) == 11 and float(wsum) == pytest.approx(w.sum(), rel=1e-15)
    assert (tmp_path / "out.smf").read_text() == (tmp_path / "in.smf").read_text()
    # the same steps through the Python binding
    S.create_field(2, 1)
    S.constrain_boundary(lambda x: (((x[:, 0] < 1e-9) | (x[:, 0] > 1 - 1e-9))[:, None], x[:, :1]))
    assert ndofobj == S.ndofobj and n == S.number_dofs()
