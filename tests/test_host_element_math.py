"""The element function of the generic HyperElastic kernel (hyper_element in
insilico_gb300/csrc/isl_hyper.cu, __host__ __device__) compiled for the host
and run on the oracle's inputs (CPU, no GPU): the element matrices and
vectors it stages, assembled with the oracle's equation numbers, equal the
oracle's system.  This checks the kernel's arithmetic in every CPU test
run; the GPU tests check the same kernel on the device
(test_gpu_elastic2d.py, test_gpu_hyper_shapes.py)."""
import os
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

import oracle as O
from insilico_gb300 import _abi as A
from insilico_gb300 import build as B
from insilico_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHAPES = {"quad": (A.QUAD, O.QUAD, 2), "tet": (A.TET, O.TET, 3), "hex": (A.HEX, O.HEX, 3)}


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    try:
        nvcc = B.nvcc()
    except RuntimeError:
        pytest.skip("no nvcc")
    lib = B.build()
    out = tmp_path_factory.mktemp("host_elem") / "hyper_element_host"
    libdir = os.path.dirname(lib)
    cmd = [nvcc, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), *B.ARCH, "-o", str(out),
           os.path.join(ROOT, "tests", "host_elem", "hyper_element_host.cu"), "-L", libdir, "-lisl_gpu", "-lcudart",
           "-Xlinker", "-rpath", "-Xlinker", libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return str(out)


def _unpack(v, n):
    K = np.zeros((n, n))
    K[np.triu_indices(n)] = v
    return K + np.triu(K, 1).T


@pytest.mark.parametrize("kind,sizes,deg,qdeg,nq,material,body,inertia,nfw", [
    ("quad", (4, 3), 2, 3, 4, "neohooke", True, False, 0),
    ("quad", (3, 3), 1, 5, 9, "stvenant", False, True, 2),
    ("tet", (2, 2, 1), 1, 2, 4, "stvenant", True, False, 0),
    ("tet", (2, 1, 1), 2, 2, 4, "neohooke", True, True, 2),
    ("tet", (2, 1, 1), 2, 1, 1, "stvenant", False, False, 0),
    ("tet", (2, 1, 1), 2, 4, 11, "neohooke", True, True, 2),
    ("hex", (2, 1, 1), 1, 4, 27, "neohooke", True, True, 1),
])
def test_hyper_element_matches_oracle(harness, tmp_path, kind, sizes, deg, qdeg, nq, material, body, inertia, nfw):
    ashape, oshape, D = SHAPES[kind]
    X, conn = W.unit_cube(kind, *sizes)
    rng = np.random.default_rng(1)
    inner = np.all((X > 1e-9) & (X < 1 - 1e-9), axis=1)
    X = X + rng.uniform(-0.03, 0.03, X.shape) * inner[:, None] / max(sizes)
    E = len(conn)
    P = O.Problem(oshape, X, conn, deg, D)
    P.number()
    lam, mu = rng.uniform(1, 2, E), rng.uniform(0.5, 1, E)
    P.set_hyperelastic(material, lam, mu, qdeg)
    nobj = P.ndofobj
    u = rng.uniform(-0.02, 0.02, nobj * D)
    P.set_values(u)
    f = rng.uniform(-1, 1, (len(X), D))
    if body:
        P.set_body_nodal(f.reshape(-1))
    hist = [rng.uniform(-0.02, 0.02, nobj * D) for _ in range(2)]
    w, fw = [3.0, -4.0, 1.0], [0.3, -0.2][:nfw]
    rho = rng.uniform(0.5, 1.5, E)
    if inertia or nfw:
        P.set_inertia(rho, 7.5, w, hist, fw)
    edof = P.elem_dofobj()
    files = {"X": np.ascontiguousarray(X, dtype=np.float64), "conn": np.ascontiguousarray(conn.T, dtype=np.int32),
             "edof": np.ascontiguousarray(edof.T, dtype=np.int32), "u": u, "coef": np.concatenate([lam, mu]),
             "fnodal": f, "rho": rho, "hvec": w[0] * u + w[1] * hist[0] + w[2] * hist[1],
             "hist": np.concatenate(hist)}
    for name, arr in files.items():
        np.ascontiguousarray(arr).tofile(tmp_path / f"{name}.bin")
    args = [ashape, E, len(X), nobj, deg, nq, qdeg, 0 if material == "stvenant" else 1, int(body), int(inertia), 7.5,
            nfw, fw[0] if nfw > 0 else 0.0, fw[1] if nfw > 1 else 0.0, 2]
    r = subprocess.run([harness, *map(str, args)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert r.stdout.startswith("flags 0")
    nloc = D * edof.shape[1]
    SK = np.fromfile(tmp_path / "SK.bin").reshape(E, nloc * (nloc + 1) // 2)
    SF = np.fromfile(tmp_path / "SF.bin").reshape(nloc, E)
    eq = P.eq_index()
    n = P.neq
    K = np.zeros((n, n))
    b = np.zeros(n)
    for e in range(E):
        idx = eq[edof[e][np.arange(nloc) // D] * D + np.arange(nloc) % D]
        K[np.ix_(idx, idx)] += _unpack(SK[e], nloc)
        np.add.at(b, idx, SF[:, e])
    rp, ci, v, bo = P.assemble(incremental=True, with_residual=True)
    Ko = sp.csr_matrix((v, ci, rp), shape=(n, n)).toarray()
    assert np.abs(K - Ko).max() <= 1e-13 * np.abs(Ko).max()
    assert np.abs(b - bo).max() <= 1e-13 * np.abs(bo).max()
