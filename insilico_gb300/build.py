"""Build the GB300 (sm_103a) shared library libisl_gpu.so in-tree.

Each translation unit is compiled by nvcc in parallel, then linked into
insilico_gb300/_build/libisl_gpu.so.  No cmake, one -gencode.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libisl_gpu.so")
SOURCES = ["isl_host.cpp", "isl_assembly.cu", "isl_hyper.cu", "isl_solver.cu", "isl_batch.cu", "isl_dofmap.cu", "isl_post.cu",
           "isl_io.cpp", "isl_krylov.cu", "isl_serve.cpp", "isl_blocks.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(verbose_ptxas: bool = False):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
                "--expt-relaxed-constexpr", "-Xcompiler", "-Wno-unused-function"]
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _compile(src: str, verbose_ptxas: bool) -> tuple[str, str]:
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    cmd = [nvcc(), *_flags(verbose_ptxas), "-x", "cu" if src.endswith(".cu") else "c++", "-c",
           os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"), "-c",
               os.path.join(CSRC, src), "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{p.stdout}\n{p.stderr}")
    return obj, p.stderr


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "isl_gpu.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    if verbose_ptxas:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"link failed:\n{p.stdout}\n{p.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
