"""SHA-256 pins of the oracle's DOF numbering and CSR pattern at the full
configuration sizes, written to tests/golden/fullsize_hashes.json.

The oracle (the CPU restatement of the reference's DOF pipeline and
TripletContainer::registerFields) numbers and patterns:

  c2  hex8 linear elasticity 64^3 (x = 0 clamped): 811,200 equations
  c3  tet10 Poisson 64^3 (Dirichlet on all faces): 2,146,689 DOF objects
  c4  single c4 instances (unit square, Dirichlet on all edges) of side 8,
      131 and 256 in Q1 and Q2

Every array is hashed as little-endian int64: the per-element DOF-object ids
([n_elem][n_fun], the first-visit numbering of base/dof/generateDoFIndicesFromFaces.hpp),
the equation index per DOF-object component (-1 constrained,
base/dof/numbering.hpp:44-68), and the CSR row pointers and column indices.
The GPU tests hash the library's arrays the same way.  Only integer work
decides these arrays (connectivity, face keys, constraint flags), so the pins
hold on any host.

    python tests/golden/make_fullsize_hashes.py
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from insilico_gb300 import workloads as W  # noqa: E402

SHAPE = {3: O.QUAD, 4: O.TET, 5: O.HEX}
C4_SIDES = (8, 131, 256)


def h64(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i8").tobytes()).hexdigest()


def pins(shape, X, conn, fedeg, ncomp, dirichlet):
    P = O.Problem(SHAPE[shape], X, conn, fedeg, ncomp)
    x, d = P.boundary_points()
    mask, vals = dirichlet(x)
    mask = np.asarray(mask, dtype=bool).reshape(len(x), ncomp)
    r, c = np.nonzero(mask)
    P.constrain(d[r], c, np.zeros(len(r)))
    P.number()
    rp, ci = P.pattern()
    return {"n_elem": int(len(conn)), "n_dofobj": int(P.ndofobj), "neq": int(P.neq), "nnz": int(len(ci)),
            "elem_dofobj_sha256": h64(P.elem_dofobj()), "eq_index_sha256": h64(P.eq_index()),
            "rowptr_sha256": h64(rp), "colind_sha256": h64(ci)}


def main():
    out = {"format": "sha256 of little-endian int64 arrays", "configs": {}, "c4_instances": {}}
    for name in ("c2", "c3"):
        t0 = time.time()
        p = W.config(name)
        out["configs"][name] = pins(p.shape, p.X, p.conn, p.fedeg, p.ncomp, p.dirichlet)
        print(name, out["configs"][name], f"{time.time() - t0:.1f}s", flush=True)
    for deg in (1, 2):
        for side in C4_SIDES:
            X, conn = W.unit_cube("quad", side, side)
            key = f"Q{deg}_side{side}"
            out["c4_instances"][key] = pins(3, X, conn, deg, 1, lambda x: (np.ones((len(x), 1), dtype=bool), 0.0))
            print(key, out["c4_instances"][key], flush=True)
    with open(os.path.join(HERE, "fullsize_hashes.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "fullsize_hashes.json"))


if __name__ == "__main__":
    main()
