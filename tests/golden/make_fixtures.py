"""Extract the reference's golden pins into tests/golden/reference_pins.json.

Run once in a checkout where the reference project is mounted (it reads the
reference's own golden files and fixture meshes); the JSON it writes is what
the tests use, so nothing at test time needs the reference tree.

    python tests/golden/make_fixtures.py /path/to/inSilico
    INSILICO_REFERENCE=/path/to/inSilico python tests/golden/make_fixtures.py

Pins extracted (file paths relative to the reference project):
  reference/03-doFHandler/sparsity.{1,2,3}.ref.dat  -> sha256 + count of the data lines
  reference/03-doFHandler/square_20.smf              -> canonical mesh hash
  reference/06-elastic/{quad,cube}.*.smf             -> canonical mesh hashes
  reference/06-elastic/linearElastic{2,3}D.ref.dat   -> (N, L2) table
  reference/06-elastic/compRefOut{D,N}.dat           -> Newton history tables
  reference/05-mixedPoisson/ref                      -> ndofs, L2, H1
  reference/05-mixedPoisson/square_020.smf           -> canonical mesh hash
  reference/04-heat/square_200.smf                   -> canonical mesh hash
  reference/04-heat/nonlinearHeat.ref.dat            -> dofs, Newton |R|/|x| history, L2 error
  reference/06-elastic/quad.020.{D,N}ref.vtk         -> sha256 + count of the grid lines and of
                                                        the POINT_DATA section lines
"""
import glob
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def mesh_hash(X, conn):
    """Canonical hash of a mesh: coordinates as %.17g and connectivity."""
    h = hashlib.sha256()
    for row in np.asarray(X, dtype=np.float64):
        h.update((" ".join("%.17g" % v for v in row) + "\n").encode())
    for row in np.asarray(conn, dtype=np.int64):
        h.update((" ".join(str(int(v)) for v in row) + "\n").encode())
    return h.hexdigest()


def lines_hash(lines):
    h = hashlib.sha256()
    for l in lines:
        h.update((l + "\n").encode())
    return h.hexdigest()


def read_smf(path):
    with open(path) as f:
        lines = [l for l in f.read().splitlines() if l.strip() and not l.startswith("#") and not l.startswith("!")]
    nn, ne = (int(t) for t in lines[0].split()[:2])
    X = np.array([[float(t) for t in l.split()] for l in lines[1:1 + nn]])
    conn = np.array([[int(t) for t in l.split()] for l in lines[1 + nn:1 + nn + ne]], dtype=np.int64)
    return X, conn


def canon_lines(lines, zero=1e-10):
    """Lines with every number of magnitude below `zero` written as "~0": the
    round-off residue of quantities that vanish (e.g. a displacement on a
    symmetry line) differs between builds, everything else is kept verbatim."""
    out = []
    for l in lines:
        toks = []
        for t in l.split(" "):
            try:
                toks.append("~0" if t and abs(float(t)) < zero else t)
            except ValueError:
                toks.append(t)
        out.append(" ".join(toks))
    return out


def table(path):
    rows = []
    with open(path) as f:
        for l in f:
            if l.startswith("#") or not l.strip():
                continue
            rows.append(l.split())
    return rows


def main(ref):
    out = {"source": "thrueberg/inSilico golden files", "sparsity": {}, "meshes": {}}
    for d in (1, 2, 3):
        p = os.path.join(ref, "reference/03-doFHandler/sparsity.%d.ref.dat" % d)
        with open(p) as f:
            data = [l.rstrip("\n") for l in f if not l.startswith("#")]
        out["sparsity"][str(d)] = {"lines": len(data), "sha256": lines_hash(data),
                                   "head": data[:12], "tail": data[-6:]}
    smfs = [os.path.join(ref, "reference/03-doFHandler/square_20.smf"),
            os.path.join(ref, "reference/05-mixedPoisson/square_020.smf"),
            os.path.join(ref, "reference/04-heat/square_200.smf")]
    smfs += sorted(glob.glob(os.path.join(ref, "reference/06-elastic/quad.*.smf")))
    smfs += sorted(glob.glob(os.path.join(ref, "reference/06-elastic/cube.*.smf")))
    for p in smfs:
        X, conn = read_smf(p)
        out["meshes"][os.path.relpath(p, ref)] = {"nodes": len(X), "elements": len(conn),
                                                  "dim_cols": X.shape[1], "sha256": mesh_hash(X, conn)}
    out["linearElastic2D"] = [[int(r[0]), float(r[1])] for r in table(os.path.join(ref, "reference/06-elastic/linearElastic2D.ref.dat"))]
    out["linearElastic3D"] = [[int(r[0]), float(r[1])] for r in table(os.path.join(ref, "reference/06-elastic/linearElastic3D.ref.dat"))]
    for tag in ("D", "N"):
        p = os.path.join(ref, "reference/06-elastic/compRefOut%s.dat" % tag)
        with open(p) as f:
            first = f.readline()
        ndofs = int(first.split()[-1])
        rows = [[int(r[0]), int(r[1])] + [float(v) for v in r[2:]] for r in table(p)]
        out["compRefOut" + tag] = {"ndofs": ndofs, "rows": rows}
    with open(os.path.join(ref, "reference/05-mixedPoisson/ref")) as f:
        txt = f.read().splitlines()
    out["mixedPoisson"] = {"ndofs": int(txt[0].split()[-1]), "L2": float(txt[1].split()[-1]),
                           "H1": float(txt[2].split()[-1]), "volume": float(txt[3].split()[-1])}
    # reference/04-heat/nonlinearHeat.ref.dat: dof count, Newton |R| / |x| per
    # iteration, iteration count, L2 error
    with open(os.path.join(ref, "reference/04-heat/nonlinearHeat.ref.dat")) as f:
        txt = f.read()
    import re
    newton = []
    for mt in re.finditer(r"(\d+):\s+\|R\| = ([0-9.eE+-]+)(?:,\s+\|x\| = ([0-9.eE+-]+))?", txt):
        newton.append([int(mt.group(1)), float(mt.group(2)), float(mt.group(3)) if mt.group(3) else None])
    out["nonlinearHeat"] = {"ndofs": int(re.search(r"Number of dofs (\d+)", txt).group(1)),
                            "newton": newton,
                            "iterations": int(re.search(r"Converged to given tolerance in (\d+)", txt).group(1)),
                            "L2": float(re.search(r"L2-error = ([0-9.eE+-]+)", txt).group(1))}
    out["vtk"] = {}
    for tag in ("D", "N"):
        rel = "reference/06-elastic/quad.020.%sref.vtk" % tag
        with open(os.path.join(ref, rel)) as f:
            lines = f.read().splitlines()
        ip = next(i for i, l in enumerate(lines) if l.startswith("POINT_DATA"))
        ic = next((i for i, l in enumerate(lines) if l.startswith("CELL_DATA")), len(lines))
        out["vtk"][tag] = {"file": rel, "grid_lines": ip, "grid_sha256": lines_hash(lines[:ip]),
                           "point_lines": ic - ip, "point_sha256": lines_hash(lines[ip:ic]),
                           "point_canon_sha256": lines_hash(canon_lines(lines[ip:ic])),
                           "point_head": lines[ip:ip + 4]}
    with open(os.path.join(HERE, "reference_pins.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "reference_pins.json"))


if __name__ == "__main__":
    ref_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("INSILICO_REFERENCE")
    if not ref_root:
        sys.exit("usage: make_fixtures.py /path/to/inSilico  (or set INSILICO_REFERENCE)")
    main(ref_root)
