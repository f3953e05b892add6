"""Regenerate the golden fixtures in this folder from the reference's own tests.

Run in a container where the underworld2 source tree is mounted:

    python tests/golden/make_golden.py /path/to/underworld2

It reads, as text or binary data only (nothing of the reference is built or
executed):

* ``L/PICellerator/Weights/tests/DVCWeightsSuite.c`` -- the hard-coded 2D and
  3D particle sets of the discrete-Voronoi suite (10 particles, 10^d grid),
  and ``tests/expected/DVCWeightsSuite_testGetCentroids{,2D}.txt`` -- the
  expected centroids and weights (printed to 6 decimals);
* ``L/StgFEM/Assembly/tests/expected/testIsoviscousSiffness.matrix`` -- the
  PETSc-binary 32x32 AIJ stiffness matrix of a 2D 3x3 Q1 mesh with unit
  viscosity, no boundary conditions (big-endian: classid, rows, cols, nnz,
  row lengths, column indices, values);
* the docstring known answers of ``P/swarm/layouts.py`` (PerCellRandomLayout,
  seed 13), ``P/systems/_timeintegration.py`` (RK2 of one particle) and
  ``P/swarm/_swarm.py`` (owner after a move), copied as numbers.

Output: ``golden.json`` (small) beside this script.
"""
import json
import os
import re
import struct
import sys

import numpy as np

L = "src/underworld/libUnderworld"


def dvc_suite(root):
    src = open(os.path.join(root, L, "PICellerator/Weights/tests/DVCWeightsSuite.c")).read()

    def grab(fn_name, comps):
        body = src[src.index(fn_name):]
        body = body[: body.index("\n}\n")]
        out = {}
        for c in comps:
            out[c] = [float(v) for v in re.findall(r"pList2?D?\[i\]\.%s\s*=\s*([-+0-9.eE]+)" % c, body)]
        return np.array([out[c] for c in comps]).T

    p3 = grab("void _DVCWeightsSuite_InitialiseParticleCoords(", "xyz")
    p2 = grab("void _DVCWeightsSuite_InitialiseParticleCoords2D(", "xy")

    def expected(name, dim):
        txt = open(os.path.join(root, L, "PICellerator/Weights/tests/expected", name)).read()
        cents = re.findall(r"centroids: \([^)]*\) = \(([^)]*)\)", txt)
        weights = re.findall(r"weight = ([-+0-9.eE]+)", txt)
        c = np.array([[float(v) for v in s.split(",")] for s in cents])
        return c[:, :dim], np.array([float(w) for w in weights])

    c3, w3 = expected("DVCWeightsSuite_testGetCentroids.txt", 3)
    c2, w2 = expected("DVCWeightsSuite_testGetCentroids2D.txt", 2)
    return {"res": 10,
            "particles_3d": p3.tolist(), "centroids_3d": c3.tolist(), "weights_3d": w3.tolist(),
            "particles_2d": p2.tolist(), "centroids_2d": c2.tolist(), "weights_2d": w2.tolist()}


def petsc_matrix(root):
    path = os.path.join(root, L, "StgFEM/Assembly/tests/expected/testIsoviscousSiffness.matrix")
    d = open(path, "rb").read()
    cid, m, n, nnz = struct.unpack(">4i", d[:16])
    assert cid == 1211216
    off = 16
    rl = np.frombuffer(d, ">i4", m, off); off += 4 * m
    cols = np.frombuffer(d, ">i4", nnz, off); off += 4 * nnz
    vals = np.frombuffer(d, ">f8", nnz, off)
    dense = np.zeros((m, n))
    k = 0
    for r in range(m):
        for _ in range(rl[r]):
            dense[r, cols[k]] += vals[k]
            k += 1
    return {"mesh": {"dim": 2, "res": [3, 3], "min": [0.0, 0.0], "max": [1.0, 1.0]},
            "eta": 1.0, "rows": m, "cols": n, "nnz": int(nnz), "dense": dense.tolist()}


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <root of the underworld2 source tree>")
    root = sys.argv[1]
    g = {
        "dvc_suite": dvc_suite(root),
        "isoviscous_K": petsc_matrix(root),
        # P/swarm/layouts.py:200-213 (PerCellRandomLayout docstring)
        "layout_seed13_1x1_ppc4": [[0.24261743, 0.67115852], [0.16116546, 0.70790335],
                                   [0.73160516, 0.08792286], [0.71953113, 0.15966135]],
        # P/systems/_timeintegration.py:132-148 (SwarmAdvector.integrate docstring)
        "rk2_9x9": {"start": [0.2, -0.2], "vel": [1.0, 1.0], "end": [0.27856742, -0.12143258]},
        # P/swarm/_swarm.py:629-639 (update_particle_owners docstring)
        "owner_16x16": {"point": [0.1, 0.1], "cell": 17},
    }
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
    with open(out, "w") as f:
        json.dump(g, f, indent=1)
    print("wrote", out)


if __name__ == "__main__":
    main()
