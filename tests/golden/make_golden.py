"""Generate the golden fixtures of the parity tests from the NGSolve source tree.

Run where a checkout of the reference exists, giving its root:
    python tests/golden/make_golden.py /path/to/ngsolve
Writes
  cube_vol.npz   points + tet vertex lists of tests/pytest/cube.vol.gz (the
                 mesh of tests/pytest/test_matrix.py:84-93), 0-based, and its
                 surface elements: bnd_faces (0-based vertex triples),
                 bnd_index (index into bc_names), bc_names;
  golden.json    the known answers quoted from the reference tests.
The GPU tests read only these files, never the reference tree.
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from ngsolve_gb300.meshes import ReadVolMesh  # noqa: E402


def main(ref):
    mesh = ReadVolMesh(os.path.join(ref, "tests", "pytest", "cube.vol.gz"))
    faces, index = mesh._boundary()
    np.savez_compressed(os.path.join(HERE, "cube_vol.npz"), points=mesh.points, tets=mesh.elements,
                        bnd_faces=faces, bnd_index=index, bc_names=np.array(mesh.bc_names))
    # reference_values of test_sparsematrix_access (tests/pytest/test_matrix.py:58-62):
    # [0] P1 mass a.mat[1,1] on square.vol.gz, [2] the same on cube.vol.gz
    src = open(os.path.join(ref, "tests", "pytest", "test_matrix.py")).read()
    block = src[src.index("reference_values = ["):]
    block = block[:block.index("]") + 1]
    nums = re.findall(r"[-+]?\d*\.\d+(?:[eE][-+]?\d+)?", block)
    golden = {
        "p1_mass_cube_vertex1": {
            "value": float(nums[2]),
            "tolerance": 1e-8,
            "source": "tests/pytest/test_matrix.py:58-62,84-93 (H1 order 1, mass, a.mat[1,1] on cube.vol.gz)",
        },
        "counts": {
            "hex16_p3": {"ndof": 117649, "free": 103823, "nnz": 13997521},
            "kuhn32_p2": {"ndof": 274625, "nnz": 7678721},
            "source": "closed-form DOF counts of comp/h1hofespace.cpp:843-939 on MakeStructured3DMesh meshes",
        },
    }
    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump(golden, fh, indent=1)
    print("wrote cube_vol.npz (%d tets) and golden.json" % mesh.ne)


if __name__ == "__main__":
    if len(sys.argv) != 2 or not os.path.isdir(sys.argv[1]):
        sys.exit("usage: python tests/golden/make_golden.py /path/to/ngsolve (the reference source tree)")
    main(sys.argv[1])
