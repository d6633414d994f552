"""The CSR pattern built on the GPU equals the host MatrixGraph build
(GH1_GRAPH=host) and the oracle's, on hex and tet meshes of several orders."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from ngsolve_gb300.meshes import MakeStructured3DMesh, JitterInterior, Mesh as RawMesh
from tests.util import permute_tets

pytestmark = pytest.mark.gpu


def _pattern(gpu, m, p, host):
    old = os.environ.get("GH1_GRAPH")
    if host:
        os.environ["GH1_GRAPH"] = "host"
    else:
        os.environ.pop("GH1_GRAPH", None)
    try:
        fes = gpu.H1(m, order=p, dirichlet=".*")
        u, v = fes.TnT()
        a = gpu.BilinearForm(fes)
        a += gpu.grad(u) * gpu.grad(v) * gpu.dx
        a.Assemble()
        rp, ci, _ = a.mat.CSR()
        return np.asarray(rp), np.asarray(ci)
    finally:
        if old is None:
            os.environ.pop("GH1_GRAPH", None)
        else:
            os.environ["GH1_GRAPH"] = old


@pytest.mark.parametrize("kind,n,p", [("hex", 3, 1), ("hex", 3, 3), ("hex", 2, 5), ("tet", 3, 2), ("tet", 2, 4),
                                      ("tet", 3, 1)])
def test_gpu_graph_matches_host_and_oracle(gpu, kind, n, p):
    m = MakeStructured3DMesh(hexes=(kind == "hex"), nx=n)
    if kind == "tet":
        m = JitterInterior(m, 0.1 / n, 4)
        m = RawMesh(m.points, permute_tets(m.elements, 5))
    rg, cg = _pattern(gpu, m, p, host=False)
    rh, ch = _pattern(gpu, m, p, host=True)
    assert np.array_equal(rg, rh) and np.array_equal(cg, ch)
    orp, oci = O.OracleSpace(m.points, m.elements, p).graph()
    assert np.array_equal(rg, orp) and np.array_equal(cg, oci)
