"""Dirichlet conditions on named boundary regions, H1(mesh, dirichlet="left|top")
(the FESpace dirichlet regex, comp/fespace.cpp:440-516), against the oracle."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O
from ngsolve_gb300.meshes import MakeStructured3DMesh, JitterInterior
from tests.util import lognormal, assert_cg_history_close

pytestmark = pytest.mark.gpu


def _mesh(kind, n, jitter, seed=71):
    m = MakeStructured3DMesh(hexes=(kind == "hex"), nx=n)
    return JitterInterior(m, jitter / n, seed) if jitter else m


@pytest.mark.parametrize("kind,p,regex", [("hex", 3, "left|top"), ("hex", 1, "bottom"), ("tet", 2, "back|front"),
                                          ("tet", 4, "right")])
def test_region_freedofs(gpu, kind, p, regex):
    """FreeDofs equal the oracle's for the same faces, bit for bit."""
    m = _mesh(kind, 3, 0.1)
    fes = gpu.H1(m, order=p, dirichlet=regex)
    S = O.OracleSpace(m.points, m.elements, p, dirichlet_faces=m.BoundaryFaces(regex))
    free = np.asarray(fes.FreeDofs(), dtype=bool)
    assert np.array_equal(free, S.freedofs().astype(bool))
    assert fes.nfree == int(free.sum()) and 0 < fes.nfree < fes.ndof
    # a regex matching every side is the whole boundary, one matching none leaves all free
    whole = np.asarray(gpu.H1(m, order=p, dirichlet="back|left|front|right|bottom|top").FreeDofs(), dtype=bool)
    assert np.array_equal(whole, O.OracleSpace(m.points, m.elements, p).freedofs().astype(bool))
    assert np.asarray(gpu.H1(m, order=p, dirichlet="nothing").FreeDofs(), dtype=bool).all()


def test_region_face_arguments(gpu):
    """gh1_space_h1_bnd rejects a face that is not in the mesh, an interior face
    and out-of-range vertices; no face leaves every DOF free."""
    m = _mesh("hex", 2, 0.0)
    gm = gpu.Mesh(m)
    lib, h = gm.ctx.lib, ctypes.c_void_p()
    interior = np.ascontiguousarray(m.elements[:1, [4, 5, 6, 7]], dtype=np.int32)  # top face of element 0
    assert lib.gh1_space_h1_bnd(gm.h, 2, 1, interior.ctypes.data, ctypes.byref(h)) == 1
    assert b"interior" in lib.gh1_last_error(gm.ctx.h)
    absent = np.array([[0, 1, 2, 4]], dtype=np.int32)
    assert lib.gh1_space_h1_bnd(gm.h, 2, 1, absent.ctypes.data, ctypes.byref(h)) == 1
    bad = np.array([[0, 1, 2, 99]], dtype=np.int32)
    assert lib.gh1_space_h1_bnd(gm.h, 2, 1, bad.ctypes.data, ctypes.byref(h)) == 1
    assert lib.gh1_space_h1_bnd(gm.h, 2, 0, None, ctypes.byref(h)) == 0
    info = np.zeros(6, dtype=np.int64)
    assert lib.gh1_space_info(h, info.ctypes.data) == 0 and info[4] == info[0]
    assert lib.gh1_space_free(h) == 0


@pytest.mark.parametrize("kind,p,matfree", [("hex", 3, True), ("tet", 2, False)])
def test_region_cg(gpu, kind, p, matfree):
    """Poisson with Dirichlet on two sides and natural conditions elsewhere: FP64
    PCG follows the oracle's CG on its mask (iterations within one, residual
    history, solution 1e-9); the batched mixed solver, which takes the space's
    own free-DOF mask, reaches 1e-10 and the same solution (1e-7)."""
    m = _mesh(kind, 4, 0.1)
    kappa = lognormal(m.ne, 1.0, 72)
    f = np.random.default_rng(73).uniform(-1, 1, m.ne)
    regex = "left|bottom"
    fes = gpu.H1(m, order=p, dirichlet=regex)
    u, v = fes.TnT()
    a = gpu.BilinearForm(fes, nonassemble=matfree, precision="fp32" if matfree else "fp64")
    a += gpu.CoefficientFunction(kappa) * gpu.grad(u) * gpu.grad(v) * gpu.dx
    a.Assemble()
    lf = gpu.LinearForm(fes)
    lf += gpu.CoefficientFunction(f) * v * gpu.dx
    lf.Assemble()
    pre = gpu.Preconditioner(a)
    sol = gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=1e-10, maxsteps=5000, printrates=False)
    solver = gpu.solvers.CG.last_solver
    S = O.OracleSpace(m.points, m.elements, p, dirichlet_faces=m.BoundaryFaces(regex))
    orp, oci, ova = S.assemble(kappa=kappa)
    d = ova[[orp[i] + np.searchsorted(oci[orp[i]:orp[i + 1]], i) for i in range(S.ndof)]]
    inv = np.where(S.freedofs().astype(bool), 1.0 / d, 0.0)
    xo, its, hist = S.cg(S.rhs(f), inv, tol=1e-10, maxit=5000, csr=(orp, oci, ova))
    assert abs(solver.iterations - its) <= 1
    assert_cg_history_close(solver.residuals, hist)
    assert np.abs(sol.NumPy() - xo).max() <= 1e-9 * np.abs(xo).max()
    if matfree:
        B = lf.vec.t.clone().reshape(1, -1)
        batch = gpu.solvers.BatchCG([a], [1])
        X, = batch.Solve([B], tol=1e-10)
        assert batch.status == 0 and batch.results[0].true_relres <= 1e-10
        assert np.abs(X[0].cpu().numpy() - xo).max() <= 1e-7 * np.abs(xo).max()
