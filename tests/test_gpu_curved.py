"""Curved elements through a mesh deformation (Mesh.SetDeformation, the
reference's MeshAccess::SetDeformation with ALE element transformations):
operators, assembled matrices and load vectors on the deformed mesh against the
oracle with the same deformation field (hexes: the same Gauss rule; tets: the
per-point B^T D B path at the space's degree-2p rule, given to the oracle); an
affine deformation equals moving the vertices; the mixed-precision CG solves on
a curved mesh."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from ngsolve_gb300.meshes import MakeStructured3DMesh, JitterInterior, Mesh as RawMesh
from tests.util import lognormal, csr_rowscaled_close

pytestmark = pytest.mark.gpu


def _deformed(gpu, hexes, n, k, seed, amp=0.03):
    """A mesh with a deformation field of order k: random values (amp * h) on
    every DOF of VectorH1(order=k), a curved, still valid element map."""
    raw = MakeStructured3DMesh(hexes=hexes, nx=n)
    if not hexes:
        raw = JitterInterior(raw, 0.1 / n, seed)
    mesh = gpu.Mesh(raw)
    vfes = gpu.VectorH1(mesh, order=k)
    gf = gpu.GridFunction(vfes)
    d = np.random.default_rng(seed).uniform(-1, 1, vfes.ndof) * amp / n
    gf.vec.data = d
    mesh.SetDeformation(gf)
    Sd = O.OracleSpace(raw.points, raw.elements, k)
    return raw, mesh, vfes, gf, d, Sd


def _rule(gpu, fes):
    import ctypes
    from ngsolve_gb300 import _lib
    nq = ctypes.c_int()
    ctx = fes.ctx
    ctx.check(ctx.lib.gh1_space_qpoints(fes.h, None, None, _lib.GH1_MEM_HOST, ctypes.byref(nq)))
    ref = np.zeros((nq.value, 4))
    ctx.check(ctx.lib.gh1_space_qpoints(fes.h, ref.ctypes.data_as(ctypes.c_void_p), None, _lib.GH1_MEM_HOST, None))
    return ref


def _mult(gpu, mat, x, dtype=torch.float64):
    xv = gpu.BaseVector(data=torch.tensor(x, dtype=dtype, device="cuda"))
    yv = gpu.BaseVector(data=torch.zeros(len(x), dtype=dtype, device="cuda"))
    mat.Mult(xv, yv)
    return yv.NumPy().astype(np.float64)


@pytest.mark.parametrize("hexes,p,k", [(True, 2, 2), (True, 4, 2), (True, 3, 3), (False, 2, 2), (False, 3, 2),
                                       (False, 4, 3)])
def test_curved_operators(gpu, hexes, p, k):
    raw, mesh, vfes, gf, d, Sd = _deformed(gpu, hexes, 3, k, 80 + p)
    kappa = lognormal(raw.ne, 1.0, 81)
    mu = lognormal(raw.ne, 0.5, 82)
    fes = gpu.H1(mesh, order=p, dirichlet=".*")
    u, v = fes.TnT()
    integrand = gpu.CoefficientFunction(kappa) * gpu.grad(u) * gpu.grad(v) * gpu.dx + \
        gpu.CoefficientFunction(mu) * u * v * gpu.dx
    amf = gpu.BilinearForm(integrand, nonassemble=True, precision="fp32").Assemble()
    acsr = gpu.BilinearForm(integrand).Assemble()
    S = O.OracleSpace(raw.points, raw.elements, p)
    S.set_deformation(Sd, d)
    x = np.random.default_rng(83).normal(size=fes.ndof)
    f = np.random.default_rng(84).uniform(-1, 1, raw.ne)
    lf = gpu.LinearForm(gpu.CoefficientFunction(f) * v * gpu.dx).Assemble()
    if hexes:  # the oracle's rule is the GPU's (tensor Gauss, p+1 points)
        yo = S.apply_mf(x, kappa=kappa, mu=mu)
        orp, oci, ova = S.assemble(kappa=kappa, mu=mu)
        _, _, noise = S.assemble(kappa=kappa, mu=mu, reverse=True)
        csr_rowscaled_close(*acsr.mat.CSR(), orp, oci, ova, noise=noise)
        bo = S.rhs(f)
    else:  # curved tets: the B^T D B path at the space's degree-2p rule
        ref = _rule(gpu, fes)
        D = np.zeros((raw.ne, 4, 4))
        D[:, 0, 0] = mu
        D[:, 1, 1] = D[:, 2, 2] = D[:, 3, 3] = kappa
        Dp = np.repeat(D.reshape(raw.ne, 1, 16), len(ref), axis=1)
        yo = S.apply_bdb(x, Dp, rule=ref)
        rp, ci, va = acsr.mat.CSR()
        assert np.abs(O.spmv(rp, ci, va, x) - yo).max() <= 1e-12 * np.abs(yo).max()
        bo = S.rhs(f, rule=ref)
    sc = np.abs(yo).max()
    assert np.abs(_mult(gpu, amf.mat, x) - yo).max() <= 1e-12 * sc
    assert np.abs(_mult(gpu, amf.mat, x, torch.float32) - yo).max() <= 2e-5 * sc
    assert np.abs(lf.vec.NumPy() - bo).max() <= 1e-13 * np.abs(bo).max()
    # the deformation moves the elements: the operator differs from the flat one
    flat = O.OracleSpace(raw.points, raw.elements, p)
    assert np.abs(flat.apply_mf(x, kappa=kappa, mu=mu) - yo).max() > 1e-4 * sc


@pytest.mark.parametrize("hexes,p", [(True, 3), (False, 3)])
def test_affine_deformation_moves_the_vertices(gpu, hexes, p):
    """d = A x on the vertices (order 1) is the mesh with vertices X + A X: the
    same operator (1e-12), load vector and rule points."""
    raw = MakeStructured3DMesh(hexes=hexes, nx=3)
    A = np.array([[0.1, 0.05, 0.0], [-0.03, 0.2, 0.04], [0.02, 0.0, -0.1]])
    mesh = gpu.Mesh(raw)
    vfes = gpu.VectorH1(mesh, order=1)
    gf = gpu.GridFunction(vfes)
    disp = raw.points @ A.T
    gf.vec.data = np.concatenate([disp[:, 0], disp[:, 1], disp[:, 2]])
    mesh.SetDeformation(gf)
    moved = gpu.Mesh(RawMesh(raw.points + disp, raw.elements))
    kappa = lognormal(raw.ne, 1.0, 85)
    ys, bs = [], []
    x = np.random.default_rng(86).normal(size=gpu.H1(moved, order=p).ndof)
    f = np.random.default_rng(87).uniform(-1, 1, raw.ne)
    for m in (mesh, moved):
        fes = gpu.H1(m, order=p)
        u, v = fes.TnT()
        a = gpu.BilinearForm(gpu.CoefficientFunction(kappa) * gpu.grad(u) * gpu.grad(v) * gpu.dx + u * v * gpu.dx,
                             nonassemble=True).Assemble()
        ys.append(_mult(gpu, a.mat, x))
        bs.append(gpu.LinearForm(gpu.CoefficientFunction(f) * v * gpu.dx).Assemble().vec.NumPy())
    assert np.abs(ys[0] - ys[1]).max() <= 1e-12 * np.abs(ys[1]).max()
    assert np.abs(bs[0] - bs[1]).max() <= 1e-13 * np.abs(bs[1]).max()


def test_curved_mixed_cg(gpu):
    """The mixed-precision CG on a curved hex mesh reaches a true residual of
    1e-10; its solution solves the oracle's curved system to 1e-9."""
    raw, mesh, vfes, gf, d, Sd = _deformed(gpu, True, 4, 2, 88)
    fes = gpu.H1(mesh, order=3, dirichlet=".*")
    u, v = fes.TnT()
    a = gpu.BilinearForm(gpu.grad(u) * gpu.grad(v) * gpu.dx, nonassemble=True, precision="mixed").Assemble()
    f = np.random.default_rng(89).uniform(-1, 1, raw.ne)
    lf = gpu.LinearForm(gpu.CoefficientFunction(f) * v * gpu.dx).Assemble()
    inv = gpu.CGSolver(a.mat, a.mat.CreateSmoother(fes.FreeDofs()), tol=1e-10, maxsteps=5000, mode="mixed",
                       stop_rule="true")
    sol = gpu.GridFunction(fes)
    sol.vec.data = inv * lf.vec
    assert inv.result.status == 0 and inv.result.true_relres <= 1e-10
    S = O.OracleSpace(raw.points, raw.elements, 3)
    S.set_deformation(Sd, d)
    free = S.freedofs().astype(bool)
    r = S.rhs(f) - S.apply_mf(sol.vec.NumPy())
    b = S.rhs(f)
    assert np.linalg.norm(r[free]) <= 1e-9 * np.linalg.norm(b[free])
