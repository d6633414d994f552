"""The Python front end's compositions on the GPU, each against an exact answer
on the unit cube (the same compositions run with host stand-ins in
tests/test_frontend.py):

- Integrate(x * gfu) with gfu.Set(1) is int x = 1/2, and Integrate(gfx * gfx)
  with gfx.Set(x) is int x^2 = 1/3: totals a^T M b through the matrix-free mass
  operator, exact because x lies in the space;
- LinearForm(x * v * dx) is M I_h(x), so its total against the constant 1 is
  again 1/2;
- Set(x, BND) then a.mat.Inverse(FreeDofs()) on the residual with f = 0 gives
  the discrete harmonic extension of the boundary data, which is I_h(x)
  itself (x is harmonic and in the space);
- CGSolver used as an operator (inv * f) matches solvers.CG.
"""
import numpy as np
import pytest
import torch

from ngsolve_gb300.meshes import MakeStructured3DMesh, JitterInterior

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("hexes,order", [(True, 1), (True, 3), (False, 2)])
def test_integrate_set_and_sources(gpu, hexes, order):
    mesh = gpu.Mesh(JitterInterior(MakeStructured3DMesh(hexes=hexes, nx=3), 0.1 / 3, 5) if not hexes
                    else MakeStructured3DMesh(hexes=True, nx=3))
    fes = gpu.H1(mesh, order=order, dirichlet=".*")
    one = gpu.GridFunction(fes)
    one.Set(1)
    assert abs(gpu.Integrate(gpu.x * one, mesh) - 0.5) < 1e-12
    gfx = gpu.GridFunction(fes)
    gfx.Set(gpu.x)
    assert abs(gpu.Integrate(gfx * gfx, mesh) - 1.0 / 3.0) < 1e-12
    assert abs(gpu.Integrate(gfx, mesh) - 0.5) < 1e-12
    u, v = fes.TnT()
    lf = gpu.LinearForm(gpu.x * v * gpu.dx).Assemble()
    assert abs(float(lf.vec.t @ one.vec.t) - 0.5) < 1e-12


@pytest.mark.parametrize("hexes,order", [(True, 2), (False, 3)])
def test_set_bnd_and_inverse_reproduce_harmonic_data(gpu, hexes, order):
    raw = MakeStructured3DMesh(hexes=hexes, nx=3)
    if not hexes:
        raw = JitterInterior(raw, 0.1 / 3, 7)
    mesh = gpu.Mesh(raw)
    fes = gpu.H1(mesh, order=order, dirichlet=".*")
    u, v = fes.TnT()
    a = gpu.BilinearForm(gpu.grad(u) * gpu.grad(v) * gpu.dx).Assemble()
    gfu = gpu.GridFunction(fes)
    gfu.Set(gpu.x + 2 * gpu.y - gpu.z, gpu.BND)
    res = gfu.vec.CreateVector()
    res.data = -1.0 * (a.mat * gfu.vec)
    gfu.vec.data += a.mat.Inverse(fes.FreeDofs()) * res
    exact = gpu.GridFunction(fes)
    exact.Set(gpu.x + 2 * gpu.y - gpu.z)
    assert np.abs(gfu.vec.NumPy() - exact.vec.NumPy()).max() < 1e-9


def test_cgsolver_as_operator(gpu):
    mesh = gpu.Mesh(MakeStructured3DMesh(hexes=True, nx=4))
    fes = gpu.H1(mesh, order=3, dirichlet=".*")
    u, v = fes.TnT()
    a = gpu.BilinearForm(gpu.grad(u) * gpu.grad(v) * gpu.dx, nonassemble=True).Assemble()
    f = gpu.LinearForm(gpu.CoefficientFunction(np.random.default_rng(3).uniform(-1, 1, mesh.ne)) * v * gpu.dx)
    f.Assemble()
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    inv = gpu.CGSolver(a.mat, pre, maxiter=2000, tol=1e-12)
    gfu = gpu.GridFunction(fes)
    gfu.vec.data = inv * f.vec
    assert inv.GetSteps() > 0
    ref = gpu.solvers.CG(mat=a.mat, rhs=f.vec, pre=pre, tol=1e-12, maxsteps=2000, printrates=False)
    # the two solves differ only in the order of the apply's atomic additions
    assert gpu.Norm(gfu.vec - ref) <= 1e-9 * gpu.Norm(ref)
