"""Projector(mask, range) (linalg/diagonalmatrix.cpp:13-110) on the GPU against
the reference's definition restated with numpy: Mult keeps the entries whose mask
bit equals range, MultAdd adds s times them, Project zeroes the others in place."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("rng_flag", [True, False])
def test_projector(gpu, dtype, rng_flag):
    n = 10007
    rng = np.random.default_rng(3)
    mask = rng.random(n) < 0.3
    x = rng.normal(size=n)
    y0 = rng.normal(size=n)
    keep = mask if rng_flag else ~mask
    P = gpu.Projector(mask, rng_flag)
    xv = gpu.BaseVector(data=torch.tensor(x, dtype=dtype, device="cuda"))
    yv = gpu.BaseVector(data=torch.tensor(y0, dtype=dtype, device="cuda"))
    tol = 0 if dtype == torch.float64 else 1e-6
    P.Mult(xv, yv)
    assert np.allclose(yv.NumPy(), np.where(keep, x, 0.0), rtol=tol, atol=tol)
    yv.t.copy_(torch.tensor(y0, dtype=dtype))
    P.MultAdd(-0.5, xv, yv)
    assert np.allclose(yv.NumPy(), y0 + np.where(keep, -0.5 * x, 0.0), rtol=tol, atol=tol)
    P.Project(xv)
    assert np.allclose(xv.NumPy(), np.where(keep, x, 0.0), rtol=tol, atol=tol)


def test_projector_freedofs(gpu):
    """Projector(fes.FreeDofs(), True) applied to a residual zeroes the Dirichlet DOFs."""
    m = gpu.MakeStructured3DMesh(hexes=True, nx=3)
    fes = gpu.H1(m, order=2, dirichlet=".*")
    free = fes.FreeDofs()
    P = gpu.Projector(free, True)
    v = gpu.BaseVector(data=torch.ones(fes.ndof, dtype=torch.float64, device="cuda"))
    P.Project(v)
    assert np.array_equal(v.NumPy() != 0, np.asarray(free, dtype=bool))
