"""Every FP32 hex apply variant -- G tile staged by TMA (0) or loaded directly
(1), one element per lane (0, 1) or two elements per lane with packed f32x2
arithmetic (2, 3) -- forced through GH1_HEX_GMODE and checked against the FP64
oracle.  Odd element counts leave the last element pair half empty.  Variant 4
(one metric per element) exists only on meshes whose element maps are all affine,
and so does variant 5 (its slice / pencil form, orders 1-4).  Variant 6 runs the
1D contractions on the tensor cores (orders 4-7, either metric form)."""
import contextlib
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from ngsolve_gb300.meshes import MakeStructured3DMesh, JitterInterior, Mesh as RawMesh
from tests.util import lognormal

pytestmark = pytest.mark.gpu


@contextlib.contextmanager
def forced_variant(mode):
    saved = {k: os.environ.get(k) for k in ("GH1_HEX_GMODE", "GH1_HEX_TC")}
    os.environ["GH1_HEX_GMODE"] = str(mode)
    os.environ.pop("GH1_HEX_TC", None)  # the tensor-core variant on (its default)
    try:
        yield
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _form(gpu, fes, kappa, mu, mode):
    u, v = fes.TnT()
    a = gpu.BilinearForm(fes, nonassemble=True, precision="fp32")
    a += gpu.CoefficientFunction(kappa) * gpu.grad(u) * gpu.grad(v) * gpu.dx
    if mu is not None:
        a += gpu.CoefficientFunction(mu) * u * v * gpu.dx
    with forced_variant(mode):
        a.Assemble()
    return a


@pytest.mark.parametrize("mass", [False, True])
@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_fp32_variant_parity(gpu, mode, p, mass):
    """y = A x in FP32 within 2e-5 of the FP64 oracle's scale (27 and 8 elements)."""
    for nx in (3, 2):
        m = JitterInterior(MakeStructured3DMesh(hexes=True, nx=nx), 0.1 / nx, 11)
        kappa = lognormal(m.ne, 1.0, 5)
        mu = lognormal(m.ne, 0.5, 6) if mass else None
        fes = gpu.H1(m, order=p, dirichlet=".*")
        a = _form(gpu, fes, kappa, mu, mode)
        S = O.OracleSpace(m.points, m.elements, p)
        x = np.random.default_rng(7).normal(size=fes.ndof)
        yo = S.apply_mf(x, kappa=kappa, mu=mu)
        x32 = gpu.BaseVector(data=torch.tensor(x, dtype=torch.float32, device="cuda"))
        y32 = gpu.BaseVector(data=torch.zeros(fes.ndof, dtype=torch.float32, device="cuda"))
        a.mat.Mult(x32, y32)
        assert np.abs(y32.NumPy().astype(np.float64) - yo).max() <= 2e-5 * np.abs(yo).max()


def _renumbered(m, seed):
    """The same mesh with its vertices numbered in a random order: the edge and
    face orientations, which follow the global vertex numbers, then take every
    class (reversed edges; transposed and reflected faces)."""
    perm = np.random.default_rng(seed).permutation(len(m.points))
    pts = np.empty_like(m.points)
    pts[perm] = m.points
    return RawMesh(pts, perm[m.elements])


@pytest.mark.parametrize("mass", [False, True])
@pytest.mark.parametrize("p", [3, 4, 5, 6])
@pytest.mark.parametrize("mode", [2, 3])
def test_fp32_paired_all_orientations(gpu, mode, p, mass):
    """The paired kernels read every DOF and shape sign from the signed tensor
    table.  On jittered meshes with randomly renumbered vertices (all edge and
    face orientation classes; 27 and 8 elements) the apply is within 2e-5 of
    the oracle."""
    for nx in (3, 2):
        m = _renumbered(JitterInterior(MakeStructured3DMesh(hexes=True, nx=nx), 0.1 / nx, 11), 20 + nx)
        kappa = lognormal(m.ne, 1.0, 5)
        mu = lognormal(m.ne, 0.5, 6) if mass else None
        fes = gpu.H1(m, order=p, dirichlet=".*")
        a = _form(gpu, fes, kappa, mu, mode)
        assert a.mat.Info()["hex_variant_fp32"] == mode
        S = O.OracleSpace(m.points, m.elements, p)
        x = np.random.default_rng(7).normal(size=fes.ndof)
        yo = S.apply_mf(x, kappa=kappa, mu=mu)
        x32 = gpu.BaseVector(data=torch.tensor(x, dtype=torch.float32, device="cuda"))
        y32 = gpu.BaseVector(data=torch.zeros(fes.ndof, dtype=torch.float32, device="cuda"))
        a.mat.Mult(x32, y32)
        assert np.abs(y32.NumPy().astype(np.float64) - yo).max() <= 2e-5 * np.abs(yo).max()


def _sheared(nx):
    """Structured hexes under a general affine map: every element is the same
    parallelepiped, so the metric is one full symmetric 3x3 per element."""
    m = MakeStructured3DMesh(hexes=True, nx=nx)
    A = np.array([[1.0, 0.3, -0.2], [0.1, 0.8, 0.25], [-0.15, 0.2, 1.3]])
    return RawMesh(m.points @ A.T + np.array([0.5, -1.0, 2.0]), m.elements)


@pytest.mark.parametrize("mass", [False, True])
@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6])
def test_fp32_affine_variant(gpu, p, mass):
    """Variant 4 (one metric per element) on affine meshes (an axis-aligned and a
    sheared one, odd and even element counts) within 2e-5 of the oracle; on a
    jittered mesh the variant is not offered and the apply stays correct."""
    for m in (MakeStructured3DMesh(hexes=True, nx=3), _sheared(2), _sheared(3)):
        kappa = lognormal(m.ne, 1.0, 5)
        mu = lognormal(m.ne, 0.5, 6) if mass else None
        fes = gpu.H1(m, order=p, dirichlet=".*")
        a = _form(gpu, fes, kappa, mu, 4)
        if p <= 6:
            assert a.mat.Info()["hex_variant_fp32"] == 4
        S = O.OracleSpace(m.points, m.elements, p)
        x = np.random.default_rng(7).normal(size=fes.ndof)
        yo = S.apply_mf(x, kappa=kappa, mu=mu)
        x32 = gpu.BaseVector(data=torch.tensor(x, dtype=torch.float32, device="cuda"))
        y32 = gpu.BaseVector(data=torch.zeros(fes.ndof, dtype=torch.float32, device="cuda"))
        a.mat.Mult(x32, y32)
        assert np.abs(y32.NumPy().astype(np.float64) - yo).max() <= 2e-5 * np.abs(yo).max()
    m = JitterInterior(MakeStructured3DMesh(hexes=True, nx=3), 0.1 / 3, 11)
    fes = gpu.H1(m, order=p, dirichlet=".*")
    a = _form(gpu, fes, lognormal(m.ne, 1.0, 5), None, 4)
    assert a.mat.Info()["hex_variant_fp32"] in (0, 1, 2, 3)


@pytest.mark.parametrize("mass", [False, True])
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_fp32_slice_variant(gpu, p, mass):
    """Variant 5 (slice / pencil form, one metric per element) within 2e-5 of the
    oracle on affine meshes whose element counts leave the last warp chunk
    ragged (1, 8, 27, 64 and 125 elements against 2 * 32 / (p + 1) per chunk).
    Its fused energy x^T A x drives the mixed CG test below."""
    for m in (MakeStructured3DMesh(hexes=True, nx=1), _sheared(2), MakeStructured3DMesh(hexes=True, nx=3),
              _sheared(4), MakeStructured3DMesh(hexes=True, nx=5)):
        kappa = lognormal(m.ne, 1.0, 5)
        mu = lognormal(m.ne, 0.5, 6) if mass else None
        fes = gpu.H1(m, order=p, dirichlet=".*")
        a = _form(gpu, fes, kappa, mu, 5)
        assert a.mat.Info()["hex_variant_fp32"] == 5
        S = O.OracleSpace(m.points, m.elements, p)
        x = np.random.default_rng(7).normal(size=fes.ndof)
        yo = S.apply_mf(x, kappa=kappa, mu=mu)
        x32 = gpu.BaseVector(data=torch.tensor(x, dtype=torch.float32, device="cuda"))
        y32 = gpu.BaseVector(data=torch.zeros(fes.ndof, dtype=torch.float32, device="cuda"))
        a.mat.Mult(x32, y32)
        assert np.abs(y32.NumPy().astype(np.float64) - yo).max() <= 2e-5 * np.abs(yo).max()


@pytest.mark.parametrize("mode", [2, 3, 4, 5])
@pytest.mark.parametrize("p", [2, 4])
def test_mixed_cg_paired_variant(gpu, mode, p):
    """Mixed-precision CG whose inner FP32 iterations run the paired apply (with
    its fused energy x^T A x) reaches 1e-10 true relative residual and agrees
    with the FP64 CG solution."""
    m = _sheared(5) if mode >= 4 else JitterInterior(MakeStructured3DMesh(hexes=True, nx=5), 0.1 / 5, 3)
    kappa = lognormal(m.ne, 0.5, 14)
    f = np.random.default_rng(15).uniform(-1, 1, m.ne)
    fes = gpu.H1(m, order=p, dirichlet=".*")
    a = _form(gpu, fes, kappa, None, mode)
    u, v = fes.TnT()
    lf = gpu.LinearForm(fes)
    lf += gpu.CoefficientFunction(f) * v * gpu.dx
    lf.Assemble()
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    solm = gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=1e-11, maxsteps=20000, printrates=False,
                          mode="mixed", stop_rule="true")
    r = gpu.solvers.CG.last_solver.result
    assert r.status == 0 and r.true_relres <= 1e-11 and r.outer >= 1 and r.applies32 > 0
    xm = solm.NumPy().copy()
    sol6 = gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=1e-12, maxsteps=20000, printrates=False,
                          mode="fp64", stop_rule="true")
    x6 = sol6.NumPy()
    assert np.abs(xm - x6).max() <= 1e-8 * np.abs(x6).max()


@pytest.mark.parametrize("mass", [False, True])
@pytest.mark.parametrize("p", [4, 5, 6, 7])
def test_fp32_tensor_core_variant(gpu, p, mass):
    """Variant 6 (the 1D contractions as tcgen05 kind::tf32 GEMMs with the
    3xTF32 split, accumulated in FP32 in tensor memory) within 2e-5 of the
    oracle: on a jittered mesh (per-point metric) and on affine ones (one
    metric per element), with 27, 8 and 1 elements, so that the last tile of
    floor(128 / (p+1)^2) elements is ragged."""
    for m in (JitterInterior(MakeStructured3DMesh(hexes=True, nx=3), 0.1 / 3, 11), _sheared(2),
              MakeStructured3DMesh(hexes=True, nx=1)):
        kappa = lognormal(m.ne, 1.0, 5)
        mu = lognormal(m.ne, 0.5, 6) if mass else None
        fes = gpu.H1(m, order=p, dirichlet=".*")
        a = _form(gpu, fes, kappa, mu, 6)
        assert a.mat.Info()["hex_variant_fp32"] == 6
        S = O.OracleSpace(m.points, m.elements, p)
        x = np.random.default_rng(7).normal(size=fes.ndof)
        yo = S.apply_mf(x, kappa=kappa, mu=mu)
        x32 = gpu.BaseVector(data=torch.tensor(x, dtype=torch.float32, device="cuda"))
        y32 = gpu.BaseVector(data=torch.zeros(fes.ndof, dtype=torch.float32, device="cuda"))
        a.mat.Mult(x32, y32)
        assert np.abs(y32.NumPy().astype(np.float64) - yo).max() <= 2e-5 * np.abs(yo).max()


@pytest.mark.parametrize("affine", [False, True])
@pytest.mark.parametrize("p", [4, 5])
def test_mixed_cg_tensor_core_variant(gpu, p, affine):
    """Mixed-precision CG with the tensor-core apply (and its fused energy
    x^T A x) as the inner FP32 operator reaches 1e-11 true relative residual
    and agrees with the FP64 CG solution."""
    m = _sheared(5) if affine else JitterInterior(MakeStructured3DMesh(hexes=True, nx=5), 0.1 / 5, 3)
    kappa = lognormal(m.ne, 0.5, 14)
    f = np.random.default_rng(15).uniform(-1, 1, m.ne)
    fes = gpu.H1(m, order=p, dirichlet=".*")
    a = _form(gpu, fes, kappa, None, 6)
    assert a.mat.Info()["hex_variant_fp32"] == 6
    u, v = fes.TnT()
    lf = gpu.LinearForm(fes)
    lf += gpu.CoefficientFunction(f) * v * gpu.dx
    lf.Assemble()
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    solm = gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=1e-11, maxsteps=20000, printrates=False,
                          mode="mixed", stop_rule="true")
    r = gpu.solvers.CG.last_solver.result
    assert r.status == 0 and r.true_relres <= 1e-11 and r.outer >= 1 and r.applies32 > 0
    xm = solm.NumPy().copy()
    sol6 = gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=1e-12, maxsteps=20000, printrates=False,
                          mode="fp64", stop_rule="true")
    x6 = sol6.NumPy()
    assert np.abs(xm - x6).max() <= 1e-8 * np.abs(x6).max()
