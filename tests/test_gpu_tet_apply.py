"""Matrix-free tet apply: the class-tiled GEMM kernel (whole class table in
shared memory for p <= 4, streamed in 16-point chunks for the large rules of
p = 5, 6) and the element-wise kernel (GH1_TET_KERNEL=elementwise) against the
FP64 oracle, FP64 and FP32, with and without the mass term; tiles straddle no
class boundary, so meshes with many classes and partially filled tiles are used."""
import contextlib
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from ngsolve_gb300.meshes import MakeStructured3DMesh, JitterInterior, Mesh as RawMesh
from tests.util import lognormal, permute_tets

pytestmark = pytest.mark.gpu


@contextlib.contextmanager
def tet_kernel(name):
    old = os.environ.get("GH1_TET_KERNEL")
    if name is None:
        os.environ.pop("GH1_TET_KERNEL", None)
    else:
        os.environ["GH1_TET_KERNEL"] = name
    try:
        yield
    finally:
        if old is None:
            os.environ.pop("GH1_TET_KERNEL", None)
        else:
            os.environ["GH1_TET_KERNEL"] = old


def _mesh(n, seed):
    m = JitterInterior(MakeStructured3DMesh(hexes=False, nx=n), 0.2 / n, seed)
    return RawMesh(m.points, permute_tets(m.elements, seed + 1))  # all 24 orientation classes


def _form(gpu, fes, kappa, mu, kernel):
    u, v = fes.TnT()
    a = gpu.BilinearForm(fes, nonassemble=True, precision="fp32")
    a += gpu.CoefficientFunction(kappa) * gpu.grad(u) * gpu.grad(v) * gpu.dx
    if mu is not None:
        a += gpu.CoefficientFunction(mu) * u * v * gpu.dx
    with tet_kernel(kernel):
        a.Assemble()
    return a


@pytest.mark.parametrize("kernel", [None, "elementwise"])
@pytest.mark.parametrize("mass", [False, True])
@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6, 7, 8])
def test_tet_apply_parity(gpu, p, mass, kernel):
    if kernel == "elementwise" and (p >= 6 or (mass and p >= 5)):
        pytest.skip("the element-wise kernel supports rules up to 128 points (p=5 mass: 343, p=6: 343)")
    if p >= 7 and mass and kernel is None:
        pytest.skip("p = 7, 8 run without the mass term here; the B^T D B tests cover reaction at p = 7")
    m = _mesh(3, 21 + p)
    kappa = lognormal(m.ne, 1.0, 5)
    mu = lognormal(m.ne, 0.5, 6) if mass else None
    fes = gpu.H1(m, order=p, dirichlet=".*")
    a = _form(gpu, fes, kappa, mu, kernel)
    S = O.OracleSpace(m.points, m.elements, p)
    x = np.random.default_rng(7).normal(size=fes.ndof)
    yo = S.apply_mf(x, kappa=kappa, mu=mu)
    sc = np.abs(yo).max()
    xv = gpu.BaseVector(fes.ndof)
    xv.data = x
    yv = gpu.BaseVector(fes.ndof)
    a.mat.Mult(xv, yv)
    assert np.abs(yv.NumPy() - yo).max() <= 1e-12 * sc
    x32 = gpu.BaseVector(data=torch.tensor(x, dtype=torch.float32, device="cuda"))
    y32 = gpu.BaseVector(data=torch.zeros(fes.ndof, dtype=torch.float32, device="cuda"))
    a.mat.Mult(x32, y32)
    assert np.abs(y32.NumPy().astype(np.float64) - yo).max() <= 2e-5 * sc


@pytest.mark.parametrize("p", [2, 4])
def test_tet_mixed_cg_tiled(gpu, p):
    """Mixed CG on tets (inner FP32 applies with the fused energy) reaches 1e-11
    and matches the FP64 solution."""
    m = _mesh(4, 3)
    kappa = lognormal(m.ne, 0.5, 14)
    f = np.random.default_rng(15).uniform(-1, 1, m.ne)
    fes = gpu.H1(m, order=p, dirichlet=".*")
    a = _form(gpu, fes, kappa, None, None)
    u, v = fes.TnT()
    lf = gpu.LinearForm(fes)
    lf += gpu.CoefficientFunction(f) * v * gpu.dx
    lf.Assemble()
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    solm = gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=1e-11, maxsteps=20000, printrates=False,
                          mode="mixed", stop_rule="true")
    r = gpu.solvers.CG.last_solver.result
    assert r.status == 0 and r.true_relres <= 1e-11 and r.applies32 > 0
    xm = solm.NumPy().copy()
    sol6 = gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=1e-12, maxsteps=20000, printrates=False,
                          mode="fp64", stop_rule="true")
    x6 = sol6.NumPy()
    assert np.abs(xm - x6).max() <= 1e-8 * np.abs(x6).max()


@pytest.mark.parametrize("p", [2, 3, 4])
def test_tet_tensor_core_apply(gpu, p):
    """The FP32 apply with both products of a same-class tile of up to 128
    elements on the tensor cores (tcgen05 kind::tf32, 3xTF32 split; forced with
    GH1_TET_KERNEL=tc) within 2e-5 of the oracle, on meshes whose classes fill
    from a fraction of a tile (162 tets) to several tiles (3,072 tets); the FP64
    apply of the same operator is unchanged.  With a mass term the tile kernel
    runs instead."""
    for n in (3, 8):
        m = _mesh(n, 31 + p)
        kappa = lognormal(m.ne, 1.0, 5)
        fes = gpu.H1(m, order=p, dirichlet=".*")
        a = _form(gpu, fes, kappa, None, "tc")
        assert a.mat.Info()["hex_variant_fp32"] == 6
        S = O.OracleSpace(m.points, m.elements, p)
        x = np.random.default_rng(7).normal(size=fes.ndof)
        yo = S.apply_mf(x, kappa=kappa)
        sc = np.abs(yo).max()
        x32 = gpu.BaseVector(data=torch.tensor(x, dtype=torch.float32, device="cuda"))
        y32 = gpu.BaseVector(data=torch.zeros(fes.ndof, dtype=torch.float32, device="cuda"))
        a.mat.Mult(x32, y32)
        assert np.abs(y32.NumPy().astype(np.float64) - yo).max() <= 2e-5 * sc
        xv, yv = gpu.BaseVector(fes.ndof), gpu.BaseVector(fes.ndof)
        xv.data = x
        a.mat.Mult(xv, yv)
        assert np.abs(yv.NumPy() - yo).max() <= 1e-12 * sc
    b = _form(gpu, fes, kappa, lognormal(m.ne, 0.5, 6), "tc")
    assert b.mat.Info()["hex_variant_fp32"] != 6


@pytest.mark.parametrize("p", [2, 3, 4])
def test_tet_tensor_core_with_mass(gpu, monkeypatch, p):
    """kappa grad.grad + mu u v in FP32 on the tensor cores (the B^T D B kernel on
    the records diag(mu, kappa) with the degree-2p rule; GH1_TET_BDB_TC=1,
    variant 10) within 2e-5 of the oracle on meshes with all 24 orientation
    classes; the FP64 apply of the same operator stays on the tiles (1e-12)."""
    monkeypatch.setenv("GH1_TET_BDB_TC", "1")
    for n in (3, 8):
        m = _mesh(n, 51 + p)
        kappa, mu = lognormal(m.ne, 1.0, 5), lognormal(m.ne, 0.5, 6)
        fes = gpu.H1(m, order=p, dirichlet=".*")
        a = _form(gpu, fes, kappa, mu, None)
        assert a.mat.Info()["hex_variant_fp32"] == 10
        S = O.OracleSpace(m.points, m.elements, p)
        x = np.random.default_rng(7).normal(size=fes.ndof)
        yo = S.apply_mf(x, kappa=kappa, mu=mu)
        sc = np.abs(yo).max()
        x32 = gpu.BaseVector(data=torch.tensor(x, dtype=torch.float32, device="cuda"))
        y32 = gpu.BaseVector(data=torch.zeros(fes.ndof, dtype=torch.float32, device="cuda"))
        a.mat.Mult(x32, y32)
        assert np.abs(y32.NumPy().astype(np.float64) - yo).max() <= 2e-5 * sc
        xv, yv = gpu.BaseVector(fes.ndof), gpu.BaseVector(fes.ndof)
        xv.data = x
        a.mat.Mult(xv, yv)
        assert np.abs(yv.NumPy() - yo).max() <= 1e-12 * sc


@pytest.mark.parametrize("p", [2, 4])
def test_tet_tensor_core_coefficient_update(gpu, p):
    """The tensor-core tet apply keeps its metric tile-major; a new kappa set on
    the form (gh1_form_set_coefs) rebuilds it before the next apply, which then
    matches the oracle with the new coefficient (FP32 2e-5)."""
    from ngsolve_gb300 import _lib
    m = _mesh(6, 40 + p)
    k1, k2 = lognormal(m.ne, 1.0, 5), lognormal(m.ne, 1.0, 6)
    fes = gpu.H1(m, order=p, dirichlet=".*")
    a = _form(gpu, fes, k1, None, "tc")
    assert a.mat.Info()["hex_variant_fp32"] == 6
    S = O.OracleSpace(m.points, m.elements, p)
    x = np.random.default_rng(7).normal(size=fes.ndof)
    x32 = gpu.BaseVector(data=torch.tensor(x, dtype=torch.float32, device="cuda"))
    for kappa in (k1, k2):
        if kappa is k2:
            kk = np.ascontiguousarray(k2, dtype=np.float64)
            fes.ctx.check(fes.ctx.lib.gh1_form_set_coefs(a._form, kk.ctypes.data, None, _lib.GH1_MEM_HOST))
        yo = S.apply_mf(x, kappa=kappa)
        y32 = gpu.BaseVector(data=torch.zeros(fes.ndof, dtype=torch.float32, device="cuda"))
        with tet_kernel("tc"):  # the rebuild keeps the tensor-core kernel
            a.mat.Mult(x32, y32)
        assert a.mat.Info()["hex_variant_fp32"] == 6
        assert np.abs(y32.NumPy().astype(np.float64) - yo).max() <= 2e-5 * np.abs(yo).max()


def test_tet_mixed_cg_tensor_core(gpu):
    """Mixed CG whose inner FP32 applies run on the tensor cores (with the fused
    energy x^T A x) reaches 1e-11 and matches the FP64 solution."""
    m = _mesh(5, 3)
    kappa = lognormal(m.ne, 0.5, 14)
    f = np.random.default_rng(15).uniform(-1, 1, m.ne)
    fes = gpu.H1(m, order=3, dirichlet=".*")
    a = _form(gpu, fes, kappa, None, "tc")
    assert a.mat.Info()["hex_variant_fp32"] == 6
    u, v = fes.TnT()
    lf = gpu.LinearForm(fes)
    lf += gpu.CoefficientFunction(f) * v * gpu.dx
    lf.Assemble()
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    solm = gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=1e-11, maxsteps=20000, printrates=False,
                          mode="mixed", stop_rule="true")
    r = gpu.solvers.CG.last_solver.result
    assert r.status == 0 and r.true_relres <= 1e-11 and r.applies32 > 0
    xm = solm.NumPy().copy()
    sol6 = gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=1e-12, maxsteps=20000, printrates=False,
                          mode="fp64", stop_rule="true")
    assert np.abs(xm - sol6.NumPy()).max() <= 1e-8 * np.abs(sol6.NumPy()).max()
