"""VectorH1 (comp/h1hofespace.cpp:2482-2700, component-major numbering): the
block operator diag(A, A, A) against the oracle, applied one block at a time
and solved as one block-diagonal CSR system."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O
from ngsolve_gb300.meshes import MakeStructured3DMesh, JitterInterior
from tests.util import lognormal, assert_cg_history_close

pytestmark = pytest.mark.gpu


def _mesh(kind, n, jitter, seed=21):
    m = MakeStructured3DMesh(hexes=(kind == "hex"), nx=n)
    return JitterInterior(m, jitter / n, seed) if jitter else m


def _block_csr(rp, ci, va, nblocks):
    n, nnz = len(rp) - 1, int(rp[-1])
    brp = np.concatenate([rp[:-1] + b * nnz for b in range(nblocks)] + [[nblocks * nnz]]).astype(rp.dtype)
    bci = np.concatenate([ci + b * n for b in range(nblocks)]).astype(ci.dtype)
    return brp, bci, np.tile(va, nblocks)


def _oracle_cg(csr, invdiag, b, tol, maxit):
    """orc_cg on an explicit CSR of any size (the space handle is unused there)."""
    rp, ci, va = (np.ascontiguousarray(a) for a in csr)
    b = np.ascontiguousarray(b, dtype=np.float64)
    invdiag = np.ascontiguousarray(invdiag, dtype=np.float64)
    x = np.zeros(len(b))
    hist = np.zeros(maxit + 2)
    its = np.zeros(1, dtype=np.int32)
    O.lib().orc_cg(None, len(b), O._p(rp), O._p(ci), O._p(va), None, None, O._p(invdiag), O._p(b), O._p(x),
                   tol, maxit, O._p(hist), O._p(its))
    return x, int(its[0]), hist[:int(its[0])].copy()


def _vector_form(gpu, fes, kappa, mu, matfree, precision="fp64"):
    u, v = fes.TnT()
    a = gpu.BilinearForm(fes, nonassemble=matfree, precision=precision)
    a += gpu.CoefficientFunction(kappa) * gpu.InnerProduct(gpu.grad(u), gpu.grad(v)) * gpu.dx
    if mu is not None:
        a += gpu.CoefficientFunction(mu) * gpu.InnerProduct(u, v) * gpu.dx
    return a.Assemble()


@pytest.mark.parametrize("kind,p,matfree,mass", [("hex", 3, True, True), ("hex", 2, False, False),
                                                 ("tet", 3, True, False), ("tet", 2, False, True)])
def test_vector_apply(gpu, kind, p, matfree, mass):
    """Block c of A_vec x is the scalar operator on block c of x, in FP64 and FP32."""
    m = _mesh(kind, 3, 0.1)
    kappa = lognormal(m.ne, 1.0, 31)
    mu = lognormal(m.ne, 0.5, 32) if mass else None
    fes = gpu.VectorH1(m, order=p, dirichlet=".*")
    a = _vector_form(gpu, fes, kappa, mu, matfree, precision="fp32" if matfree else "fp64")
    n = fes.scalar.ndof
    assert fes.ndof == 3 * n and isinstance(a.mat, gpu.BlockMatrix)
    info = a.mat.Info()
    assert info["kind"] == 2 and info["nrows"] == 3 * n
    S = O.OracleSpace(m.points, m.elements, p)
    x = np.random.default_rng(33).normal(size=3 * n)
    if matfree:
        yo = np.concatenate([S.apply_mf(x[c * n:(c + 1) * n], kappa=kappa, mu=mu) for c in range(3)])
    else:
        orp, oci, ova = S.assemble(kappa=kappa, mu=mu)
        yo = np.concatenate([O.spmv(orp, oci, ova, x[c * n:(c + 1) * n]) for c in range(3)])
    xv = gpu.BaseVector(3 * n)
    xv.data = x
    yv = gpu.BaseVector(3 * n)
    a.mat.Mult(xv, yv)
    sc = np.abs(yo).max()
    assert np.abs(yv.NumPy() - yo).max() <= 1e-12 * sc
    a.mat.MultAdd(-0.5, xv, yv)
    assert np.abs(yv.NumPy() - 0.5 * yo).max() <= 1e-12 * sc
    if matfree:
        x32 = gpu.BaseVector(data=torch.tensor(x, dtype=torch.float32, device="cuda"))
        y32 = gpu.BaseVector(data=torch.zeros(3 * n, dtype=torch.float32, device="cuda"))
        a.mat.Mult(x32, y32)
        assert np.abs(y32.NumPy().astype(np.float64) - yo).max() <= 2e-5 * sc


def test_vector_rhs_and_freedofs(gpu):
    m = _mesh("hex", 3, 0.1)
    f = np.random.default_rng(34).uniform(-1, 1, (3, m.ne))
    fes = gpu.VectorH1(m, order=2, dirichlet=".*")
    u, v = fes.TnT()
    lf = gpu.LinearForm(fes)
    lf += gpu.CoefficientFunction((f[0], f[1], f[2])) * v * gpu.dx
    lf += gpu.CoefficientFunction((0.0, 1.5, 0.0)) * v * gpu.dx
    lf.Assemble()
    S = O.OracleSpace(m.points, m.elements, 2)
    n = fes.scalar.ndof
    bo = np.concatenate([S.rhs(f[c] + (1.5 if c == 1 else 0.0)) for c in range(3)])
    assert np.abs(lf.vec.NumPy() - bo).max() <= 1e-13 * np.abs(bo).max()
    free = np.asarray(fes.FreeDofs(), dtype=bool)
    assert np.array_equal(free, np.tile(S.freedofs().astype(bool), 3))
    assert list(fes.Range(2)) == list(range(2 * n, 3 * n))
    with pytest.raises(ValueError):
        lf += gpu.CoefficientFunction(1.0) * v * gpu.dx


@pytest.mark.parametrize("kind,p,matfree", [("hex", 3, True), ("tet", 2, False)])
def test_vector_cg_fp64(gpu, kind, p, matfree):
    """FP64 Jacobi-PCG on the vector system follows the oracle's CG on the
    block-diagonal CSR: iteration count within one, residual history (to 1e-6
    above 1e-4 of the first residual), solution within 1e-9."""
    m = _mesh(kind, 4, 0.1)
    kappa = lognormal(m.ne, 1.0, 35)
    f = np.random.default_rng(36).uniform(-1, 1, (3, m.ne))
    fes = gpu.VectorH1(m, order=p, dirichlet=".*")
    a = _vector_form(gpu, fes, kappa, None, matfree)
    u, v = fes.TnT()
    lf = gpu.LinearForm(fes)
    lf += gpu.CoefficientFunction(tuple(f)) * v * gpu.dx
    lf.Assemble()
    pre = gpu.Preconditioner(a)
    sol = gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=1e-10, maxsteps=3000, printrates=False)
    solver = gpu.solvers.CG.last_solver
    S = O.OracleSpace(m.points, m.elements, p)
    orp, oci, ova = S.assemble(kappa=kappa)
    bcsr = _block_csr(orp, oci, ova, 3)
    diag = ova[[orp[i] + np.searchsorted(oci[orp[i]:orp[i + 1]], i) for i in range(len(orp) - 1)]]
    inv = np.where(np.tile(S.freedofs().astype(bool), 3), 1.0 / np.tile(diag, 3), 0.0)
    bo = np.concatenate([S.rhs(f[c]) for c in range(3)])
    xo, its, hist = _oracle_cg(bcsr, inv, bo, 1e-10, 3000)
    assert abs(solver.iterations - its) <= 1
    assert_cg_history_close(solver.residuals, hist)
    assert np.abs(sol.NumPy() - xo).max() <= 1e-9 * np.abs(xo).max()


def test_vector_cg_mixed(gpu):
    """FP32 inner CG with FP64 refinement on the hex vector system reaches a true
    relative residual of 1e-10."""
    m = _mesh("hex", 4, 0.1)
    kappa = lognormal(m.ne, 0.5, 37)
    f = np.random.default_rng(38).uniform(-1, 1, (3, m.ne))
    fes = gpu.VectorH1(m, order=4, dirichlet=".*")
    a = _vector_form(gpu, fes, kappa, None, True, precision="fp32")
    u, v = fes.TnT()
    lf = gpu.LinearForm(fes)
    lf += gpu.CoefficientFunction(tuple(f)) * v * gpu.dx
    lf.Assemble()
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=1e-10, maxsteps=20000, printrates=False,
                   mode="mixed", stop_rule="true")
    r = gpu.solvers.CG.last_solver.result
    assert r.status == 0 and r.true_relres <= 1e-10 and r.outer >= 1


def test_block_create_arguments(gpu):
    m = _mesh("hex", 2, 0.0)
    fes = gpu.H1(m, order=2)
    u, v = fes.TnT()
    a = gpu.BilinearForm(fes, nonassemble=True)
    a += gpu.grad(u) * gpu.grad(v) * gpu.dx
    a.Assemble()
    lib, h = fes.ctx.lib, ctypes.c_void_p()
    assert lib.gh1_op_block_create(a.mat.h, 0, ctypes.byref(h)) == 1
    assert lib.gh1_op_block_create(None, 3, ctypes.byref(h)) == 1
    assert lib.gh1_op_block_create(a.mat.h, 2, ctypes.byref(h)) == 0
    assert lib.gh1_op_block_create(h, 2, ctypes.byref(ctypes.c_void_p())) == 1  # no blocks of blocks
    assert lib.gh1_op_free(h) == 0


def test_vector_batch(gpu):
    """A VectorH1 form in the batched solver: its (nrhs, 3n) right-hand sides run
    as 3 * nrhs scalar ones beside a scalar problem; every component reaches a
    true relative residual of 1e-10 and matches the oracle's FP64 CG."""
    mv = _mesh("hex", 3, 0.1)
    kv = lognormal(mv.ne, 1.0, 41)
    fv = gpu.VectorH1(mv, order=3, dirichlet=".*")
    av = _vector_form(gpu, fv, kv, None, True, precision="fp32")
    ms = _mesh("hex", 4, 0.0)
    ks = lognormal(ms.ne, 1.0, 42)
    fs = gpu.H1(ms, order=2, dirichlet=".*")
    u, v = fs.TnT()
    as_ = gpu.BilinearForm(fs, nonassemble=True, precision="fp32")
    as_ += gpu.CoefficientFunction(ks) * gpu.grad(u) * gpu.grad(v) * gpu.dx
    as_.Assemble()
    rng = np.random.default_rng(43)
    Bv = torch.tensor(rng.uniform(-1, 1, (2, fv.ndof)), device="cuda")
    Bv *= torch.tensor(np.tile(np.asarray(fv.FreeDofs(), dtype=np.float64), (2, 1)), device="cuda")
    Bs = torch.tensor(rng.uniform(-1, 1, (1, fs.ndof)), device="cuda")
    solver = gpu.solvers.BatchCG([av, as_], [2, 1])
    Xv, Xs = solver.Solve([Bv, Bs], tol=1e-10)
    assert solver.status == 0 and len(solver.results) == 2 * 3 + 1
    assert all(r.status == 0 and r.true_relres <= 1e-10 for r in solver.results)
    n = fv.scalar.ndof
    S = O.OracleSpace(mv.points, mv.elements, 3)
    rp, ci, va = S.assemble(kappa=kv)
    d = va[[rp[i] + np.searchsorted(ci[rp[i]:rp[i + 1]], i) for i in range(n)]]
    free = S.freedofs().astype(bool)
    inv = np.where(free, 1.0 / d, 0.0)
    for r in range(2):
        yv = gpu.BaseVector(fv.ndof)
        av.mat.Mult(gpu.BaseVector(data=Xv[r].clone()), yv)
        for c in range(3):
            sl = slice(c * n, (c + 1) * n)
            b = Bv[r, sl].cpu().numpy()
            res = np.linalg.norm((b - yv.NumPy()[sl])[free]) / np.linalg.norm(b[free])
            assert res <= 1.2e-10
            xo, _, _ = S.cg(b, inv, tol=1e-13, maxit=20000, csr=(rp, ci, va))
            assert np.abs(Xv[r, sl].cpu().numpy() - xo).max() <= 1e-7 * np.abs(xo).max()
