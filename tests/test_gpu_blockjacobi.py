"""The additive Schwarz preconditioner of the reference's CUDA tutorial,
jac + loemb @ loinv @ loemb.T: the smoothing blocks (CreateSmoothingBlocks)
against the oracle's restatement, the block-Jacobi apply and the exact
low-order solve against dense inverses of the oracle's matrices (numpy), and
PCG with the sum against the same PCG (krylovspace.py's recurrences) in numpy."""
import numpy as np
import pytest
import scipy.sparse as sps
import torch

from oracle import oracle as O
from ngsolve_gb300.meshes import MakeStructured3DMesh, JitterInterior
from tests.util import lognormal

pytestmark = pytest.mark.gpu


def _problem(gpu, hexes, p, n=3, jit=0.1, mass=True):
    raw = MakeStructured3DMesh(hexes=hexes, nx=n)
    if jit:
        raw = JitterInterior(raw, jit / n, 71)
    kappa = lognormal(raw.ne, 1.0, 72)
    mu = lognormal(raw.ne, 0.5, 73) if mass else None
    fes = gpu.H1(gpu.Mesh(raw), order=p, dirichlet=".*")
    u, v = fes.TnT()
    a = gpu.BilinearForm(fes)
    a += gpu.CoefficientFunction(kappa) * gpu.grad(u) * gpu.grad(v) * gpu.dx
    if mass:
        a += gpu.CoefficientFunction(mu) * u * v * gpu.dx
    a.Assemble()
    S = O.OracleSpace(raw.points, raw.elements, p)
    rp, ci, va = S.assemble(kappa=kappa, mu=mu)
    A = sps.csr_matrix((va, ci, rp), shape=(S.ndof, S.ndof))
    S1 = O.OracleSpace(raw.points, raw.elements, 1)
    rp1, ci1, va1 = S1.assemble(kappa=kappa, mu=mu)
    A1 = sps.csr_matrix((va1, ci1, rp1), shape=(S1.ndof, S1.ndof))
    return raw, fes, a, S, A, S1, A1


def _vec(gpu, x, dtype=torch.float64):
    return gpu.BaseVector(data=torch.tensor(x, dtype=dtype, device="cuda"))


def _mult(gpu, op, x, dtype=torch.float64):
    y = _vec(gpu, np.zeros(len(x)), dtype)
    op.Mult(_vec(gpu, x, dtype), y)
    return y.NumPy().astype(np.float64)


def _schwarz_dense(A, off, dofs, A1, free1):
    """sum_b E_b A_b^{-1} E_b^T + P A1_ff^{-1} P^T as a dense matrix."""
    n = A.shape[0]
    Ad = A.toarray()
    C = np.zeros((n, n))
    for b in range(len(off) - 1):
        d = dofs[off[b]:off[b + 1]]
        C[np.ix_(d, d)] += np.linalg.inv(Ad[np.ix_(d, d)])
    f = np.flatnonzero(free1)
    C[np.ix_(f, f)] += np.linalg.inv(A1.toarray()[np.ix_(f, f)])
    return C


@pytest.mark.parametrize("hexes,p,bt", [(True, 1, 4), (True, 3, 4), (True, 2, 3), (False, 2, 4), (False, 4, 4),
                                        (False, 3, 3)])
def test_smoothing_blocks(gpu, hexes, p, bt):
    raw = MakeStructured3DMesh(hexes=hexes, nx=3)
    fes = gpu.H1(gpu.Mesh(raw), order=p, dirichlet="left|top")
    S = O.OracleSpace(raw.points, raw.elements, p, dirichlet_faces=raw.BoundaryFaces("left|top"))
    blocks = fes.CreateSmoothingBlocks(blocktype=bt)
    off, dofs = S.smoothing_blocks(bt)
    assert np.array_equal(blocks.offsets, off) and np.array_equal(blocks.dofs, dofs)
    free = np.asarray(fes.FreeDofs(), dtype=bool)
    assert np.all(free[blocks.dofs]) and set(blocks.dofs.tolist()) == set(np.flatnonzero(free).tolist())


@pytest.mark.parametrize("hexes,p", [(True, 2), (True, 4), (False, 3)])
def test_block_jacobi_and_low_order_solve(gpu, hexes, p):
    """FP64 within 1e-12 of the dense numpy inverses, FP32 within 1e-4."""
    raw, fes, a, S, A, S1, A1 = _problem(gpu, hexes, p)
    blocks = fes.CreateSmoothingBlocks()
    jac = a.mat.CreateBlockSmoother(blocks)
    x = np.random.default_rng(74).normal(size=fes.ndof)
    Ad = A.toarray()
    yb = np.zeros(fes.ndof)
    for b in range(len(blocks)):
        d = blocks.dofs[blocks.offsets[b]:blocks.offsets[b + 1]]
        yb[d] += np.linalg.solve(Ad[np.ix_(d, d)], x[d])
    assert np.abs(_mult(gpu, jac, x) - yb).max() <= 1e-12 * np.abs(yb).max()
    assert np.abs(_mult(gpu, jac, x, torch.float32) - yb).max() <= 1e-4 * np.abs(yb).max()
    lospace = fes.lospace
    free1 = np.asarray(lospace.FreeDofs(), dtype=bool)
    loinv = a.loform.mat.Inverse(inverse="sparsecholesky", freedofs=lospace.FreeDofs())
    loemb = fes.loembedding
    coarse = loemb @ loinv @ loemb.T
    f = np.flatnonzero(free1)
    yc = np.zeros(fes.ndof)
    yc[f] = np.linalg.solve(A1.toarray()[np.ix_(f, f)], x[f])
    assert np.abs(_mult(gpu, coarse, x) - yc).max() <= 1e-10 * np.abs(yc).max()
    pre = jac + coarse
    assert np.abs(_mult(gpu, pre, x) - (yb + yc)).max() <= 1e-10 * np.abs(yb + yc).max()


def _numpy_pcg(A, C, b, free, tol, maxit):
    """krylovspace.py CGSolver._SolveImpl with the preconditioner C (dense)."""
    x = np.zeros_like(b)
    d = b.copy()
    w = C @ d
    s = w.copy()
    wdn = w @ d
    err0 = np.sqrt(abs(wdn))
    hist = [err0]
    it = 0
    while it < maxit:
        y = A @ s
        wd = wdn
        alpha = wd / (s @ y)
        x += alpha * s
        d -= alpha * y
        w = C @ d
        wdn = w @ d
        err = np.sqrt(abs(wdn))
        it += 1
        hist.append(err)
        if err < tol * err0:
            break
        s = w + (wdn / wd) * s
    return x, it, hist


@pytest.mark.parametrize("hexes,p", [(True, 3), (False, 2)])
def test_schwarz_pcg(gpu, hexes, p):
    """CG with jac + loemb @ loinv @ loemb.T follows the numpy PCG with the same
    preconditioner (iterations +-1, solution 1e-8); the mixed-precision solve
    with it reaches a true residual of 1e-10."""
    raw, fes, a, S, A, S1, A1 = _problem(gpu, hexes, p, n=4)
    blocks = fes.CreateSmoothingBlocks()
    jac = a.mat.CreateBlockSmoother(blocks)
    lospace = fes.lospace
    loinv = a.loform.mat.Inverse(inverse="sparsecholesky", freedofs=lospace.FreeDofs())
    pre = jac + fes.loembedding @ loinv @ fes.loembedding.T
    f = np.random.default_rng(75).uniform(-1, 1, raw.ne)
    lf = gpu.LinearForm(gpu.CoefficientFunction(f) * fes.TestFunction() * gpu.dx).Assemble()
    inv = gpu.CGSolver(a.mat, pre, tol=1e-10, maxsteps=2000)
    sol = gpu.GridFunction(fes)
    sol.vec.data = inv * lf.vec
    C = _schwarz_dense(A, blocks.offsets, blocks.dofs, A1, np.asarray(lospace.FreeDofs(), dtype=bool))
    b = S.rhs(f)
    free = S.freedofs().astype(bool)
    b[~free] = 0.0
    xo, its, _ = _numpy_pcg(A, C, b, free, 1e-10, 2000)
    assert abs(inv.GetSteps() - its) <= 1
    assert np.abs(sol.vec.NumPy() - xo).max() <= 1e-8 * np.abs(xo).max()
    mixed = gpu.CGSolver(a.mat, pre, tol=1e-10, maxsteps=2000, mode="mixed", stop_rule="true")
    solm = gpu.GridFunction(fes)
    solm.vec.data = mixed * lf.vec
    assert mixed.result.status == 0 and mixed.result.true_relres <= 1e-10
    assert np.abs(solm.vec.NumPy() - xo).max() <= 1e-7 * np.abs(xo).max()
