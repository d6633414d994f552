"""Batched solves (many problems x many right-hand sides in one CUDA graph)
against the single-problem solver and the FP64 oracle."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.util import lognormal

pytestmark = pytest.mark.gpu


def _problem(gpu, n, p, seed, nrhs):
    mesh = gpu.MakeStructured3DMesh(hexes=True, nx=n)
    kappa = lognormal(mesh.ne, 1.0, seed)
    fes = gpu.H1(mesh, order=p, dirichlet=".*")
    u, v = fes.TnT()
    a = gpu.BilinearForm(fes, nonassemble=True, precision="fp32")
    a += gpu.CoefficientFunction(kappa) * gpu.grad(u) * gpu.grad(v) * gpu.dx
    a.Assemble()
    rng = np.random.default_rng(seed + 100)
    B = torch.zeros((nrhs, fes.ndof), dtype=torch.float64, device="cuda")
    fs = []
    for r in range(nrhs):
        f = rng.uniform(-1, 1, mesh.ne)
        lf = gpu.LinearForm(fes)
        lf += gpu.CoefficientFunction(f) * v * gpu.dx
        lf.Assemble()
        B[r].copy_(lf.vec.t)
        fs.append(f)
    return mesh, kappa, fes, a, B, fs


def test_batch_matches_single_and_oracle(gpu):
    specs = [(3, 2, 1, 3), (4, 3, 2, 2), (2, 5, 3, 4), (5, 1, 4, 1), (3, 4, 5, 5)]
    probs = [_problem(gpu, n, p, seed, r) for n, p, seed, r in specs]
    solver = gpu.solvers.BatchCG([pr[3] for pr in probs], [s[3] for s in specs])
    X = solver.Solve([pr[4] for pr in probs], tol=1e-10)
    assert solver.status == 0
    assert len(solver.results) == sum(s[3] for s in specs)
    assert all(r.status == 0 and r.true_relres <= 1e-10 for r in solver.results)
    for (mesh, kappa, fes, a, B, fs), x, (n, p, seed, nrhs) in zip(probs, X, specs):
        # FP64 true residual recomputed through the public apply
        for r in range(nrhs):
            xv = gpu.BaseVector(data=x[r].clone())
            yv = gpu.BaseVector(fes.ndof)
            a.mat.Mult(xv, yv)
            free = torch.tensor(fes.FreeDofs(), device="cuda")
            res = (B[r] - yv.t)[free].norm() / B[r][free].norm()
            assert res.item() <= 1.2e-10
        # against the oracle's FP64 CG on the assembled matrix
        S = O.OracleSpace(mesh.points, mesh.elements, p)
        rp, ci, va = S.assemble(kappa=kappa)
        d = va[[rp[i] + np.searchsorted(ci[rp[i]:rp[i + 1]], i) for i in range(S.ndof)]]
        inv = np.where(S.freedofs().astype(bool), 1.0 / d, 0.0)
        for r in range(nrhs):
            xo, _, _ = S.cg(B[r].cpu().numpy(), inv, tol=1e-13, maxit=20000, csr=(rp, ci, va))
            assert np.abs(x[r].cpu().numpy() - xo).max() <= 1e-7 * np.abs(xo).max()
