"""Parity at the full sizes of the five benchmark configurations, through the C
ABI, against the FP64 CPU oracle (oracle/gh1_oracle.cpp).

C1  16^3 hex, p=3, kappa=1, f ~ U[-1,1] per element (seed 1), zero Dirichlet:
    Assemble (pattern bit-exact, entries 1e-12 row-scaled), LinearForm, and
    Jacobi-PCG to 1e-10 (iterations +-1, residual history, solution 1e-9).
C2  32^3 grid, six Kuhn tets per cube (196,608 tets), interior vertices jittered
    U[-0.2h, 0.2h] (seed 2), kappa lognormal(0,1) (seed 3), p = 2, 3, 4: full
    CSR against the oracle's Assemble, 100 SpMVs, and the matrix-free apply.
C3  64^3 hex, p=4 (16,974,593 DOFs), kappa lognormal(0,0.5) (seed 4): FP64 and
    FP32 matrix-free applies (affine-metric and per-point-metric variants)
    against the oracle's element-wise ApplyElementMatrix; the FP64 GPU solution
    behind the mixed-precision error is checked through the oracle's operator.
C4  32^3 hex, p=3, kappa lognormal(0,1) (seed 6), kappa* (seed 7): dJ/dkappa
    against the oracle's adjoint recipe (oracle CG for both solves) and against
    central finite differences with h = 1e-6 on 32 elements (seed 8).
C5  a seeded subsample of 16 of the 256 batched problems (n ~ U{8..40},
    p ~ U{1..6}, 16 right-hand sides each), spanning every order and the extreme
    sides: every solution's residual through the oracle's operator.
"""
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from ngsolve_gb300.meshes import MakeStructured3DMesh, JitterInterior
from tests.util import lognormal, csr_rowscaled_close, assert_cg_history_close

pytestmark = pytest.mark.gpu


def _jacobi_inv(rp, ci, va, free):
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    on = ci == rows
    d = np.zeros(len(rp) - 1)
    d[rows[on]] = va[on]
    return np.where(free, 1.0 / np.where(d != 0, d, 1.0), 0.0)


def _vec(gpu, a, dtype=torch.float64):
    return gpu.BaseVector(data=torch.as_tensor(np.asarray(a), dtype=dtype, device="cuda").contiguous())


def _free_relres(r, b, free):
    return float(np.linalg.norm(r[free]) / np.linalg.norm(b[free]))


# ---------------------------------------------------------------------------
def test_c1_assemble_and_pcg(gpu):
    mesh = MakeStructured3DMesh(hexes=True, nx=16)
    f = np.random.default_rng(1).uniform(-1, 1, mesh.ne)
    fes = gpu.H1(mesh, order=3, dirichlet=".*")
    assert (fes.ndof, fes.nfree) == (117649, 103823)
    S = O.OracleSpace(mesh.points, mesh.elements, 3)
    assert np.array_equal(fes.ElementDofs(), S.element_dofs())
    free = S.freedofs().astype(bool)
    assert np.array_equal(fes.FreeDofs(), free)
    u, v = fes.TnT()
    a = gpu.BilinearForm(fes)
    a += gpu.grad(u) * gpu.grad(v) * gpu.dx
    a.Assemble()
    rp, ci, va = a.mat.CSR()
    assert len(ci) == 13997521
    orp, oci, ova = S.assemble()
    _, _, noise = S.assemble(reverse=True)
    csr_rowscaled_close(rp, ci, va, orp, oci, ova, rtol=1e-12, noise=noise)
    lf = gpu.LinearForm(fes)
    lf += gpu.CoefficientFunction(f) * v * gpu.dx
    lf.Assemble()
    bo = S.rhs(f)
    assert np.abs(lf.vec.NumPy() - bo).max() <= 1e-13 * np.abs(bo).max()
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    sol = gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=1e-10, maxsteps=10000, printrates=False)
    solver = gpu.solvers.CG.last_solver
    assert solver.result.status == 0
    xo, its, hist = S.cg(bo, _jacobi_inv(orp, oci, ova, free), tol=1e-10, maxit=10000, csr=(orp, oci, ova))
    assert abs(solver.iterations - its) <= 1
    assert_cg_history_close(solver.residuals, hist)
    assert np.abs(sol.NumPy() - xo).max() <= 1e-9 * np.abs(xo).max()


# ---------------------------------------------------------------------------
_C2_NNZ = {2: 7678721, 3: 43430305, 4: 159230209}
_C2_NDOF = {2: 274625, 3: 912673, 4: 2146689}


@pytest.fixture(scope="module")
def c2_mesh():
    mesh = JitterInterior(MakeStructured3DMesh(hexes=False, nx=32), 0.2 / 32, 2)
    return mesh, lognormal(mesh.ne, 1.0, 3)


@pytest.mark.parametrize("p", [2, 3, 4])
def test_c2_assemble_spmv_apply(gpu, c2_mesh, p):
    mesh, kappa = c2_mesh
    assert mesh.ne == 196608
    fes = gpu.H1(mesh, order=p, dirichlet=".*")
    assert fes.ndof == _C2_NDOF[p]
    u, v = fes.TnT()
    a = gpu.BilinearForm(fes)
    a += gpu.CoefficientFunction(kappa) * gpu.grad(u) * gpu.grad(v) * gpu.dx
    a.Assemble()
    S = O.OracleSpace(mesh.points, mesh.elements, p)
    assert np.array_equal(fes.ElementDofs(), S.element_dofs())
    assert np.array_equal(fes.FreeDofs(), S.freedofs().astype(bool))
    rp, ci, va = a.mat.CSR()
    assert len(ci) == _C2_NNZ[p]
    orp, oci, ova = S.assemble(kappa=kappa)
    _, _, noise = S.assemble(kappa=kappa, reverse=True)
    csr_rowscaled_close(rp, ci, va, orp, oci, ova, rtol=1e-12, noise=noise)
    del rp, ci, va, noise
    # 100 SpMVs through BaseMatrix.Mult; the last product against the oracle's SpMV
    x = np.random.default_rng(20 + p).uniform(-1, 1, fes.ndof)
    xv, yv = _vec(gpu, x), gpu.BaseVector(fes.ndof)
    for _ in range(100):
        a.mat.Mult(xv, yv)
    yo = O.spmv(orp, oci, ova, x)
    assert np.abs(yv.NumPy() - yo).max() <= 1e-13 * np.abs(yo).max()
    del orp, oci, ova
    a.mat = None
    # matrix-free apply (FP64 and FP32 data) against the oracle's element-wise apply
    amf = gpu.BilinearForm(fes, nonassemble=True, precision="fp32")
    amf += gpu.CoefficientFunction(kappa) * gpu.grad(u) * gpu.grad(v) * gpu.dx
    amf.Assemble()
    ym = S.apply_mf(x, kappa=kappa)
    sc = np.abs(ym).max()
    amf.mat.Mult(xv, yv)
    assert np.abs(yv.NumPy() - ym).max() <= 1e-12 * sc
    y32 = _vec(gpu, np.zeros(fes.ndof), torch.float32)
    amf.mat.Mult(_vec(gpu, x, torch.float32), y32)
    assert np.abs(y32.NumPy().astype(np.float64) - ym).max() <= 2e-5 * sc


# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def c3(gpu):
    mesh = MakeStructured3DMesh(hexes=True, nx=64)
    kappa = lognormal(mesh.ne, 0.5, 4)
    fes = gpu.H1(mesh, order=4, dirichlet=".*")
    S = O.OracleSpace(mesh.points, mesh.elements, 4)
    return mesh, kappa, fes, S


def _c3_form(gpu, fes, kappa, affine):
    if not affine:
        os.environ["GH1_HEX_AFFINE"] = "0"
    try:
        u, v = fes.TnT()
        a = gpu.BilinearForm(fes, nonassemble=True, precision="fp32")
        a += gpu.CoefficientFunction(kappa) * gpu.grad(u) * gpu.grad(v) * gpu.dx
        a.Assemble()
    finally:
        os.environ.pop("GH1_HEX_AFFINE", None)
    return a


def test_c3_apply_full_size(gpu, c3):
    """FP64 apply within 1e-12 and FP32 within 2e-5 of max|y| of the oracle's
    ApplyElementMatrix sum, for the autotuned (affine-metric) operator and the
    per-point-metric operator."""
    mesh, kappa, fes, S = c3
    assert fes.ndof == 16974593
    x = np.random.default_rng(30).uniform(-1, 1, fes.ndof)
    yo = S.apply_mf(x, kappa=kappa)
    sc = np.abs(yo).max()
    x64, x32 = _vec(gpu, x), _vec(gpu, x, torch.float32)
    for affine in (True, False):
        a = _c3_form(gpu, fes, kappa, affine)
        var = a.mat.Info()["hex_variant_fp32"]
        assert (var in (4, 5)) == affine
        y64 = gpu.BaseVector(fes.ndof)
        a.mat.Mult(x64, y64)
        assert np.abs(y64.NumPy() - yo).max() <= 1e-12 * sc
        y32 = _vec(gpu, np.zeros(fes.ndof), torch.float32)
        a.mat.Mult(x32, y32)
        assert np.abs(y32.NumPy().astype(np.float64) - yo).max() <= 2e-5 * sc
        del a


def test_c3_solutions_oracle_anchored(gpu, c3):
    """The FP64 GPU solve to 1e-13 solves the oracle's system (its residual
    through the oracle's operator and load vector); the mixed-precision solves
    reach 1e-10 in the oracle's residual too, and the mixed solve run to 1e-12
    is within 1e-9 of the anchored FP64 solution."""
    mesh, kappa, fes, S = c3
    f = np.random.default_rng(5).uniform(-1, 1, mesh.ne)
    a = _c3_form(gpu, fes, kappa, True)
    u, v = fes.TnT()
    lf = gpu.LinearForm(fes)
    lf += gpu.CoefficientFunction(f) * v * gpu.dx
    lf.Assemble()
    bo = S.rhs(f)
    assert np.abs(lf.vec.NumPy() - bo).max() <= 1e-13 * np.abs(bo).max()
    free = S.freedofs().astype(bool)
    pre = a.mat.CreateSmoother(fes.FreeDofs())

    def solve(mode, tol):
        sol = gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=tol, maxsteps=100000, printrates=False,
                             mode=mode, stop_rule="true")
        r = gpu.solvers.CG.last_solver.result
        assert r.status == 0 and r.true_relres <= tol
        return sol.NumPy().copy()

    xr = solve("fp64", 1e-13)
    res_ref = _free_relres(bo - S.apply_mf(xr, kappa=kappa), bo, free)
    assert res_ref <= 1e-12, res_ref
    xm = solve("mixed", 1e-10)
    res_m = _free_relres(bo - S.apply_mf(xm, kappa=kappa), bo, free)
    assert res_m <= 1.01e-10, res_m
    x12 = solve("mixed", 1e-12)
    nr = np.abs(xr).max()
    assert np.abs(x12 - xr).max() <= 1e-9 * nr


# ---------------------------------------------------------------------------
def test_c4_adjoint_gradient(gpu):
    """dJ/dkappa at 32^3 hex p=3 against (1) the oracle's adjoint recipe, u and
    lambda from the oracle's FP64 CG on its assembled matrix, and (2) central
    finite differences with h = 1e-6 on 32 seeded elements (seed 8).

    The difference quotient (J(kappa + h e_k) - J(kappa - h e_k)) / 2h is
    formed without cancellation: with u_0 the solution at kappa, the solution
    at kappa +- h e_k is u_0 + w, where A(kappa +- h e_k) w = f - A(kappa) u_0
    -+ h A_k u_0 (A_k: element k's stiffness with unit coefficient), and
    J(u_0 + w) - J(u_0) = w^T M (u_0 - u_t) + w^T M w / 2.  Each w is solved
    to 1e-12 relative in FP64, so the quotient carries the O(h^2) truncation
    (~1e-12 relative) and no rounding of J itself."""
    mesh = MakeStructured3DMesh(hexes=True, nx=32)
    p = 3
    kappa = lognormal(mesh.ne, 1.0, 6)
    kstar = lognormal(mesh.ne, 1.0, 7)
    f = np.random.default_rng(5).uniform(-1, 1, mesh.ne)
    fes = gpu.H1(mesh, order=p, dirichlet=".*")
    assert fes.ndof == 912673
    u, v = fes.TnT()
    lf = gpu.LinearForm(fes)
    lf += gpu.CoefficientFunction(f) * v * gpu.dx
    lf.Assemble()
    target = gpu.AdjointProblem(fes, lf.vec, torch.zeros(fes.ndof, dtype=torch.float64, device="cuda"), tol=1e-14)
    target.evaluate(kstar)
    ut = target.u.clone()
    prob = gpu.AdjointProblem(fes, lf.vec, ut, tol=1e-14)
    kt = torch.tensor(kappa, dtype=torch.float64, requires_grad=True)
    J = gpu.AdjointJ.apply(kt, prob)
    J.backward()
    g = kt.grad.numpy().copy()
    u0 = prob.u.clone()

    # (1) the oracle's recipe: CG solves on the oracle's assembled matrices
    S = O.OracleSpace(mesh.points, mesh.elements, p)
    free = S.freedofs().astype(bool)
    rp, ci, va = S.assemble(kappa=kappa)
    inv = _jacobi_inv(rp, ci, va, free)
    uo, _, _ = S.cg(S.rhs(f), inv, tol=1e-13, maxit=20000, csr=(rp, ci, va))
    mrp, mci, mva = S.assemble(kappa=np.zeros(mesh.ne), mu=np.ones(mesh.ne))
    ut_h = ut.cpu().numpy()
    lo, _, _ = S.cg(O.spmv(mrp, mci, mva, uo - ut_h), inv, tol=1e-13, maxit=20000, csr=(rp, ci, va))
    go = -S.elem_grad_dot(uo, lo)
    Jo = 0.5 * float((uo - ut_h) @ O.spmv(mrp, mci, mva, uo - ut_h))
    assert abs(J.item() - Jo) <= 1e-10 * abs(Jo)
    assert np.abs(g - go).max() <= 1e-8 * np.abs(go).max()
    del rp, ci, va, mrp, mci, mva

    # (2) central differences, h = 1e-6
    h = 1e-6
    els = np.random.default_rng(8).choice(mesh.ne, 32, replace=False)

    def matfree(coef, mass=False):
        a = gpu.BilinearForm(fes, nonassemble=True)
        if mass:
            a += gpu.CoefficientFunction(coef) * u * v * gpu.dx
        else:
            a += gpu.CoefficientFunction(coef) * gpu.grad(u) * gpu.grad(v) * gpu.dx
        a.Assemble()
        return a.mat

    def apply(mat, x):
        y = gpu.BaseVector(fes.ndof)
        mat.Mult(gpu.BaseVector(data=x), y)
        return y.t

    A0 = matfree(kappa)
    M = matfree(np.ones(mesh.ne), mass=True)
    r0 = lf.vec.t - apply(A0, u0)
    m_err = apply(M, u0 - ut)
    freedofs = fes.FreeDofs()
    for e in els:
        ind = np.zeros(mesh.ne)
        ind[e] = 1.0
        z = apply(matfree(ind), u0)
        dJ = {}
        for s in (1, -1):
            k = kappa.copy()
            k[e] += s * h
            A = matfree(k)
            rhs = gpu.BaseVector(data=(r0 - s * h * z).contiguous())
            w = gpu.solvers.CG(mat=A, rhs=rhs, pre=A.CreateSmoother(freedofs), tol=1e-12, maxsteps=20000,
                               printrates=False, stop_rule="true").t
            assert gpu.solvers.CG.last_solver.result.status == 0
            dJ[s] = float(w @ m_err) + 0.5 * float(w @ apply(M, w))
        fd = (dJ[1] - dJ[-1]) / (2 * h)
        assert abs(fd - g[e]) <= 1e-6 * abs(g[e]), (int(e), fd, g[e])


# ---------------------------------------------------------------------------
def _c5_subsample():
    """The 256 problems of the batched configuration (sides and orders from
    seed 9, problem i's data from seed (9, i)); per order the smallest and the
    largest side, plus four more seeded picks (seed 10)."""
    rng = np.random.default_rng(9)
    sides = rng.integers(8, 41, 256)
    orders = rng.integers(1, 7, 256)
    pick = []
    for p in range(1, 7):
        idx = np.flatnonzero(orders == p)
        for i in (idx[np.argmin(sides[idx])], idx[np.argmax(sides[idx])]):
            if i not in pick:
                pick.append(int(i))
    for i in np.random.default_rng(10).permutation(256):
        if len(pick) >= 16:
            break
        if int(i) not in pick:
            pick.append(int(i))
    return [(i, int(sides[i]), int(orders[i])) for i in pick]


def test_c5_subsample_spans_the_configuration():
    sub = _c5_subsample()
    assert len(sub) == 16
    assert {p for _, _, p in sub} == set(range(1, 7))
    ns = [n for _, n, _ in sub]
    assert min(ns) <= 9 and max(ns) >= 39


def test_c5_batched_subsample(gpu):
    R = 16
    sub = _c5_subsample()
    forms, rhs, data = [], [], []
    for i, n, p in sub:
        prng = np.random.default_rng([9, i])
        mesh = MakeStructured3DMesh(hexes=True, nx=n)
        kappa = np.exp(prng.normal(0, 1, mesh.ne))
        fes = gpu.H1(mesh, order=p, dirichlet=".*")
        u, v = fes.TnT()
        a = gpu.BilinearForm(fes, nonassemble=True, precision="fp32")
        a += gpu.CoefficientFunction(kappa) * gpu.grad(u) * gpu.grad(v) * gpu.dx
        B = torch.zeros((R, fes.ndof), dtype=torch.float64, device="cuda")
        fs = []
        for r in range(R):
            fr = prng.uniform(-1, 1, mesh.ne)
            lf = gpu.LinearForm(fes)
            lf += gpu.CoefficientFunction(fr) * v * gpu.dx
            lf.Assemble()
            B[r].copy_(lf.vec.t)
            fs.append(fr)
        forms.append(a)
        rhs.append(B)
        data.append((mesh, kappa, fs))
    solver = gpu.solvers.BatchCG(forms, [R] * len(forms))
    X = solver.Solve(rhs, tol=1e-10)
    assert solver.status == 0
    assert all(r.status == 0 and r.true_relres <= 1e-10 for r in solver.results)
    for (i, n, p), a, x, (mesh, kappa, fs) in zip(sub, forms, X, data):
        S = O.OracleSpace(mesh.points, mesh.elements, p)
        free = S.freedofs().astype(bool)
        # right-hand sides 0 and 15 (0 only above a million DOFs) of every
        # problem through the oracle's load vector and operator (FP64,
        # element-wise ApplyElementMatrix)
        for r in ((0, R - 1) if S.ndof < 1000000 else (0,)):
            bo = S.rhs(fs[r])
            xr = x[r].cpu().numpy()
            res = _free_relres(bo - S.apply_mf(xr, kappa=kappa), bo, free)
            assert res <= 1.05e-10, (i, n, p, r, res)
        del S
