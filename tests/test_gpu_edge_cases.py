"""Edge cases the reference's solver and spaces meet, on the GPU path:

- zero right-hand sides and spaces without free DOFs (CGSolver stops at its
  first check with x = 0: python/krylovspace.py:129-160, 263-272);
- the iteration limit (maxsteps reached: not converged, status GH1_MAXITER);
- single-element meshes and all-Dirichlet spaces in assembly and apply;
- the argument checks of the C ABI: orders outside the supported range, vertex
  indices outside the mesh, empty meshes, vectors of the wrong size or precision.
Results are compared with the oracle wherever there is one to compare."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O
from ngsolve_gb300._lib import GH1Error
from ngsolve_gb300.meshes import MakeStructured3DMesh, Mesh as RawMesh
from tests.util import lognormal

pytestmark = pytest.mark.gpu


def _forms(gpu, fes, kappa, f, matfree):
    u, v = fes.TnT()
    a = gpu.BilinearForm(fes, nonassemble=matfree, precision="fp32" if matfree else "fp64")
    a += gpu.CoefficientFunction(kappa) * gpu.grad(u) * gpu.grad(v) * gpu.dx
    a.Assemble()
    lf = gpu.LinearForm(fes)
    lf += gpu.CoefficientFunction(f) * v * gpu.dx
    lf.Assemble()
    return a, lf


@pytest.mark.parametrize("kind,p,matfree,mode", [("hex", 3, False, "fp64"), ("hex", 4, True, "fp64"),
                                                 ("hex", 4, True, "mixed"), ("tet", 3, False, "fp64"),
                                                 ("tet", 3, True, "mixed")])
def test_cg_zero_rhs(gpu, kind, p, matfree, mode):
    """b = 0: the first residual is 0, the solver stops at its first check with
    x = 0 and status OK (no division by the zero residual, no NaN)."""
    m = MakeStructured3DMesh(hexes=(kind == "hex"), nx=3)
    fes = gpu.H1(m, order=p, dirichlet=".*")
    a, lf = _forms(gpu, fes, lognormal(m.ne, 0.5, 3), np.zeros(m.ne), matfree)
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    x = gpu.BaseVector(fes.ndof)
    x.data = np.random.default_rng(4).normal(size=fes.ndof)  # overwritten: initialize=True
    sol = gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, sol=x, tol=1e-10, maxsteps=100, printrates=False,
                         mode=mode)
    solver = gpu.solvers.CG.last_solver
    assert solver.result.status == 0
    assert solver.iterations <= 1
    xs = sol.NumPy()
    assert np.all(np.isfinite(xs)) and np.abs(xs).max() == 0.0


@pytest.mark.parametrize("kind,matfree", [("hex", False), ("hex", True), ("tet", False)])
def test_cg_no_free_dofs(gpu, kind, matfree):
    """p = 1 on one cube (hex) or its six tets with every boundary DOF fixed: no
    free DOF is left, the preconditioned residual is 0 and the solution stays 0."""
    m = MakeStructured3DMesh(hexes=(kind == "hex"), nx=1)
    fes = gpu.H1(m, order=1, dirichlet=".*")
    assert fes.nfree == 0 and not fes.FreeDofs().any()
    a, lf = _forms(gpu, fes, np.ones(m.ne), np.ones(m.ne), matfree)
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    sol = gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=1e-10, maxsteps=50, printrates=False)
    solver = gpu.solvers.CG.last_solver
    assert solver.result.status == 0 and solver.iterations <= 1
    assert np.abs(sol.NumPy()).max() == 0.0


def test_cg_iteration_limit(gpu):
    """maxsteps reached before tol: CheckResidual's maxiter exit, reported as not
    converged (GH1_MAXITER = 6) with exactly maxsteps checks and the oracle's
    residual history."""
    m = MakeStructured3DMesh(hexes=True, nx=3)
    kappa, f = lognormal(m.ne, 1.0, 5), np.random.default_rng(6).uniform(-1, 1, m.ne)
    fes = gpu.H1(m, order=3, dirichlet=".*")
    a, lf = _forms(gpu, fes, kappa, f, False)
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=1e-14, maxsteps=7, printrates=False)
    solver = gpu.solvers.CG.last_solver
    assert solver.result.status == 6
    assert solver.iterations == 7 and len(solver.residuals) == 7
    S = O.OracleSpace(m.points, m.elements, 3)
    rp, ci, va = S.assemble(kappa=kappa)
    free = S.freedofs().astype(bool)
    d = va[[rp[i] + np.searchsorted(ci[rp[i]:rp[i + 1]], i) for i in range(len(rp) - 1)]]
    inv = np.where(free, 1.0 / d, 0.0)
    _, its, hist = S.cg(S.rhs(f), inv, tol=1e-14, maxit=7, csr=(rp, ci, va))
    assert its == 7
    assert np.allclose(solver.residuals, hist[:7], rtol=1e-9)


@pytest.mark.parametrize("kind,p", [("hex", 1), ("hex", 4), ("hex", 8), ("tet", 1), ("tet", 4), ("tet", 6)])
def test_single_element(gpu, kind, p):
    """One hex (or one tet): assembled matrix and FP64 / FP32 matrix-free apply
    against the oracle."""
    if kind == "hex":
        pts = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
        pts = pts @ np.array([[1.0, 0.2, 0.0], [0.0, 0.9, 0.1], [0.1, 0.0, 1.2]])
        els = np.arange(8, dtype=np.int32)[None, :]
    else:
        pts = np.array([[0, 0, 0], [1, 0, 0], [0.2, 1, 0], [0.3, 0.2, 0.9]], float)
        els = np.array([[2, 0, 3, 1]], dtype=np.int32)
    m = RawMesh(pts, els)
    kappa, mu = np.array([1.7]), np.array([0.6])
    fes = gpu.H1(m, order=p)
    S = O.OracleSpace(m.points, m.elements, p)
    assert fes.ndof == S.ndof
    u, v = fes.TnT()
    a = gpu.BilinearForm(fes)
    a += gpu.CoefficientFunction(kappa) * gpu.grad(u) * gpu.grad(v) * gpu.dx
    a += gpu.CoefficientFunction(mu) * u * v * gpu.dx
    a.Assemble()
    orp, oci, ova = S.assemble(kappa=kappa, mu=mu)
    rp, ci, va = a.mat.CSR()
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    assert np.abs(va - ova).max() <= 1e-12 * np.abs(ova).max()
    b = gpu.BilinearForm(fes, nonassemble=True, precision="fp32")
    b += gpu.CoefficientFunction(kappa) * gpu.grad(u) * gpu.grad(v) * gpu.dx
    b += gpu.CoefficientFunction(mu) * u * v * gpu.dx
    b.Assemble()
    x = np.random.default_rng(p).normal(size=fes.ndof)
    yo = S.apply_mf(x, kappa=kappa, mu=mu)
    xv, yv = gpu.BaseVector(fes.ndof), gpu.BaseVector(fes.ndof)
    xv.data = x
    b.mat.Mult(xv, yv)
    assert np.abs(yv.NumPy() - yo).max() <= 1e-12 * np.abs(yo).max()
    x32 = gpu.BaseVector(data=torch.tensor(x, dtype=torch.float32, device="cuda"))
    y32 = gpu.BaseVector(data=torch.zeros(fes.ndof, dtype=torch.float32, device="cuda"))
    b.mat.Mult(x32, y32)
    assert np.abs(y32.NumPy().astype(np.float64) - yo).max() <= 2e-5 * np.abs(yo).max()


def test_abi_argument_checks(gpu):
    """Invalid inputs fail with an error and a message instead of reaching a kernel."""
    m = MakeStructured3DMesh(hexes=True, nx=2)
    with pytest.raises(GH1Error, match="order"):
        gpu.H1(m, order=0)
    with pytest.raises(GH1Error, match="order"):
        gpu.H1(m, order=9)
    with pytest.raises(GH1Error, match="order"):
        gpu.H1(MakeStructured3DMesh(hexes=False, nx=1), order=9)
    bad = m.elements.copy()
    bad[3, 5] = m.points.shape[0]
    with pytest.raises(ValueError, match="out of range"):  # the host-side mesh check
        RawMesh(m.points, bad)
    ctx = gpu.context(0)  # the same check inside gh1_mesh_upload
    h = ctypes.c_void_p()
    rc = ctx.lib.gh1_mesh_upload(ctx.h, m.points.shape[0], m.points.ctypes.data, bad.shape[0], 8,
                                 np.ascontiguousarray(bad).ctypes.data, ctypes.byref(h))
    assert rc == 1 and b"out of range" in ctx.lib.gh1_last_error(ctx.h)
    with pytest.raises(GH1Error, match="empty"):
        gpu.H1(RawMesh(m.points, np.zeros((0, 8), dtype=np.int32)), order=1)
    fes = gpu.H1(m, order=2)
    a, _ = _forms(gpu, fes, np.ones(m.ne), np.ones(m.ne), True)
    x = gpu.BaseVector(fes.ndof)
    with pytest.raises(ValueError):
        a.mat.Mult(x, gpu.BaseVector(fes.ndof + 1))
    with pytest.raises(TypeError):
        a.mat.Mult(x, gpu.BaseVector(data=torch.zeros(fes.ndof, dtype=torch.float32, device="cuda")))
    with pytest.raises(GH1Error, match="alias"):
        a.mat.Mult(x, x)
    c = gpu.BilinearForm(fes, nonassemble=True)  # FP64 data only
    u, v = fes.TnT()
    c += gpu.grad(u) * gpu.grad(v) * gpu.dx
    c.Assemble()
    x32 = gpu.BaseVector(data=torch.zeros(fes.ndof, dtype=torch.float32, device="cuda"))
    y32 = gpu.BaseVector(data=torch.zeros(fes.ndof, dtype=torch.float32, device="cuda"))
    with pytest.raises(GH1Error):
        c.mat.Mult(x32, y32)
    # the library stays usable after the errors
    # the constant function (1 on the vertex DOFs, which come first, 0 on the
    # edge, face and cell DOFs) is in the kernel of the Laplacian
    xv, yv = gpu.BaseVector(fes.ndof), gpu.BaseVector(fes.ndof)
    one = np.zeros(fes.ndof)
    one[:m.nv] = 1.0
    xv.data = one
    a.mat.Mult(xv, yv)
    assert np.abs(yv.NumPy()).max() < 1e-13


def test_operator_outlives_its_form(gpu):
    """An operator keeps the form it was made from: a BilinearForm dropped
    while its .mat lives on (matrix-free and assembled) leaves the operator
    valid, also after other forms have been created and freed in between
    (the reference's BilinearFormApplication holds its form the same way)."""
    import gc
    m = MakeStructured3DMesh(hexes=True, nx=3)
    fes = gpu.H1(m, order=3)
    kappa = lognormal(m.ne, 1.0, 2)

    def make(nonassemble, coef):
        u, v = fes.TnT()
        a = gpu.BilinearForm(fes, nonassemble=nonassemble)
        a += gpu.CoefficientFunction(coef) * gpu.grad(u) * gpu.grad(v) * gpu.dx
        a.Assemble()
        return a.mat

    S = O.OracleSpace(m.points, m.elements, 3)
    x = np.random.default_rng(3).normal(size=fes.ndof)
    yo = S.apply_mf(x, kappa=kappa)
    for nonassemble in (True, False):
        mat = make(nonassemble, kappa)
        gc.collect()
        for s in range(3):
            make(True, lognormal(m.ne, 1.0, 10 + s))
            gc.collect()
        xv, yv = gpu.BaseVector(fes.ndof), gpu.BaseVector(fes.ndof)
        xv.data = x
        mat.Mult(xv, yv)
        assert np.abs(yv.NumPy() - yo).max() <= 1e-12 * np.abs(yo).max()
        del mat
        gc.collect()


def test_bounded_wait_timeout_reports_error(gpu, monkeypatch):
    """A device wait that runs out of its bound is an error the host sees, and
    the context stays usable.  GH1_FIRST_WAIT_POLLS=0 at operator setup makes
    the first mbarrier wait of the paired FP32 apply give up without polling
    (the DOF-row copy it waits for is still in flight and lands); the kernel
    records the timeout, drains its copies with the full bound and returns.
    gh1_op_check and a mixed-precision CG solve then report ERR_CUDA; an
    operator set up afterwards without the knob applies correctly."""
    m = MakeStructured3DMesh(hexes=True, nx=4)
    kappa = lognormal(m.ne, 1.0, 4)
    fes = gpu.H1(m, order=3, dirichlet=".*")
    u, v = fes.TnT()

    def operator():
        a = gpu.BilinearForm(fes, nonassemble=True, precision="fp32")
        a += gpu.CoefficientFunction(kappa) * gpu.grad(u) * gpu.grad(v) * gpu.dx
        a.Assemble()
        assert a.mat.Info()["hex_variant_fp32"] == 3
        return a

    monkeypatch.setenv("GH1_HEX_GMODE", "3")
    monkeypatch.setenv("GH1_FIRST_WAIT_POLLS", "0")
    a = operator()
    ctx = fes.ctx
    x32 = gpu.BaseVector(data=torch.ones(fes.ndof, dtype=torch.float32, device="cuda"))
    y32 = gpu.BaseVector(data=torch.zeros(fes.ndof, dtype=torch.float32, device="cuda"))
    a.mat.Mult(x32, y32)  # asynchronous: the timeout is reported by the check
    with pytest.raises(GH1Error) as ei:
        ctx.check(ctx.lib.gh1_op_check(a.mat.h))
    assert ei.value.code == 2 and "timed out" in str(ei.value)
    ctx.check(ctx.lib.gh1_op_check(a.mat.h))  # reported once, then cleared
    lf = gpu.LinearForm(fes)
    lf += gpu.CoefficientFunction(np.ones(m.ne)) * v * gpu.dx
    lf.Assemble()
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    with pytest.raises(GH1Error) as ei:
        gpu.solvers.CG(mat=a.mat, rhs=lf.vec, pre=pre, tol=1e-10, maxsteps=200, printrates=False, mode="mixed",
                       stop_rule="true")
    assert ei.value.code == 2
    # the same context, a new operator without the knob
    monkeypatch.delenv("GH1_FIRST_WAIT_POLLS")
    b = operator()
    S = O.OracleSpace(m.points, m.elements, 3)
    x = np.random.default_rng(5).normal(size=fes.ndof)
    yo = S.apply_mf(x, kappa=kappa)
    xv = gpu.BaseVector(data=torch.tensor(x, dtype=torch.float32, device="cuda"))
    b.mat.Mult(xv, y32)
    ctx.check(ctx.lib.gh1_op_check(b.mat.h))
    assert np.abs(y32.NumPy().astype(np.float64) - yo).max() <= 2e-5 * np.abs(yo).max()
