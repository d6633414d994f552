"""Generic B^T D B operator (gh1_form_set_bdb) against the oracle's element-by-
element B^T D B apply: convection b . grad(u) v, its transpose u (c . grad v), a
non-symmetric diffusion matrix and reaction, with D per element (the reference's
AssembleBDBFused evaluation) or per rule point (coefficients in x, y, z).
FP64 within 1e-12 and FP32 within 2e-5 of max |y|; the diagonal behind Jacobi
within 1e-12; a generic form equal to kappa grad.grad + mu u v solves like it."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O
from ngsolve_gb300 import comp as C
from ngsolve_gb300 import _lib
from ngsolve_gb300.meshes import MakeStructured3DMesh, JitterInterior
from tests.util import lognormal

pytestmark = pytest.mark.gpu


def _mesh(hexes, n, jitter, seed=61):
    m = MakeStructured3DMesh(hexes=hexes, nx=n)
    return JitterInterior(m, jitter / n, seed) if jitter else m


def _terms(gpu, fes, ne, seed, pointwise):
    """kappa grad.grad + (b . grad u) v + u (c . grad v) + (Kn grad u).grad v + r u v;
    with pointwise, r and one convection component depend on x, y, z."""
    rng = np.random.default_rng(seed)
    u, v = fes.TnT()
    kap = lognormal(ne, 0.5, seed + 1)
    Kn = np.eye(3) * 0.5 + rng.normal(size=(3, 3)) * 0.2  # not symmetric
    b = gpu.CoefficientFunction((rng.normal(size=ne), 0.7, gpu.y if pointwise else -0.4))
    c = gpu.CoefficientFunction((0.3, rng.normal(size=ne), 0.2))
    r = (1.0 + gpu.x) if pointwise else gpu.CoefficientFunction(rng.uniform(0.5, 2.0, ne))
    return [gpu.CoefficientFunction(kap) * gpu.grad(u) * gpu.grad(v) * gpu.dx,
            gpu.InnerProduct(b, gpu.grad(u)) * v * gpu.dx,
            u * gpu.InnerProduct(c, gpu.grad(v)) * gpu.dx,
            gpu.InnerProduct(gpu.CoefficientFunction(Kn) * gpu.grad(u), gpu.grad(v)) * gpu.dx,
            r * u * v * gpu.dx]


def _rule(gpu, fes):
    nq = ctypes.c_int()
    ctx = fes.ctx
    ctx.check(ctx.lib.gh1_space_qpoints(fes.h, None, None, _lib.GH1_MEM_HOST, ctypes.byref(nq)))
    ref = np.zeros((nq.value, 4))
    ctx.check(ctx.lib.gh1_space_qpoints(fes.h, ref.ctypes.data_as(ctypes.c_void_p), None, _lib.GH1_MEM_HOST, None))
    xyz = torch.empty((fes.ne, nq.value, 3), dtype=torch.float64, device="cuda")
    ctx.sync_stream()
    ctx.check(ctx.lib.gh1_space_qpoints(fes.h, None, ctypes.c_void_p(xyz.data_ptr()), _lib.GH1_MEM_DEVICE, None))
    torch.cuda.synchronize()
    return ref, xyz


def _oracle_D(terms, ne, xyz):
    D = C._bdb_D(terms, ne, xyz, torch.device("cuda"))
    return (D[:, 0] if xyz is None else D).reshape(ne, -1, 16).squeeze(1).cpu().numpy()


def _apply(gpu, a, x, dtype):
    xv = gpu.BaseVector(data=torch.tensor(x, dtype=dtype, device="cuda"))
    yv = gpu.BaseVector(data=torch.zeros(len(x), dtype=dtype, device="cuda"))
    a.mat.Mult(xv, yv)
    return yv.NumPy().astype(np.float64)


CASES = [(True, 1, 0.0, False), (True, 2, 0.0, False), (True, 4, 0.0, False), (True, 6, 0.0, False),
         (True, 3, 0.15, False), (True, 5, 0.1, False), (True, 3, 0.0, True), (True, 4, 0.1, True),
         (False, 1, 0.2, False), (False, 2, 0.2, False), (False, 3, 0.2, False), (False, 4, 0.2, False),
         (False, 5, 0.2, False), (False, 6, 0.2, False), (False, 7, 0.2, False), (False, 3, 0.2, True)]


@pytest.mark.parametrize("hexes,p,jit,pointwise", CASES)
def test_bdb_apply_parity(gpu, hexes, p, jit, pointwise):
    m = _mesh(hexes, 3 if hexes else 2, jit)
    fes = gpu.H1(m, order=p, dirichlet=".*")
    terms = _terms(gpu, fes, m.ne, 62 + p, pointwise)
    a = gpu.BilinearForm(fes, nonassemble=True, precision="fp32")
    for t in terms:
        a += t
    a.Assemble()
    info = a.mat.Info()
    affine_elem = hexes and not pointwise and jit == 0.0
    want = 8 if (affine_elem or (not hexes and not pointwise)) else 7
    # FP32 on hexes: the one-element kernel or the paired one (9 with records per
    # element, 11 per point), whichever the setup timed faster; tets: the FP32
    # pipe or the tensor cores (10)
    alt = (9 if want == 8 else 11) if hexes else (10 if want == 8 else want)
    assert info["hex_variant_fp64"] == want and info["hex_variant_fp32"] in (want, alt)
    S = O.OracleSpace(m.points, m.elements, p)
    ref, xyz = _rule(gpu, fes)
    D = _oracle_D(terms, m.ne, xyz if pointwise else None)
    x = np.random.default_rng(63).normal(size=fes.ndof)
    yo = S.apply_bdb(x, D, rule=ref if pointwise else None)
    sc = np.abs(yo).max()
    assert np.abs(_apply(gpu, a, x, torch.float64) - yo).max() <= 1e-12 * sc
    assert np.abs(_apply(gpu, a, x, torch.float32) - yo).max() <= 2e-5 * sc


@pytest.mark.parametrize("hexes,p,jit,pointwise", [(True, 4, 0.0, False), (True, 3, 0.15, True), (False, 3, 0.2, False),
                                                   (False, 2, 0.2, True)])
def test_bdb_diagonal(gpu, hexes, p, jit, pointwise):
    """The Jacobi preconditioner of a generic operator inverts the oracle's diagonal."""
    m = _mesh(hexes, 3, jit)
    fes = gpu.H1(m, order=p, dirichlet=".*")
    terms = _terms(gpu, fes, m.ne, 64, pointwise)
    a = gpu.BilinearForm(sum(terms[1:], terms[0]), nonassemble=True).Assemble()
    S = O.OracleSpace(m.points, m.elements, p)
    ref, xyz = _rule(gpu, fes)
    d = S.diag_bdb(_oracle_D(terms, m.ne, xyz if pointwise else None), rule=ref if pointwise else None)
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    ones = gpu.BaseVector(fes.ndof)
    ones.data = np.ones(fes.ndof)
    inv = gpu.BaseVector(fes.ndof)
    pre.Mult(ones, inv)
    free = np.asarray(fes.FreeDofs(), dtype=bool)
    got = inv.NumPy()
    assert np.all(got[~free] == 0)
    assert np.abs(got[free] * d[free] - 1.0).max() <= 1e-12


@pytest.mark.parametrize("hexes,p", [(True, 4), (False, 3)])
def test_bdb_variant_paths_agree(gpu, hexes, p, monkeypatch):
    """On affine hexes the per-element records (variant 8) and the per-point
    records (GH1_BDB_AFFINE=0, variant 7) give the same operator; a point-wise D
    that repeats each element's matrix equals the per-element form."""
    m = _mesh(hexes, 4, 0.0 if hexes else 0.2)
    fes = gpu.H1(m, order=p)
    terms = _terms(gpu, fes, m.ne, 65, False)
    x = np.random.default_rng(66).normal(size=fes.ndof)
    a1 = gpu.BilinearForm(sum(terms[1:], terms[0]), nonassemble=True, precision="fp32").Assemble()
    y1 = _apply(gpu, a1, x, torch.float64)
    if hexes:
        monkeypatch.setenv("GH1_BDB_AFFINE", "0")
        a2 = gpu.BilinearForm(sum(terms[1:], terms[0]), nonassemble=True, precision="fp32").Assemble()
        assert a2.mat.Info()["hex_variant_fp64"] == 7
        assert np.abs(_apply(gpu, a2, x, torch.float64) - y1).max() <= 1e-13 * np.abs(y1).max()
        monkeypatch.delenv("GH1_BDB_AFFINE")
    # the same D given per point through the C ABI
    _, xyz = _rule(gpu, fes)
    D = C._bdb_D(terms, m.ne, None, torch.device("cuda"))[:, 0].reshape(m.ne, 1, 16)
    Dp = D.expand(m.ne, xyz.shape[1], 16).contiguous()
    ctx = fes.ctx
    h = ctypes.c_void_p()
    ctx.check(ctx.lib.gh1_form_create(fes.h, None, None, _lib.GH1_MEM_HOST, ctypes.byref(h)))
    try:
        ctx.check(ctx.lib.gh1_form_set_bdb(h, ctypes.c_void_p(Dp.data_ptr()), 1, _lib.GH1_MEM_DEVICE))
        op = ctypes.c_void_p()
        ctx.check(ctx.lib.gh1_matfree_create(h, 1, ctypes.byref(op)))
        mat = C.BilinearFormApplication(ctx, op, fes.ndof, fes)
        assert mat.Info()["hex_variant_fp64"] == 7
        xv = gpu.BaseVector(fes.ndof)
        xv.data = x
        yv = gpu.BaseVector(fes.ndof)
        mat.Mult(xv, yv)
        assert np.abs(yv.NumPy() - y1).max() <= 1e-13 * np.abs(y1).max()
        del mat
    finally:
        ctx.lib.gh1_form_free(h)


def _affine_hexes(nx):
    """Structured hexes under a general affine map (every element the same
    parallelepiped): one record per element applies."""
    from ngsolve_gb300.meshes import Mesh as RawMesh
    m = MakeStructured3DMesh(hexes=True, nx=nx)
    A = np.array([[1.0, 0.3, -0.2], [0.1, 0.8, 0.25], [-0.15, 0.2, 1.3]])
    return RawMesh(m.points @ A.T + np.array([0.5, -1.0, 2.0]), m.elements)


@pytest.mark.parametrize("pair", ["0", "1"])
@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6])
def test_bdb_paired_records(gpu, monkeypatch, p, pair):
    """FP32 B^T D B with one record per affine element, on the paired kernel
    (two elements per lane; GH1_BDB_PAIR=1, variant 9) and on the one-element
    kernel (GH1_BDB_PAIR=0, variant 8): within 2e-5 of the oracle, with 27 and 8
    elements (the odd count leaves the last pair half empty)."""
    monkeypatch.setenv("GH1_BDB_PAIR", pair)
    for nx in (3, 2):
        m = _affine_hexes(nx)
        fes = gpu.H1(m, order=p)
        terms = _terms(gpu, fes, m.ne, 90 + p, False)
        a = gpu.BilinearForm(sum(terms[1:], terms[0]), nonassemble=True, precision="fp32").Assemble()
        assert a.mat.Info()["hex_variant_fp32"] == (9 if pair == "1" else 8)
        D = _oracle_D(terms, m.ne, None)
        x = np.random.default_rng(91).normal(size=fes.ndof)
        yo = O.OracleSpace(m.points, m.elements, p).apply_bdb(x, D)
        assert np.abs(_apply(gpu, a, x, torch.float32) - yo).max() <= 2e-5 * np.abs(yo).max()
        assert np.abs(_apply(gpu, a, x, torch.float64) - yo).max() <= 1e-12 * np.abs(yo).max()


@pytest.mark.parametrize("pair", ["0", "1"])
@pytest.mark.parametrize("p,pointwise", [(1, False), (2, True), (3, False), (4, True), (5, False), (6, False)])
def test_bdb_paired_point_records(gpu, monkeypatch, p, pointwise, pair):
    """FP32 B^T D B with a record per rule point (jittered hexes; a D that varies
    with x, y, z for some orders) on the paired kernel (GH1_BDB_PAIR=1, variant 11)
    and on the one-element kernel (=0, variant 7): within 2e-5 of the oracle, with
    27 and 8 elements."""
    monkeypatch.setenv("GH1_BDB_PAIR", pair)
    for nx in (3, 2):
        m = _mesh(True, nx, 0.15, seed=100 + p)
        fes = gpu.H1(m, order=p)
        terms = _terms(gpu, fes, m.ne, 101 + p, pointwise)
        a = gpu.BilinearForm(sum(terms[1:], terms[0]), nonassemble=True, precision="fp32").Assemble()
        assert a.mat.Info()["hex_variant_fp32"] == (11 if pair == "1" else 7)
        ref, xyz = _rule(gpu, fes)
        D = _oracle_D(terms, m.ne, xyz if pointwise else None)
        x = np.random.default_rng(102).normal(size=fes.ndof)
        yo = O.OracleSpace(m.points, m.elements, p).apply_bdb(x, D, rule=ref if pointwise else None)
        assert np.abs(_apply(gpu, a, x, torch.float32) - yo).max() <= 2e-5 * np.abs(yo).max()
        assert np.abs(_apply(gpu, a, x, torch.float64) - yo).max() <= 1e-12 * np.abs(yo).max()


def test_bdb_paired_point_records_mixed_cg(gpu, monkeypatch):
    """The value-gradient coupled symmetric form on jittered hexes (records per
    rule point) on the paired kernel: the mixed CG, which uses the kernel's fused
    energy, reaches the FP64 CG's solution (1e-8)."""
    monkeypatch.setenv("GH1_BDB_PAIR", "1")
    m = _mesh(True, 4, 0.15, seed=103)
    fes = gpu.H1(m, order=3, dirichlet=".*")
    u, v = fes.TnT()
    c = gpu.CoefficientFunction((0.2, -0.1, 0.15))
    form = (gpu.CoefficientFunction(lognormal(m.ne, 0.5, 104)) * gpu.grad(u) * gpu.grad(v) * gpu.dx
            + gpu.InnerProduct(c, gpu.grad(u)) * v * gpu.dx + u * gpu.InnerProduct(c, gpu.grad(v)) * gpu.dx
            + gpu.CoefficientFunction(2.0) * u * v * gpu.dx)
    a = gpu.BilinearForm(form, nonassemble=True, precision="mixed").Assemble()
    assert a.mat.Info()["hex_variant_fp32"] == 11
    f = gpu.LinearForm(gpu.CoefficientFunction(np.random.default_rng(105).uniform(-1, 1, m.ne)) * v * gpu.dx).Assemble()
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    xm = gpu.solvers.CG(mat=a.mat, rhs=f.vec, pre=pre, tol=1e-11, maxsteps=5000, printrates=False,
                        mode="mixed").NumPy().copy()
    assert gpu.solvers.CG.last_solver.result.applies32 > 0
    x6 = gpu.solvers.CG(mat=a.mat, rhs=f.vec, pre=pre, tol=1e-12, maxsteps=5000, printrates=False,
                        mode="fp64").NumPy()
    assert np.abs(xm - x6).max() <= 1e-8 * np.abs(x6).max()


@pytest.mark.parametrize("tc", ["0", "1"])
@pytest.mark.parametrize("p", [2, 3, 4])
def test_bdb_tet_tensor_core(gpu, monkeypatch, p, tc):
    """FP32 B^T D B on tets with one record per element, both products of a
    same-class tile of up to 128 elements on the tensor cores (GH1_TET_BDB_TC=1,
    variant 10) or on the FP32 pipe (=0, variant 8): within 2e-5 of the oracle on
    meshes with all 24 orientation classes, 162 and 3,072 tets (one partial tile
    per class, several tiles)."""
    from tests.util import permute_tets
    from ngsolve_gb300.meshes import Mesh as RawMesh
    monkeypatch.setenv("GH1_TET_BDB_TC", tc)
    for n in (3, 8):
        m0 = _mesh(False, n, 0.2)
        m = RawMesh(m0.points, permute_tets(m0.elements, 95 + n))
        fes = gpu.H1(m, order=p)
        terms = _terms(gpu, fes, m.ne, 96 + p, False)
        a = gpu.BilinearForm(sum(terms[1:], terms[0]), nonassemble=True, precision="fp32").Assemble()
        assert a.mat.Info()["hex_variant_fp32"] == (10 if tc == "1" else 8)
        D = _oracle_D(terms, m.ne, None)
        x = np.random.default_rng(97).normal(size=fes.ndof)
        yo = O.OracleSpace(m.points, m.elements, p).apply_bdb(x, D)
        assert np.abs(_apply(gpu, a, x, torch.float32) - yo).max() <= 2e-5 * np.abs(yo).max()
        assert np.abs(_apply(gpu, a, x, torch.float64) - yo).max() <= 1e-12 * np.abs(yo).max()


def test_bdb_tet_tensor_core_mixed_cg(gpu, monkeypatch):
    """A symmetric generic tet form (value-gradient coupling in both directions)
    with its FP32 applies on the tensor cores: the mixed CG, which uses the
    kernel's fused energy, reaches the FP64 CG's solution (1e-8)."""
    monkeypatch.setenv("GH1_TET_BDB_TC", "1")
    m = _mesh(False, 5, 0.2)
    fes = gpu.H1(m, order=3, dirichlet=".*")
    u, v = fes.TnT()
    c = gpu.CoefficientFunction((0.2, -0.1, 0.15))
    form = (gpu.CoefficientFunction(lognormal(m.ne, 0.5, 98)) * gpu.grad(u) * gpu.grad(v) * gpu.dx
            + gpu.InnerProduct(c, gpu.grad(u)) * v * gpu.dx + u * gpu.InnerProduct(c, gpu.grad(v)) * gpu.dx
            + gpu.CoefficientFunction(2.0) * u * v * gpu.dx)
    a = gpu.BilinearForm(form, nonassemble=True, precision="mixed").Assemble()
    assert a.mat.Info()["hex_variant_fp32"] == 10
    f = gpu.LinearForm(gpu.CoefficientFunction(np.random.default_rng(99).uniform(-1, 1, m.ne)) * v * gpu.dx).Assemble()
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    xm = gpu.solvers.CG(mat=a.mat, rhs=f.vec, pre=pre, tol=1e-11, maxsteps=5000, printrates=False,
                        mode="mixed").NumPy().copy()
    assert gpu.solvers.CG.last_solver.result.applies32 > 0
    x6 = gpu.solvers.CG(mat=a.mat, rhs=f.vec, pre=pre, tol=1e-12, maxsteps=5000, printrates=False,
                        mode="fp64").NumPy()
    assert np.abs(xm - x6).max() <= 1e-8 * np.abs(x6).max()


def test_bdb_paired_records_mixed_cg(gpu, monkeypatch):
    """A symmetric generic form outside the Laplace type (value-gradient coupling
    u (c . grad v) + (c . grad u) v) on the paired record kernel: the mixed CG,
    which uses the kernel's fused energy, reaches the FP64 CG's solution (1e-8)."""
    monkeypatch.setenv("GH1_BDB_PAIR", "1")
    m = _affine_hexes(4)
    fes = gpu.H1(m, order=3, dirichlet=".*")
    u, v = fes.TnT()
    c = gpu.CoefficientFunction((0.2, -0.1, 0.15))
    form = (gpu.CoefficientFunction(lognormal(m.ne, 0.5, 92)) * gpu.grad(u) * gpu.grad(v) * gpu.dx
            + gpu.InnerProduct(c, gpu.grad(u)) * v * gpu.dx + u * gpu.InnerProduct(c, gpu.grad(v)) * gpu.dx
            + gpu.CoefficientFunction(2.0) * u * v * gpu.dx)
    a = gpu.BilinearForm(form, nonassemble=True, precision="mixed").Assemble()
    assert a.mat.Info()["hex_variant_fp32"] == 9
    f = gpu.LinearForm(gpu.CoefficientFunction(np.random.default_rng(93).uniform(-1, 1, m.ne)) * v * gpu.dx).Assemble()
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    xm = gpu.solvers.CG(mat=a.mat, rhs=f.vec, pre=pre, tol=1e-11, maxsteps=5000, printrates=False,
                        mode="mixed").NumPy().copy()
    assert gpu.solvers.CG.last_solver.result.applies32 > 0
    x6 = gpu.solvers.CG(mat=a.mat, rhs=f.vec, pre=pre, tol=1e-12, maxsteps=5000, printrates=False,
                        mode="fp64").NumPy()
    assert np.abs(xm - x6).max() <= 1e-8 * np.abs(x6).max()


@pytest.mark.parametrize("hexes,p", [(True, 3), (False, 2)])
def test_bdb_symmetric_form_solves_like_laplace(gpu, hexes, p):
    """(1 + 0 x) grad u . grad v + mu u v is the Laplace + mass operator written as
    a point-wise generic form: the mixed-precision CG on it reaches the same
    solution as on the standard form (1e-9)."""
    m = _mesh(hexes, 4, 0.1)
    fes = gpu.H1(m, order=p, dirichlet=".*")
    u, v = fes.TnT()
    mu = lognormal(m.ne, 0.5, 67)
    one = 0.0 * gpu.x + 1.0
    ag = gpu.BilinearForm(one * gpu.grad(u) * gpu.grad(v) * gpu.dx + gpu.CoefficientFunction(mu) * u * v * gpu.dx,
                          nonassemble=True, precision="mixed").Assemble()
    # hexes: a form of Laplace type takes the standard kernels (per-point metric
    # variants 0-3 or the tensor-core form); tets keep the B^T D B kernel
    assert (ag.mat.Info()["hex_variant_fp64"] in (0, 1)) if hexes else ag.mat.Info()["hex_variant_fp64"] == 7
    al = gpu.BilinearForm(gpu.grad(u) * gpu.grad(v) * gpu.dx + gpu.CoefficientFunction(mu) * u * v * gpu.dx,
                          nonassemble=True, precision="mixed").Assemble()
    f = gpu.LinearForm(gpu.CoefficientFunction(np.random.default_rng(68).uniform(-1, 1, m.ne)) * v * gpu.dx).Assemble()
    sols = []
    for a in (ag, al):
        pre = a.mat.CreateSmoother(fes.FreeDofs())
        sols.append(gpu.solvers.CG(mat=a.mat, rhs=f.vec, pre=pre, tol=1e-11, maxsteps=5000, printrates=False,
                                   mode="mixed"))
    assert gpu.Norm(sols[0] - sols[1]) <= 1e-9 * gpu.Norm(sols[1])


@pytest.mark.parametrize("hexes,p,jit,pointwise", [(True, 2, 0.0, False), (True, 3, 0.15, True), (True, 5, 0.0, False),
                                                   (False, 2, 0.2, False), (False, 3, 0.2, True), (False, 4, 0.2, False)])
def test_bdb_assembled(gpu, hexes, p, jit, pointwise):
    """BilinearForm(generic).Assemble(): the CSR pattern is the space's
    MatrixGraph, A x matches the oracle's B^T D B apply (1e-12) and the
    matrix-free operator of the same form; transposing D transposes A."""
    m = _mesh(hexes, 3 if hexes else 2, jit)
    fes = gpu.H1(m, order=p)
    terms = _terms(gpu, fes, m.ne, 69 + p, pointwise)
    a = gpu.BilinearForm(sum(terms[1:], terms[0])).Assemble()
    rp, ci, va = a.mat.CSR()
    S = O.OracleSpace(m.points, m.elements, p)
    orp, oci = S.graph()
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    ref, xyz = _rule(gpu, fes)
    D = _oracle_D(terms, m.ne, xyz if pointwise else None)
    x = np.random.default_rng(70).normal(size=fes.ndof)
    yo = S.apply_bdb(x, D, rule=ref if pointwise else None)
    sc = np.abs(yo).max()
    assert np.abs(O.spmv(rp, ci, va, x) - yo).max() <= 1e-12 * sc
    amf = gpu.BilinearForm(sum(terms[1:], terms[0]), nonassemble=True).Assemble()
    assert np.abs(_apply(gpu, amf, x, torch.float64) - O.spmv(rp, ci, va, x)).max() <= 1e-12 * sc
    z = np.random.default_rng(71).normal(size=fes.ndof)
    Dt = np.ascontiguousarray(np.swapaxes(D.reshape(D.shape[:-1] + (4, 4)), -1, -2).reshape(D.shape))
    Ax = O.spmv(rp, ci, va, x)
    lhs, rhs = z @ Ax, x @ S.apply_bdb(z, Dt, rule=ref if pointwise else None)
    assert abs(lhs - rhs) <= 1e-11 * np.linalg.norm(z) * np.linalg.norm(Ax)


def _csr_T_apply(rp, ci, va, x):
    """(CSR)^T x on the host."""
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    y = np.zeros(len(rp) - 1)
    np.add.at(y, ci, np.asarray(va) * x[rows])
    return y


@pytest.mark.parametrize("hexes,p,pointwise", [(True, 3, False), (True, 2, True), (False, 3, False), (False, 2, True)])
def test_bdb_transpose_products(gpu, hexes, p, pointwise):
    """A non-symmetric B^T D B form: MultTrans, MultTransAdd and .T of the
    matrix-free and the assembled operator apply A^T (the form with D^T),
    checked against the transpose of the assembled CSR (1e-12); .T.T is A.  A
    symmetric form's transpose is the operator itself."""
    m = _mesh(hexes, 3 if hexes else 2, 0.1)
    fes = gpu.H1(m, order=p)
    terms = _terms(gpu, fes, m.ne, 80 + p, pointwise)
    form = sum(terms[1:], terms[0])
    acsr = gpu.BilinearForm(form).Assemble()
    rp, ci, va = acsr.mat.CSR()
    x = np.random.default_rng(81).normal(size=fes.ndof)
    yT = _csr_T_apply(rp, ci, va, x)
    yA = O.spmv(rp, ci, va, x)
    sc = np.abs(yT).max()
    assert np.abs(yT - yA).max() > 1e-3 * sc  # the form is not symmetric
    amf = gpu.BilinearForm(form, nonassemble=True).Assemble()
    for mat in (amf.mat, acsr.mat):
        xv = gpu.BaseVector(data=torch.tensor(x, dtype=torch.float64, device="cuda"))
        yv = gpu.BaseVector(fes.ndof)
        mat.MultTrans(1.0, xv, yv)
        assert np.abs(yv.NumPy() - yT).max() <= 1e-12 * sc
        yv.data = x
        mat.MultTransAdd(2.0, xv, yv)
        assert np.abs(yv.NumPy() - (x + 2.0 * yT)).max() <= 1e-12 * (sc + np.abs(x).max())
        yv2 = gpu.BaseVector(fes.ndof)
        mat.T.Mult(xv, yv2)
        assert np.abs(yv2.NumPy() - yT).max() <= 1e-12 * sc
        assert mat.T.T is mat
    u, v = fes.TnT()
    sym = gpu.BilinearForm(fes, nonassemble=True)
    sym += gpu.CoefficientFunction(lognormal(m.ne, 0.5, 3)) * gpu.grad(u) * gpu.grad(v) * gpu.dx
    sym.Assemble()
    assert sym.mat.T is sym.mat


@pytest.mark.parametrize("pointwise,p", [(False, 3), (True, 3), (True, 5)])
def test_bdb_laplace_type_takes_standard_kernels(gpu, pointwise, p, monkeypatch):
    """A generic hex form whose D is diag(mu, K) with K symmetric runs on the
    standard kernels (the autotuned variants; per-element records on affine
    meshes when D is per element) and matches the oracle's B^T D B apply and the
    B^T D B kernel itself (GH1_BDB_STANDARD=0).  Per point: (1 + x) grad.grad +
    K grad.grad + r u v from the front end; per element: D set through the C ABI."""
    m = _mesh(True, 3, 0.0)
    fes = gpu.H1(m, order=p, dirichlet=".*")
    u, v = fes.TnT()
    rng = np.random.default_rng(90)
    A = rng.normal(size=(3, 3)) * 0.2
    Ks = np.eye(3) + A @ A.T
    kap = (1.0 + gpu.x) if pointwise else gpu.CoefficientFunction(lognormal(m.ne, 0.5, 91))
    terms = [kap * gpu.grad(u) * gpu.grad(v) * gpu.dx,
             gpu.InnerProduct(gpu.CoefficientFunction(Ks) * gpu.grad(u), gpu.grad(v)) * gpu.dx,
             gpu.CoefficientFunction(rng.uniform(0.5, 2.0, m.ne)) * u * v * gpu.dx]
    ref, xyz = _rule(gpu, fes)
    D = _oracle_D(terms, m.ne, xyz if pointwise else None)
    S = O.OracleSpace(m.points, m.elements, p)
    x = np.random.default_rng(92).normal(size=fes.ndof)
    yo = S.apply_bdb(x, D, rule=ref if pointwise else None)
    sc = np.abs(yo).max()

    def make():
        if pointwise:
            return gpu.BilinearForm(sum(terms[1:], terms[0]), nonassemble=True, precision="fp32").Assemble().mat, None
        ctx = fes.ctx
        h = ctypes.c_void_p()
        ctx.check(ctx.lib.gh1_form_create(fes.h, None, None, _lib.GH1_MEM_HOST, ctypes.byref(h)))
        Dc = np.ascontiguousarray(D, dtype=np.float64)
        ctx.check(ctx.lib.gh1_form_set_bdb(h, Dc.ctypes.data_as(ctypes.c_void_p), 0, _lib.GH1_MEM_HOST))
        op = ctypes.c_void_p()
        ctx.check(ctx.lib.gh1_matfree_create(h, 3, ctypes.byref(op)))
        ctx.lib.gh1_form_free(h)  # the operator keeps the form alive
        return C.BilinearFormApplication(ctx, op, fes.ndof, fes), None

    class _A:
        pass
    for standard in (True, False):
        if not standard:
            monkeypatch.setenv("GH1_BDB_STANDARD", "0")
        mat, _ = make()
        a = _A()
        a.mat = mat
        info = mat.Info()["hex_variant_fp64"]
        assert (info in (0, 1)) if standard else (info in (7, 8))
        assert np.abs(_apply(gpu, a, x, torch.float64) - yo).max() <= 1e-12 * sc
        assert np.abs(_apply(gpu, a, x, torch.float32) - yo).max() <= 2e-5 * sc
    monkeypatch.delenv("GH1_BDB_STANDARD")
