"""Host logic of the Python front end (no GPU): coefficient parsing and the
classification of integrands into the forms the library runs."""
import numpy as np
import pytest
import torch

from ngsolve_gb300 import comp as C


class _Space:  # the proxies need the element count, a LinearForm the DOF count
    ne = 4
    ndof = 8


def _uv():
    fes = _Space()
    return C._Proxy(fes, False), C._Proxy(fes, True)


def test_scalar_and_elementwise_coefficients():
    cf = C.CoefficientFunction(2.5)
    assert np.array_equal(cf.element_values(4), np.full(4, 2.5))
    v = np.arange(4.0)
    assert np.array_equal(C.CoefficientFunction(v).element_values(4), v)
    with pytest.raises(ValueError):
        C.CoefficientFunction(np.arange(3.0)).element_values(4)


def test_tensor_coefficients():
    """dims=(3, 3) takes 9 row-major entries, scalar or per element; the tensor
    goes to the library as (xx yy zz xy xz yz); non-symmetric tensors and
    tensors used as scalars are rejected; a tuple of 3 arrays stays a vector."""
    K = C.CoefficientFunction((1, 0.5, 0.2, 0.5, 2, 0.1, 0.2, 0.1, 3), dims=(3, 3))
    assert K.is_tensor()
    assert np.array_equal(K.tensor_values(4), np.tile([1, 2, 3, 0.5, 0.2, 0.1], (4, 1)))
    a = np.arange(1.0, 5.0)
    Ke = C.CoefficientFunction((a, 0, 0, 0, 2 * a, 0, 0, 0, 3), dims=(3, 3))
    t = Ke.tensor_values(4)
    assert np.array_equal(t[:, 0], a) and np.array_equal(t[:, 1], 2 * a) and np.all(t[:, 2] == 3)
    assert C.CoefficientFunction(np.eye(3)[None].repeat(4, 0)).is_tensor()
    with pytest.raises(ValueError):
        C.CoefficientFunction(np.array([[1, 2, 0], [0, 1, 0], [0, 0, 1.0]])).tensor_values(4)
    with pytest.raises(ValueError):
        K.element_values(4)
    with pytest.raises(ValueError):
        C.CoefficientFunction((1, 2, 3), dims=(3, 3))
    assert not C.CoefficientFunction((a, a, a)).is_tensor()
    with pytest.raises(ValueError):
        C.CoefficientFunction(np.eye(3)[None].repeat(3, 0)).tensor_values(4)


def test_classify_integrands():
    u, v = _uv()
    kap = np.arange(1.0, 5.0)
    kind, coef = (C.CoefficientFunction(kap) * C.grad(u) * C.grad(v) * C.dx).classify(4)
    assert kind == "laplace" and np.array_equal(coef, kap)
    kind, coef = (3.0 * C.InnerProduct(C.grad(u), C.grad(v)) * C.dx).classify(4)
    assert kind == "laplace" and np.all(coef == 3.0)
    kind, coef = (C.InnerProduct(u, v) * C.dx).classify(4)
    assert kind == "mass" and np.all(coef == 1.0)
    kind, coef = (C.CoefficientFunction(kap) * v * C.dx).classify(4)
    assert kind == "source" and np.array_equal(coef, kap)
    K = C.CoefficientFunction(np.diag([1.0, 2.0, 3.0]))
    kind, coef = (C.CoefficientFunction(kap) * C.InnerProduct(K * C.grad(u), C.grad(v)) * C.dx).classify(4)
    assert kind == "laplace_tensor" and coef.shape == (4, 6)
    assert np.array_equal(coef[:, 1], 2 * kap) and np.all(coef[:, 3:] == 0)
    with pytest.raises(ValueError):  # no measure
        (C.grad(u) * C.grad(v)).classify(4)
    with pytest.raises(NotImplementedError):  # a tensor outside the diffusion term
        (K * u * v * C.dx).classify(4)
    with pytest.raises(NotImplementedError):  # two trial functions
        (C.grad(u) * C.grad(u) * C.dx).classify(4)
    with pytest.raises(TypeError):
        C.grad(2.0)


def test_vector_space_rejects_tensor_term():
    """On VectorH1, K * grad(u) multiplies the Jacobian of u and couples the
    components, so the block-diagonal operator cannot represent it."""
    class _Vec(C.VectorH1):
        def __init__(self):  # no GPU space: only what BilinearForm reads
            self.scalar, self.dim, self.ne, self.ndof = _Space(), 3, 4, 12
    fes = _Vec()
    u, v = C._Proxy(fes, False), C._Proxy(fes, True)
    a = C.BilinearForm(fes)
    a += C.InnerProduct(C.grad(u), C.grad(v)) * C.dx
    with pytest.raises(NotImplementedError):
        a += C.InnerProduct(C.CoefficientFunction(np.eye(3)) * C.grad(u), C.grad(v)) * C.dx


def test_dirichlet_regex_resolution():
    """None (the all-or-nothing flag) for no Dirichlet boundary, a regex that
    matches every name, or a mesh without names; else the matched faces."""
    from ngsolve_gb300.meshes import MakeStructured3DMesh, Mesh
    m = MakeStructured3DMesh(hexes=True, nx=2)
    assert C._dirichlet_faces(m, "") is None and C._dirichlet_faces(m, ".*") is None
    assert C._dirichlet_faces(m, "back|left|front|right|bottom|top") is None
    f = C._dirichlet_faces(m, "left|top")
    assert f.shape == (8, 4) and f.dtype == np.int32
    assert C._dirichlet_faces(m, "nothing").shape == (0, 4)
    assert C._dirichlet_faces(Mesh(m.points, m.elements), "left") is None
    # 1-based boundary-condition numbers, as in H1(mesh, dirichlet=[1, 2, 3, 4])
    assert np.array_equal(C._dirichlet_faces(m, [2, 6]), f)
    assert C._dirichlet_faces(m, [1, 2, 3, 4, 5, 6]) is None and C._dirichlet_faces(m, []) is None
    assert C._no_dirichlet([]) and C._no_dirichlet("") and not C._no_dirichlet(".*") and not C._no_dirichlet([1])
    with pytest.raises(ValueError):
        C._dirichlet_faces(m, [0])
    with pytest.raises(TypeError):
        C._dirichlet_faces(m, ["left"])
    with pytest.raises(TypeError):
        C._dirichlet_faces(m, 3)


def test_vector_gridfunction_components():
    """gfu.components on VectorH1 are views of the component blocks (host
    tensors stand in for device vectors here)."""
    import torch

    class _Vec(C.VectorH1):
        def __init__(self):  # no GPU space: only what GridFunction reads
            self.scalar, self.dim, self.ne, self.ndof = _Space(), 3, 4, 12
            self.scalar.ndof = 4
    fes = _Vec()
    g = C.GridFunction(fes, vec=C.BaseVector(data=torch.arange(12.0)))
    comps = g.components
    assert len(comps) == 3 and all(c.fes is fes.scalar for c in comps)
    assert torch.equal(comps[1].vec.t, torch.tensor([4.0, 5, 6, 7]))
    comps[2].vec.t[:] = -1.0
    assert torch.all(g.vec.t[8:] == -1.0) and torch.all(g.vec.t[:8] >= 0)
    with pytest.raises(TypeError):
        C.GridFunction(_Space(), vec=C.BaseVector(data=torch.zeros(4))).components


def test_vector_inner_product_and_norm():
    """InnerProduct / Norm of vectors are numbers; of proxies, integrands."""
    import torch
    x = C.BaseVector(data=torch.tensor([1.0, 2.0, 2.0]))
    y = C.BaseVector(data=torch.tensor([3.0, 0.0, -1.0]))
    assert C.InnerProduct(x, y) == 1.0 and C.InnerProduct(x, torch.tensor([1.0, 1.0, 1.0])) == 5.0
    assert C.Norm(x) == 3.0
    u, v = _uv()
    assert isinstance(C.InnerProduct(u, v), C._Product)


def test_inverse_operator_plumbing(monkeypatch):
    """a.mat.Inverse(freedofs) * f: one CG solve per product (a dense host
    stand-in replaces the GPU solver here), scaled, added, zero on non-free
    rows; a solve that stops above tol raises."""
    import torch
    from ngsolve_gb300 import solvers as SV

    A = torch.tensor([[4.0, 1, 0], [1, 3, 1], [0, 1, 2]])
    free = torch.tensor([True, True, False])

    class _Mat:
        height = width = 3

        def CreateSmoother(self, freedofs=None):
            return ("jacobi", freedofs)

        def CreateVector(self):
            return C.BaseVector(data=torch.zeros(3))

    calls = []

    class _Solver:
        def __init__(self, mat, pre, tol, maxiter):
            self.pre, self.tol = pre, tol
            self.iterations = 7
            self.result = type("R", (), {"status": 6 if tol > 1 else 0})()

        def Solve(self, rhs, sol, initialize):
            calls.append((self.pre, self.tol, initialize))
            Af = A[free][:, free]
            out = torch.zeros(3)
            out[free] = torch.linalg.solve(Af, rhs.t[free])
            sol.t.copy_(out)

    monkeypatch.setattr(SV, "CGSolver", _Solver)
    mat = _Mat()
    inv = C.BaseMatrix.Inverse(mat, freedofs=[1, 1, 0], inverse="sparsecholesky")
    f = C.BaseVector(data=torch.tensor([1.0, 2.0, 3.0]))
    x = C.BaseVector(data=torch.zeros(3))
    x.data = inv * f
    expect = torch.zeros(3)
    expect[free] = torch.linalg.solve(A[free][:, free], f.t[free])
    assert torch.allclose(x.t, expect) and x.t[2] == 0
    assert calls[-1] == (("jacobi", [1, 1, 0]), 1e-12, True) and inv.iterations == 7
    x.data = 2.0 * (inv * f)
    assert torch.allclose(x.t, 2 * expect)
    inv.MultAdd(-1.0, f, x)
    assert torch.allclose(x.t, expect)
    assert inv.T is inv and inv.shape == (3, 3)
    with pytest.raises(ValueError):
        C.BaseMatrix.Inverse(mat, inverse="magic")
    from ngsolve_gb300._lib import GH1Error
    with pytest.raises(GH1Error):
        C.InverseOperator(mat, tol=10.0).Mult(f, x)


def test_coupling_free_dofs():
    """FreeDofs(coupling=True) drops the element-interior DOFs, numbered last,
    and keeps the rest of the mask; the oracle's numbering agrees."""
    from oracle import oracle as O
    from ngsolve_gb300.meshes import MakeStructured3DMesh
    for hexes, p in ((True, 3), (False, 4), (False, 3), (True, 1)):
        m = MakeStructured3DMesh(hexes=hexes, nx=2)
        S = O.OracleSpace(m.points, m.elements, p)
        free = S.freedofs().astype(bool)
        ext = C._coupling_mask(free, S.ne, m.et, p)
        cell = np.zeros(S.ndof, dtype=bool)
        cell[S.first_cell:] = True
        assert np.array_equal(ext, free & ~cell)


def test_bilinearform_flags():
    """Flags that would change the operator raise unless at their default;
    unrelated flags pass; the precision is checked."""
    fes = _Space()
    for flag in ("condense", "eliminate_internal", "symmetric_storage", "diagonal", "hermitian"):
        with pytest.raises(NotImplementedError):
            C.BilinearForm(fes, **{flag: True})
        C.BilinearForm(fes, **{flag: False})
    C.BilinearForm(fes, check_unused=False, printelmat=False)
    with pytest.raises(ValueError):
        C.BilinearForm(fes, precision="bf16")


def test_space_flags():
    C._check_space_flags({"complex": False, "dgjumps": False, "autoupdate": True})
    with pytest.raises(NotImplementedError):
        C._check_space_flags({"complex": True})
    with pytest.raises(TypeError):
        C._check_space_flags({"orderinner": 2})


def test_script_boilerplate():
    import ngsolve_gb300 as ng
    ng.SetHeapSize(10 * 1000 * 1000)
    ng.SetNumThreads(4)
    with ng.TaskManager(pajetrace=10 ** 8) as tm:
        assert isinstance(tm, ng.TaskManager)


def test_tutorial_idioms(monkeypatch):
    """The idioms of NGSolve's CUDA Poisson tutorial (docs/i-tutorials/
    unit-5.5-cuda/poisson_cuda.ipynb) on host stand-ins for the GPU parts:
    forms built from integrand sums, CGSolver as an operator with GetSteps,
    (inv * f).Evaluate(), Norm of a vector difference, CreateDeviceVector /
    CreateDeviceMatrix."""
    import torch
    from ngsolve_gb300 import solvers as SV

    class _HostVec(C.BaseVector):
        def __init__(self, n=None, data=None, dtype=torch.float64, device=0):
            self.t = data if data is not None else torch.zeros(int(n), dtype=dtype)

    monkeypatch.setattr(C, "BaseVector", _HostVec)
    u, v = _uv()
    a = C.BilinearForm(C.grad(u) * C.grad(v) * C.dx + u * v * C.dx)
    assert a.fes is u.fes and np.all(a.kappa == 1.0) and np.all(a.mu == 1.0)
    b = C.BilinearForm(u.fes)
    b += C.grad(u) * C.grad(v) * C.dx - 2.0 * u * v * C.dx
    assert np.all(b.kappa == 1.0) and np.all(b.mu == -2.0)
    lf = C.LinearForm(C.CoefficientFunction(3.0) * v * C.dx + C.CoefficientFunction(1.0) * v * C.dx)
    assert lf.fes is u.fes and np.all(lf.f == 4.0)
    with pytest.raises(ValueError):
        C.BilinearForm(C.CoefficientFunction(1.0) * C.dx)

    A = torch.tensor([[4.0, 1, 0], [1, 3, 1], [0, 1, 2]], dtype=torch.float64)

    class _Mat:
        height = width = 3

        def CreateVector(self):
            return _HostVec(3)

        def GetOperatorInfo(self):
            return "A\n"

    def _solve(self, rhs, sol=None, initialize=True):
        sol.t.copy_(torch.linalg.solve(A, rhs.t))
        self.iterations = 5
        return sol

    monkeypatch.setattr(SV.CGSolver, "Solve", _solve)
    inv = SV.CGSolver(_Mat(), None, maxiter=2000, printrates=False)
    assert inv.CreateDeviceMatrix() is inv and "CGSolver" in inv.GetOperatorInfo()
    f = _HostVec(data=torch.tensor([1.0, 2.0, 3.0], dtype=torch.float64))
    fdev = f.CreateDeviceVector(copy=True)
    assert torch.equal(fdev.t, f.t) and fdev.t.data_ptr() != f.t.data_ptr()
    assert torch.all(f.CreateDeviceVector(copy=False).t == 0)
    res = (inv * fdev).Evaluate()
    assert inv.GetSteps() == 5
    assert C.Norm(res - _HostVec(data=torch.linalg.solve(A, f.t))) < 1e-12
    assert abs(C.InnerProduct(res, f) - float(res.t @ f.t)) < 1e-12
    gfu = _HostVec(3)
    gfu.data = 2.0 * (inv * f)
    assert torch.allclose(gfu.t, 2 * torch.linalg.solve(A, f.t))


def test_coordinate_sources(monkeypatch):
    """x, y, z and their affine combinations: classified as affine sources,
    accumulated by the LinearForm, assembled as M I_h(f) (a dense host mass
    matrix stands in for the GPU operator); other uses are rejected."""
    import torch
    f = 2 * C.x - C.y + 3
    assert np.array_equal(f.a, [2, -1, 0]) and f.d == 3.0
    assert np.array_equal((1 - C.z).a, [0, 0, -1]) and (1 - C.z).d == 1.0
    u, v = _uv()
    kind, val = (2.0 * C.x * v * C.dx).classify(4)
    assert kind == "source_affine" and np.array_equal(val, [2, 0, 0, 0])
    with pytest.raises(NotImplementedError):
        (C.x * C.grad(u) * C.grad(v) * C.dx).classify(4)
    with pytest.raises(NotImplementedError):
        (C.CoefficientFunction(np.arange(4.0)) * C.x * v * C.dx).classify(4)
    with pytest.raises(ValueError):
        C.x.element_values(4)

    pts = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0]])
    Md = torch.tensor(np.diag([1.0, 2, 3, 4, 5]))

    class _Mesh:
        raw = type("R", (), {"points": pts})()

    class _Fes(_Space):
        ndof, mesh = 5, _Mesh()

        def TnT(self):
            return C._Proxy(self, False), C._Proxy(self, True)

    class _Form:
        def __init__(self, fes, nonassemble=False):
            self.terms = []

        def __iadd__(self, t):
            self.terms.append(t.classify(4)[0])
            return self

        def Assemble(self):
            assert self.terms == ["mass"]
            self.mat = type("M", (), {"MultAdd": staticmethod(lambda s, xv, yv: yv.t.add_(s * (Md @ xv.t)))})()
            return self

    monkeypatch.setattr(C, "BilinearForm", _Form)
    lf = type("LF", (), {})()
    lf.fes, lf._mass = _Fes(), None
    lf.vec = C.BaseVector(data=torch.ones(5, dtype=torch.float64))
    C._affine_source(lf, f)
    fi = np.array([3.0, 5.0, 2.0, 0, 0])
    assert np.allclose(lf.vec.t.numpy(), 1.0 + np.diag(Md.numpy()) * fi)
    mass = lf._mass
    C._affine_source(lf, C.x)  # the mass operator is built once
    assert lf._mass is mass


def test_gridfunction_set():
    """Set(f) for constant / affine f writes the interpolant (vertex values, zero
    elsewhere); Set(f, BND) touches only the boundary DOFs; other
    coefficients are rejected (host stand-ins for the GPU space)."""
    import torch
    pts = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0], [0.5, 0.5, 0.5]])
    fes = C.H1.__new__(C.H1)
    fes.mesh = type("M", (), {"raw": type("R", (), {"points": pts})()})()
    fes.ndof = 7
    fes._bnd_dofs = np.array([1, 1, 1, 0, 1, 0, 0], dtype=bool)  # vertex 3 and DOFs 5, 6 interior
    g = C.GridFunction(fes, vec=C.BaseVector(data=torch.arange(7.0, dtype=torch.float64)))
    g.Set(2 * C.x + 1)
    assert np.array_equal(g.vec.NumPy(), [1, 3, 1, 2, 0, 0, 0])
    g.vec.t.copy_(torch.arange(7.0, dtype=torch.float64))
    g.Set(C.y - 1, C.BND)
    assert np.array_equal(g.vec.NumPy(), [-1, -1, 0, 3, 0, 5, 6])
    g.Set(C.CoefficientFunction(4.0))
    assert np.array_equal(g.vec.NumPy(), [4, 4, 4, 4, 0, 0, 0])
    with pytest.raises(NotImplementedError):
        g.Set(C.CoefficientFunction(np.arange(4.0)))
    with pytest.raises(ValueError):
        g.Set(C.x, "SURFACE")


def test_integrate(monkeypatch):
    """Integrate on host stand-ins: grad(a)*grad(b) element-wise through the
    element kernel's entry (summed when not element-wise); totals of products
    and single factors as a^T M b with the mass operator (a dense host matrix
    here), affine / constant factors as their interpolants; the rest raises."""
    import torch
    pts = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0]])
    M = torch.tensor(np.diag([1.0, 2, 3, 4]), dtype=torch.float64)

    class _Fes(_Space):
        ndof = 4
        mesh = type("M", (), {"raw": type("R", (), {"points": pts})()})()

        def TnT(self):
            return C._Proxy(self, False), C._Proxy(self, True)

    class _Form:
        def __init__(self, fes, nonassemble=False):
            pass

        def __iadd__(self, t):
            return self

        def Assemble(self):
            self.mat = type("Mat", (), {"Mult": staticmethod(lambda xv, yv: yv.t.copy_(M @ xv.t))})()
            return self

    seen = []

    def _gd(fes, u, w):
        seen.append((u, w))
        return torch.tensor([1.0, 2.0, 3.0, 4.0], dtype=torch.float64)

    monkeypatch.setattr(C, "BilinearForm", _Form)
    monkeypatch.setattr(C, "Integrate_grad_dot", _gd)
    fes = _Fes()
    a = C.GridFunction(fes, vec=C.BaseVector(data=torch.tensor([1.0, 1, 1, 1], dtype=torch.float64)))
    b = C.GridFunction(fes, vec=C.BaseVector(data=torch.tensor([0.0, 1, 2, 3], dtype=torch.float64)))
    per = C.Integrate(C.grad(a) * C.grad(b), None, element_wise=True)
    assert torch.equal(per, torch.tensor([1.0, 2, 3, 4], dtype=torch.float64)) and seen[-1] == (a.vec, b.vec)
    assert C.Integrate(C.grad(a) * C.grad(b), None) == 10.0
    assert C.Integrate(a * b, None) == float(a.vec.t @ M @ b.vec.t)        # 0 + 2 + 6 + 12 = 20
    assert C.Integrate(b, None) == float(b.vec.t @ M @ torch.tensor([1.0, 1, 1, 0], dtype=torch.float64))
    xi = torch.tensor([0.0, 1, 0, 0], dtype=torch.float64)                  # x at the vertices, 0 elsewhere
    assert C.Integrate(C.x * a, None) == float(xi @ M @ a.vec.t) == C.Integrate(a * C.x, None)
    assert C.Integrate(2.0 * a, None) == float(a.vec.t @ M @ (2 * torch.tensor([1.0, 1, 1, 0], dtype=torch.float64)))
    with pytest.raises(NotImplementedError):
        C.Integrate(a * b, None, element_wise=True)
    with pytest.raises(NotImplementedError):
        C.Integrate(C.x, None)
    with pytest.raises(TypeError):
        a * C.CoefficientFunction(np.arange(4.0))


def test_cg_rejects_unknown_keywords():
    """CGSolver takes the reference's keywords (plotrates, printing, maxsteps
    ...) and raises on any other, before it touches a device."""
    from ngsolve_gb300 import solvers as SV

    class _Mat:
        height = width = 3

    s = SV.CGSolver(_Mat(), None, maxsteps=7, plotrates=True, printing=False)
    assert s.maxiter == 7
    with pytest.raises(TypeError):
        SV.CGSolver(_Mat(), None, plotrate=True)
    with pytest.raises(TypeError):
        SV.CG(_Mat(), None, pre=None, maxstep=10)
    with pytest.raises(ValueError):
        SV.CGSolver(_Mat(), None, mode="fp16")
    with pytest.raises(NotImplementedError):
        SV.CGSolver(_Mat(), None, atol=1e-12)


def test_integrate_rejects_bad_operands(monkeypatch):
    """Integrate(grad(a)*grad(b)) checks its operands before the element
    kernel reads fes.ndof doubles through each pointer: same space, scalar H1,
    contiguous FP64 CUDA vectors of the space's length.  A coefficient times a
    VectorH1 function raises instead of integrating one component."""
    import torch

    class _Fes(_Space):
        ndof = 4

    fes, other = _Fes(), _Fes()
    a = C.GridFunction(fes, vec=C.BaseVector(data=torch.ones(4, dtype=torch.float64)))
    b = C.GridFunction(other, vec=C.BaseVector(data=torch.ones(4, dtype=torch.float64)))
    with pytest.raises(ValueError):
        C.Integrate(C.grad(a) * C.grad(b), None, element_wise=True)
    with pytest.raises(TypeError):  # host tensors never reach the kernel
        C.Integrate_grad_dot(fes, a.vec, a.vec)
    with pytest.raises(TypeError):
        C.Integrate_grad_dot(fes, torch.ones(4, dtype=torch.float32), torch.ones(4, dtype=torch.float32))
    vfes = object.__new__(C.VectorH1)
    with pytest.raises(TypeError):
        C.Integrate_grad_dot(vfes, a.vec, a.vec)
    vf = C.GridFunction(_Fes(), vec=C.BaseVector(data=torch.ones(4, dtype=torch.float64)))
    vf.fes = vfes
    with pytest.raises(NotImplementedError):
        C.Integrate(2.0 * vf, None)
    with pytest.raises(NotImplementedError):
        C.Integrate(C.x * vf, None)


def test_generic_bdb_terms():
    """Terms outside kappa grad.grad / mu u v / symmetric K go into the generic
    B^T D B matrix (rows test (v, grad v), columns trial (u, grad u)): convection
    b . grad(u) v in row 0, its transpose u (b . grad v) in column 0, a
    non-symmetric K in the gradient block; a coordinate factor makes D point-wise."""
    u, v = _uv()
    ne = 4
    kap = np.arange(1.0, 5.0)
    b = C.CoefficientFunction((kap, 2.0, -1.0))
    Kn = np.array([[1.0, 0.5, 0.0], [0.0, 2.0, 0.0], [0.3, 0.0, 3.0]])
    terms = [C.CoefficientFunction(kap) * C.grad(u) * C.grad(v) * C.dx,
             C.InnerProduct(b, C.grad(u)) * v * C.dx,
             3.0 * u * C.InnerProduct(C.CoefficientFunction((0.0, 1.0, 0.0)), C.grad(v)) * C.dx,
             C.InnerProduct(C.CoefficientFunction(Kn) * C.grad(u), C.grad(v)) * C.dx,
             2.0 * u * v * C.dx]
    assert all(C._bdb_needed(t) for t in terms[1:4]) and not C._bdb_needed(terms[0])
    D = C._bdb_D(terms, ne, None, torch.device("cpu"))
    assert D.shape == (ne, 1, 4, 4)
    D = D[:, 0].numpy()
    assert np.allclose(D[:, 0, 0], 2.0)
    assert np.allclose(D[:, 0, 1], kap) and np.allclose(D[:, 0, 2], 2.0) and np.allclose(D[:, 0, 3], -1.0)
    assert np.allclose(D[:, 1:, 0], [0.0, 3.0, 0.0])
    assert np.allclose(D[:, 1:, 1:], kap[:, None, None] * np.eye(3) + Kn)
    # point-wise: x * u * v at two points per element
    pts = torch.tensor(np.random.default_rng(1).uniform(size=(ne, 2, 3)))
    Dp = C._bdb_D([C.x * u * v * C.dx], ne, pts, torch.device("cpu")).numpy()
    assert Dp.shape == (ne, 2, 4, 4) and np.allclose(Dp[:, :, 0, 0], pts[..., 0].numpy())
    assert C._is_pointwise(C.CoefficientFunction((C.y, 0.0, 0.0)))
    # shapes the generic form cannot take
    with pytest.raises(NotImplementedError):
        C._bdb_parts(b * C.grad(u) * C.grad(v) * C.dx)   # a vector with two gradients
    with pytest.raises(NotImplementedError):
        C._bdb_parts(C.CoefficientFunction(Kn) * C.grad(u) * v * C.dx)
    with pytest.raises(NotImplementedError):
        C._bdb_parts(u * u * C.dx)
    with pytest.raises(ValueError):
        C._bdb_parts(u * C.grad(v))
