"""Python front end mirroring the NGSolve objects on the H1 operator path.

    mesh = Mesh(MakeStructured3DMesh(hexes=True, nx=16))
    fes = H1(mesh, order=3, dirichlet=".*")
    u, v = fes.TnT()
    a = BilinearForm(fes)
    a += CoefficientFunction(kappa) * grad(u) * grad(v) * dx
    a.Assemble()                           # a.mat: SparseMatrix on the GPU
    f = LinearForm(fes); f += CoefficientFunction(fe) * v * dx; f.Assemble()
    pre = a.mat.CreateSmoother(fes.FreeDofs())
    gfu = GridFunction(fes)
    gfu.vec.data = solvers.CG(mat=a.mat, rhs=f.vec, pre=pre, tol=1e-10, maxsteps=1000)

Names, argument meanings and error behaviour follow comp/python_comp.cpp
(BilinearForm :2800-3060, LinearForm, GridFunction), linalg/python_linalg.cpp
(BaseMatrix.Mult/MultAdd :1072-1073, CreateSmoother :1220) and
python/krylovspace.py (solvers.CG).  Coefficients are per-element constants
(an order-0 L2 GridFunction in the reference's adjoint tutorial).  Every
numerical call goes to libgh1.so on the GPU; there is no CPU path.
"""
import ctypes
import weakref

import numpy as np
import torch

from . import _lib
from .meshes import Mesh as _RawMesh

_contexts = {}


class Context:
    """One gh1 context per CUDA device; work runs on torch's current stream."""

    def __init__(self, device=0):
        if not torch.cuda.is_available():
            raise _lib.GH1Error(2, "no CUDA device available (the H1 engine has no CPU fallback)")
        self.lib = _lib.load()
        self.device = device
        h = ctypes.c_void_p()
        rc = self.lib.gh1_create(ctypes.byref(h), device)
        if rc != 0:
            msg = self.lib.gh1_last_error(h) if h.value else b"gh1_create failed"
            raise _lib.GH1Error(rc, msg.decode())
        self.h = h

    def sync_stream(self):
        s = torch.cuda.current_stream(self.device).cuda_stream
        self.lib.gh1_set_stream(self.h, ctypes.c_void_p(s))
        return self

    def check(self, rc):
        _lib.check(rc, self.h)


def context(device=0):
    if device not in _contexts:
        _contexts[device] = Context(device)
    return _contexts[device].sync_stream()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _np_ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


# ---------------------------------------------------------------------------
class Mesh:
    """Uploaded volume mesh (tets or hexes) -- ngsolve.Mesh for the H1 path."""

    def __init__(self, mesh, device=0):
        if not isinstance(mesh, _RawMesh):
            raise TypeError("Mesh expects a meshes.Mesh (points + element vertex lists)")
        self.raw = mesh
        self.device = device
        self.ctx = context(device)
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.gh1_mesh_upload(self.ctx.h, mesh.nv, _np_ptr(mesh.points), mesh.ne, mesh.et,
                                                    _np_ptr(mesh.elements), ctypes.byref(h)))
        self.h = h

    @property
    def ne(self):
        return self.raw.ne

    @property
    def nv(self):
        return self.raw.nv

    def SetDeformation(self, gf):
        """MeshAccess::SetDeformation (comp/meshaccess.cpp:1573-1580): gf is a
        GridFunction of VectorH1(mesh, order=k) whose values displace the mesh;
        forms assembled afterwards integrate over the deformed (curved) elements."""
        fes = gf.fes
        if not isinstance(fes, VectorH1) or fes.dim != 3 or fes.mesh is not self:
            raise ValueError("SetDeformation needs a GridFunction of VectorH1(mesh, dim=3) on this mesh")
        v = gf.vec.t
        if v.dtype != torch.float64 or not v.is_cuda or not v.is_contiguous() or v.numel() != fes.ndof:
            raise TypeError("the deformation vector must be a contiguous CUDA float64 vector of the space's size")
        self.ctx.sync_stream()
        # the values are copied; the library borrows the field's space, so the
        # deformation lasts while the GridFunction's space does
        self.ctx.check(self.ctx.lib.gh1_mesh_set_deformation(self.h, fes.scalar.h, _ptr(v), _lib.GH1_MEM_DEVICE))

    def UnsetDeformation(self):
        self.ctx.check(self.ctx.lib.gh1_mesh_set_deformation(self.h, None, None, _lib.GH1_MEM_HOST))

    def __del__(self):
        try:
            self.ctx.lib.gh1_mesh_free(self.h)
        except Exception:
            pass


class BitArray(np.ndarray):
    """Free-DOF mask (bool per DOF), the role of ngstd BitArray."""


# ---------------------------------------------------------------------------
# symbolic placeholders for the two integrators on the path
class _Proxy:
    def __init__(self, fes, test):
        self.fes, self.test = fes, test

    def __mul__(self, other):
        return _Product.of(self, other)

    __rmul__ = __mul__


class _Grad:
    def __init__(self, proxy):
        self.proxy = proxy

    def __mul__(self, other):
        return _Product.of(self, other)

    __rmul__ = __mul__


def grad(u):
    if isinstance(u, GridFunction):
        return _GFGrad(u)
    if not isinstance(u, _Proxy):
        raise TypeError("grad() expects a trial or test function or a GridFunction")
    return _Grad(u)


class _GFGrad:
    """grad(gfu) of a GridFunction: for Integrate(grad(a) * grad(b), mesh)."""

    def __init__(self, gf):
        self.gf = gf

    def __mul__(self, other):
        if isinstance(other, _GFGrad):
            return _GFIntegrand("graddot", self.gf, other.gf)
        raise NotImplementedError("grad(gfu) multiplies grad(gfu) only")


class CoefficientFunction:
    """Piecewise-constant coefficient: one value per element (or a scalar); a
    tuple of such values is a vector (VectorH1 sources); a 3x3 matrix -- an
    ndarray of shape (3, 3) or (ne, 3, 3), or 9 entries with dims=(3, 3) as in
    NGSolve -- is a diffusion tensor for InnerProduct(K * grad(u), grad(v))."""

    def __init__(self, values, dims=None):
        if dims is not None:
            if tuple(dims) != (3, 3) or len(values) != 9:
                raise ValueError("matrix coefficients are 3x3: 9 entries with dims=(3, 3)")
            values = np.moveaxis(np.array(np.broadcast_arrays(*[np.asarray(v, dtype=np.float64) for v in values])),
                                 0, -1).reshape(np.shape(np.broadcast(*values)) + (3, 3))
        self.values = values

    def is_tensor(self):
        return isinstance(self.values, np.ndarray) and self.values.ndim in (2, 3) and self.values.shape[-2:] == (3, 3)

    def tensor_values(self, ne):
        """(ne, 6): xx yy zz xy xz yz of the symmetric tensor on each element."""
        K = np.asarray(self.values, dtype=np.float64)
        if K.ndim == 2:
            K = np.broadcast_to(K, (ne, 3, 3))
        if K.shape != (ne, 3, 3):
            raise ValueError("element-wise tensor needs shape (%d, 3, 3), got %s" % (ne, K.shape))
        if np.abs(K - K.transpose(0, 2, 1)).max() > 1e-12 * max(np.abs(K).max(), 1e-300):
            raise ValueError("the diffusion tensor must be symmetric")
        return np.ascontiguousarray(np.stack([K[:, 0, 0], K[:, 1, 1], K[:, 2, 2], K[:, 0, 1], K[:, 0, 2], K[:, 1, 2]],
                                             axis=1))

    def element_values(self, ne):
        if self.is_tensor():
            raise ValueError("a matrix coefficient goes into InnerProduct(K * grad(u), grad(v))")
        v = np.asarray(self.values, dtype=np.float64)
        if v.ndim == 0:
            return np.full(ne, float(v))
        if v.shape != (ne,):
            raise ValueError("element-wise coefficient needs %d values, got %s" % (ne, v.shape))
        return np.ascontiguousarray(v)

    def __mul__(self, other):
        if isinstance(other, GridFunction):
            return NotImplemented
        return _Product.of(self, other)

    __rmul__ = __mul__


class _AffineCF(CoefficientFunction):
    """a.x + b.y + c.z + d in physical coordinates: the coordinate functions x,
    y, z and their affine combinations.  As a source, f*v*dx, it is exactly
    the H1 interpolant of f (vertex values, all other DOFs zero: on affine tets
    and on trilinear hexes the vertex functions reproduce the map), so the load
    vector is M I_h(f) with the mass operator, integrated by the same order-2p
    rule as the right-hand-side kernel."""

    def __init__(self, a=(0.0, 0.0, 0.0), d=0.0):
        self.a, self.d = np.array(a, dtype=np.float64), float(d)
        self.values = None

    def is_tensor(self):
        return False

    def element_values(self, ne):
        raise ValueError("a coordinate function is not constant per element; it enters as f * v * dx")

    def vertex_values(self, points):
        return np.asarray(points, dtype=np.float64) @ self.a + self.d

    def _num(self, other):
        return isinstance(other, (int, float, np.floating, np.integer)) and not isinstance(other, bool)

    def __mul__(self, other):
        if self._num(other):
            return _AffineCF(self.a * other, self.d * other)
        if isinstance(other, GridFunction):
            return NotImplemented
        return _Product.of(self, other)

    __rmul__ = __mul__

    def __add__(self, other):
        if self._num(other):
            return _AffineCF(self.a, self.d + other)
        if isinstance(other, _AffineCF):
            return _AffineCF(self.a + other.a, self.d + other.d)
        return NotImplemented

    __radd__ = __add__

    def __neg__(self):
        return _AffineCF(-self.a, -self.d)

    def __sub__(self, other):
        return self + (-other)

    def __rsub__(self, other):
        return (-self) + other


x = _AffineCF((1.0, 0.0, 0.0))
y = _AffineCF((0.0, 1.0, 0.0))
z = _AffineCF((0.0, 0.0, 1.0))


class _Measure:
    pass


dx = _Measure()


class _Product:
    """kind in {'laplace', 'mass', 'source'} with an element-wise coefficient."""

    def __init__(self, factors):
        self.factors = factors

    @staticmethod
    def of(a, b):
        fa = a.factors if isinstance(a, _Product) else [a]
        fb = b.factors if isinstance(b, _Product) else [b]
        return _Product(fa + fb)

    def __mul__(self, other):
        return _Product.of(self, other)

    __rmul__ = __mul__

    def __neg__(self):
        return _Product(self.factors + [-1.0])

    def __add__(self, other):
        return _Sum([self]) + other

    def __radd__(self, other):
        return _Sum([other]) + self

    def __sub__(self, other):
        return _Sum([self]) + (-other)

    def classify(self, ne):
        grads = [f for f in self.factors if isinstance(f, _Grad)]
        proxies = [f for f in self.factors if isinstance(f, _Proxy)]
        tensors = [f for f in self.factors if isinstance(f, CoefficientFunction) and f.is_tensor()]
        affine = [f for f in self.factors if isinstance(f, _AffineCF)]
        coef = np.ones(ne)
        has_dx = False
        for f in self.factors:
            if isinstance(f, CoefficientFunction) and (f.is_tensor() or isinstance(f, _AffineCF)):
                continue
            if isinstance(f, CoefficientFunction):
                coef = coef * f.element_values(ne)
            elif isinstance(f, (int, float, np.floating)):
                coef = coef * float(f)
            elif isinstance(f, _Measure):
                has_dx = True
        if not has_dx:
            raise ValueError("integrand needs * dx")
        if affine:
            if len(affine) == 1 and len(proxies) == 1 and not grads and proxies[0].test and not tensors:
                if np.ptp(coef) != 0.0:
                    raise NotImplementedError("a coordinate source times an element-wise coefficient")
                f = affine[0] * float(coef[0])
                return "source_affine", np.concatenate([f.a, [f.d]])
            raise NotImplementedError("a coordinate function is only on the path as a source, f * v * dx")
        if tensors:
            if len(tensors) == 1 and len(grads) == 2 and not proxies and grads[0].proxy.test != grads[1].proxy.test:
                return "laplace_tensor", tensors[0].tensor_values(ne) * coef[:, None]
            raise NotImplementedError("a matrix coefficient is only on the path as InnerProduct(K * grad(u), grad(v))")
        if len(grads) == 2 and not proxies and grads[0].proxy.test != grads[1].proxy.test:
            return "laplace", coef
        if len(proxies) == 2 and not grads and proxies[0].test != proxies[1].test:
            return "mass", coef
        if len(proxies) == 1 and not grads and proxies[0].test:
            return "source", coef
        raise NotImplementedError("only kappa*grad(u)*grad(v)*dx, mu*u*v*dx and f*v*dx are on the H1 path")


def _is_vector_cf(f):
    return isinstance(f, CoefficientFunction) and isinstance(f.values, (tuple, list)) and len(f.values) == 3


def _is_pointwise(f):
    """A coefficient that varies inside an element (a coordinate function or a
    vector with such a component)."""
    if isinstance(f, _AffineCF):
        return True
    return _is_vector_cf(f) and any(isinstance(c, _AffineCF) for c in f.values)


def _bdb_needed(term):
    """True when a bilinear term lies outside kappa grad.grad / mu u v / symmetric
    K grad.grad: it then goes into the generic B^T D B form."""
    if not isinstance(term, _Product):
        return False
    fs = term.factors
    grads = [f for f in fs if isinstance(f, _Grad)]
    proxies = [f for f in fs if isinstance(f, _Proxy)]
    if any(_is_pointwise(f) or _is_vector_cf(f) for f in fs):
        return len(grads) + len(proxies) == 2
    if len(grads) == 1 and len(proxies) == 1:
        return True
    for f in fs:
        if isinstance(f, CoefficientFunction) and f.is_tensor():
            K = np.asarray(f.values, dtype=np.float64)
            if np.abs(K - np.swapaxes(K, -1, -2)).max() > 1e-12 * max(np.abs(K).max(), 1e-300):
                return True
    return False


def _bdb_parts(term):
    """Splits a bilinear term into (trial, test, scalars, vector, matrix): trial /
    test are ("val" | "grad"); raises NotImplementedError for shapes the generic
    form does not take."""
    trial = test = None
    scalars, vectors, matrices, has_dx = [], [], [], False
    for f in term.factors:
        if isinstance(f, _Grad) or isinstance(f, _Proxy):
            kind = "grad" if isinstance(f, _Grad) else "val"
            is_test = (f.proxy if isinstance(f, _Grad) else f).test
            if is_test:
                if test is not None:
                    raise NotImplementedError("two test functions in one term")
                test = kind
            else:
                if trial is not None:
                    raise NotImplementedError("two trial functions in one term")
                trial = kind
        elif isinstance(f, _Measure):
            has_dx = True
        elif _is_vector_cf(f):
            vectors.append(f)
        elif isinstance(f, CoefficientFunction) and f.is_tensor():
            matrices.append(f)
        elif isinstance(f, (CoefficientFunction, int, float, np.floating, np.integer)):
            scalars.append(f)
        else:
            raise NotImplementedError("factor %r is not on the B^T D B path" % (f,))
    if not has_dx:
        raise ValueError("integrand needs * dx")
    if trial is None or test is None:
        raise NotImplementedError("a bilinear term needs one trial and one test function")
    ok = {("grad", "grad"): (0, (0, 1)), ("grad", "val"): (1, (0,)), ("val", "grad"): (1, (0,)),
          ("val", "val"): (0, (0,))}[(trial, test)]
    if len(vectors) != ok[0] or len(matrices) not in ok[1]:
        raise NotImplementedError("term shape (%s u, %s v) with %d vector and %d matrix factors is not a scalar "
                                  "B^T D B integrand" % (trial, test, len(vectors), len(matrices)))
    return trial, test, scalars, (vectors[0] if vectors else None), (matrices[0] if matrices else None)


def _bdb_scalar(f, ne, pts, dev):
    """Values of a scalar factor: (ne, P) with P = nq at points or 1 per element."""
    if isinstance(f, _AffineCF):
        return pts @ torch.tensor(f.a, dtype=torch.float64, device=dev) + f.d
    if not isinstance(f, CoefficientFunction):  # a number or an array per element (vector components)
        f = CoefficientFunction(f)
    return torch.tensor(f.element_values(ne), dtype=torch.float64, device=dev)[:, None]


def _bdb_D(terms, ne, pts, dev):
    """Sum of the terms' D matrices in physical coordinates, rows test (v, grad v),
    columns trial (u, grad u): (ne, P, 4, 4), P = nq when pts is given, else 1 --
    the reference's per-(trial, test)-component evaluation of the integrand
    (comp/matrixfree.cpp:1240-1275)."""
    P = 1 if pts is None else pts.shape[1]
    D = torch.zeros((ne, P, 4, 4), dtype=torch.float64, device=dev)
    for t in terms:
        trial, test, scalars, vec, mat = _bdb_parts(t)
        c = torch.ones((ne, 1), dtype=torch.float64, device=dev)
        for f in scalars:
            c = c * _bdb_scalar(f, ne, pts, dev)
        c = c.expand(ne, P)
        if trial == "grad" and test == "grad":
            if mat is None:
                K = torch.eye(3, dtype=torch.float64, device=dev).expand(ne, 3, 3)
            else:
                K = torch.tensor(np.broadcast_to(np.asarray(mat.values, dtype=np.float64), (ne, 3, 3)).copy(),
                                 dtype=torch.float64, device=dev)
            D[:, :, 1:, 1:] += c[:, :, None, None] * K[:, None]
        elif trial == "val" and test == "val":
            D[:, :, 0, 0] += c
        else:
            b = torch.stack([_bdb_scalar(comp, ne, pts, dev).expand(ne, P) for comp in vec.values], dim=-1)
            if trial == "grad":   # (b . grad u) v
                D[:, :, 0, 1:] += c[:, :, None] * b
            else:                 # u (b . grad v)
                D[:, :, 1:, 0] += c[:, :, None] * b
    return D


def _coupling_mask(free, ne, et, order):
    """free without the element-interior DOFs: the last ne * n_cell DOFs in this
    numbering ((p-1)^3 per hex, (p-1)(p-2)(p-3)/6 per tet)."""
    p = int(order)
    n_cell = (p - 1) ** 3 if et == 8 else max(0, (p - 1) * (p - 2) * (p - 3) // 6)
    out = np.array(free, dtype=bool)
    if n_cell:
        out[len(out) - ne * n_cell:] = False
    return out


def _no_dirichlet(dirichlet):
    return dirichlet is None or dirichlet is False or (isinstance(dirichlet, (str, list, tuple)) and len(dirichlet) == 0)


def _dirichlet_faces(raw, dirichlet):
    """The boundary faces the "dirichlet" flag selects -- a regular expression
    matched in full against each boundary-condition name, or a list of 1-based
    boundary-condition numbers (comp/fespace.cpp:440-516) -- or None where the
    all-or-nothing flag says the same: no Dirichlet boundary, a selection of
    every name, or a mesh without named boundaries (where any non-empty
    dirichlet means the whole boundary)."""
    if _no_dirichlet(dirichlet) or dirichlet is True or raw.bc_names is None:
        return None
    if not isinstance(dirichlet, (str, list, tuple)) or (
            not isinstance(dirichlet, str) and not all(isinstance(k, (int, np.integer)) for k in dirichlet)):
        raise TypeError("dirichlet is a regular expression over the boundary names or a list of their numbers")
    if raw.SelectBoundaries(dirichlet).all():
        return None
    return np.ascontiguousarray(raw.BoundaryFaces(dirichlet), dtype=np.int32)


# space flags of the reference's H1 accepted here: these at their default only,
# and autoupdate (mesh refinement never happens on this path) at any value
_SPACE_FIXED_FLAGS = {"complex": False, "dgjumps": False}


def _check_space_flags(flags):
    for flag, value in flags.items():
        if flag == "autoupdate":
            continue
        if flag not in _SPACE_FIXED_FLAGS:
            raise TypeError("H1() got an unexpected flag %r" % flag)
        if bool(value) != _SPACE_FIXED_FLAGS[flag]:
            raise NotImplementedError("H1(%s=%r) is not on the H1 path" % (flag, value))


class _Sum:
    """A sum of integrands, grad(u)*grad(v)*dx + u*v*dx: each term goes into
    the form on its own."""

    def __init__(self, terms):
        self.terms = list(terms)

    def __add__(self, other):
        if isinstance(other, _Sum):
            return _Sum(self.terms + other.terms)
        if not isinstance(other, _Product):
            raise TypeError("only integrands (... * dx) add up")
        return _Sum(self.terms + [other])

    def __sub__(self, other):
        return self + (-other)

    def __neg__(self):
        return _Sum([-t for t in self.terms])


def _space_of(integrand):
    """The space of the first trial or test function in an integrand."""
    terms = integrand.terms if isinstance(integrand, _Sum) else [integrand]
    for t in terms:
        for f in getattr(t, "factors", []):
            if isinstance(f, _Proxy):
                return f.fes
            if isinstance(f, _Grad):
                return f.proxy.fes
    raise ValueError("the integrand has no trial or test function")


# ---------------------------------------------------------------------------
class H1:
    """H1HighOrderFESpace of uniform order (comp/h1hofespace.cpp)."""

    def __init__(self, mesh, order=1, dirichlet="", **flags):
        _check_space_flags(flags)
        if not isinstance(mesh, Mesh):
            mesh = Mesh(mesh)
        self.mesh = mesh
        self.order = int(order)
        self.ctx = mesh.ctx
        faces = _dirichlet_faces(mesh.raw, dirichlet)
        h = ctypes.c_void_p()
        if faces is None:
            dir_all = 0 if _no_dirichlet(dirichlet) else 1
            self.ctx.check(self.ctx.lib.gh1_space_h1(mesh.h, self.order, dir_all, ctypes.byref(h)))
        else:
            self.ctx.check(self.ctx.lib.gh1_space_h1_bnd(mesh.h, self.order, len(faces), _np_ptr(faces),
                                                         ctypes.byref(h)))
        self.h = h
        info = np.zeros(6, dtype=np.int64)
        self.ctx.check(self.ctx.lib.gh1_space_info(h, _np_ptr(info)))
        self.ndof, self.nloc, self.nedges, self.nfaces, self.nfree, self.ne = (int(v) for v in info)
        self._dofs = None
        self._dirichlet = dirichlet
        self._lospace = None

    @property
    def lospace(self):
        """The low-order (p = 1) space of the hierarchical basis on the same mesh
        and Dirichlet boundary; its DOFs are the first (vertex) DOFs of this space."""
        if self.order == 1:
            return self
        if self._lospace is None:
            self._lospace = H1(self.mesh, order=1, dirichlet=self._dirichlet)
        return self._lospace

    @property
    def loembedding(self):
        """The embedding of lospace into this space (identity on the vertex DOFs)."""
        return _Embedding(self)

    def CreateSmoothingBlocks(self, blocktype=4, **flags):
        """CreateSmoothingBlocks (comp/h1hofespace.cpp:1477-1600): blocktype 4 =
        VE + F + I, 3 = V + E + F + I; free DOFs only."""
        if isinstance(blocktype, str):
            blocktype = {"vertexedge": 4, "vertex": 3}.get(blocktype, blocktype)
        nb, ntot = ctypes.c_int64(), ctypes.c_int64()
        self.ctx.check(self.ctx.lib.gh1_space_smoothing_blocks(self.h, int(blocktype), ctypes.byref(nb),
                                                               ctypes.byref(ntot), None, None))
        off = np.zeros(nb.value + 1, dtype=np.int64)
        dofs = np.zeros(max(ntot.value, 1), dtype=np.int32)
        self.ctx.check(self.ctx.lib.gh1_space_smoothing_blocks(self.h, int(blocktype), ctypes.byref(nb),
                                                               ctypes.byref(ntot), _np_ptr(off), _np_ptr(dofs)))
        return SmoothingBlocks(off, dofs[:ntot.value])

    def __del__(self):
        try:
            self.ctx.lib.gh1_space_free(self.h)
        except Exception:
            pass

    def TnT(self):
        return _Proxy(self, False), _Proxy(self, True)

    def TrialFunction(self):
        return _Proxy(self, False)

    def TestFunction(self):
        return _Proxy(self, True)

    def FreeDofs(self, coupling=False):
        """Free DOFs; coupling=True leaves out the element-interior DOFs, which
        static condensation eliminates (GetFreeDofs(external),
        comp/fespace.cpp:2130-2136, with LOCAL_DOF cells, comp/h1hofespace.cpp:1001-1007)."""
        out = np.zeros(self.ndof, dtype=np.uint8)
        self.ctx.check(self.ctx.lib.gh1_space_get_freedofs(self.h, _np_ptr(out)))
        free = out.astype(bool)
        if coupling:
            free = _coupling_mask(free, self.ne, self.mesh.raw.et, self.order)
        return free.view(BitArray)

    def _boundary_dofs(self):
        """DOFs on the boundary (of boundary faces, their edges and vertices):
        the non-free DOFs of the same space with the whole boundary Dirichlet."""
        if getattr(self, "_bnd_dofs", None) is None:
            h = ctypes.c_void_p()
            self.ctx.check(self.ctx.lib.gh1_space_h1(self.mesh.h, self.order, 1, ctypes.byref(h)))
            try:
                out = np.zeros(self.ndof, dtype=np.uint8)
                self.ctx.check(self.ctx.lib.gh1_space_get_freedofs(h, _np_ptr(out)))
            finally:
                self.ctx.lib.gh1_space_free(h)
            self._bnd_dofs = out == 0
        return self._bnd_dofs

    def ElementDofs(self):
        if self._dofs is None:
            out = np.zeros((self.ne, self.nloc), dtype=np.int32)
            self.ctx.check(self.ctx.lib.gh1_space_get_dofs(self.h, _np_ptr(out)))
            self._dofs = out
        return self._dofs

    def GetDofNrs(self, el):
        return tuple(int(d) for d in self.ElementDofs()[int(el)])


class VectorH1:
    """VectorH1 (comp/h1hofespace.cpp:2482-2700): dim copies of H1(order,
    dirichlet), the DOFs of component c at c*n .. (c+1)*n - 1 with n the scalar
    space's ndof (the CompoundFESpace numbering, interleaved = False)."""

    def __init__(self, mesh, order=1, dirichlet="", dim=3, **flags):
        self.scalar = H1(mesh, order=order, dirichlet=dirichlet, **flags)
        self.dim = int(dim)
        self.mesh, self.order, self.ctx = self.scalar.mesh, self.scalar.order, self.scalar.ctx
        self.ne = self.scalar.ne
        self.ndof = self.dim * self.scalar.ndof
        self.nfree = self.dim * self.scalar.nfree

    def TnT(self):
        return _Proxy(self, False), _Proxy(self, True)

    def TrialFunction(self):
        return _Proxy(self, False)

    def TestFunction(self):
        return _Proxy(self, True)

    def FreeDofs(self, coupling=False):
        return np.tile(np.asarray(self.scalar.FreeDofs(coupling)), self.dim).view(BitArray)

    def Range(self, component):
        n = self.scalar.ndof
        return range(component * n, (component + 1) * n)


def InnerProduct(a, b, conjugate=False):
    """InnerProduct(grad(u), grad(v)) and InnerProduct(u, v) of VectorH1 (or H1)
    trial and test functions: the sums over components of grad u_c . grad v_c and
    u_c v_c.  On two vectors (BaseVector or tensors) it is their dot product, a
    float, as ngsolve.InnerProduct of BaseVectors."""
    vec = (BaseVector, torch.Tensor, _Expr)
    if isinstance(a, vec) and isinstance(b, vec):
        return _value(a).InnerProduct(_value(b))
    return _Product.of(a, b)


def _value(x):
    return x.Evaluate() if isinstance(x, _Expr) else _as_vec(x)


def Norm(x):
    """Euclidean norm of a vector or vector expression (ngsolve.Norm)."""
    return _value(x).Norm()


# ---------------------------------------------------------------------------
class BaseVector:
    """Device vector (FP64 unless stated) -- ngla BaseVector / UnifiedVector."""

    def __init__(self, n=None, data=None, dtype=torch.float64, device=0):
        if data is not None:
            self.t = data
        else:
            self.t = torch.zeros(int(n), dtype=dtype, device="cuda:%d" % device)

    def __len__(self):
        return self.t.numel()

    @property
    def size(self):
        return self.t.numel()

    def CreateVector(self):
        return BaseVector(data=torch.zeros_like(self.t))

    def CreateDeviceVector(self, unified=True, copy=True):
        """The vector already lives on the device: a copy (copy=True, the
        reference's default) or a zero vector of the same size and type."""
        return BaseVector(data=self.t.clone() if copy else torch.zeros_like(self.t))

    def NumPy(self):
        return self.t.detach().cpu().numpy()

    def FV(self):
        return self.t

    @property
    def data(self):
        return self

    @data.setter
    def data(self, value):
        if isinstance(value, _Expr):
            value.eval_into(self)
        elif isinstance(value, BaseVector):
            self.t.copy_(value.t)
        elif isinstance(value, torch.Tensor):
            self.t.copy_(value.to(self.t.device, self.t.dtype))
        else:
            self.t.copy_(torch.as_tensor(np.asarray(value), dtype=self.t.dtype, device=self.t.device))

    def __setitem__(self, key, value):
        self.t[key] = value

    def __getitem__(self, key):
        return self.t[key]

    def InnerProduct(self, other, conjugate=False):
        return float(torch.dot(self.t, other.t))

    def Norm(self):
        return float(torch.linalg.vector_norm(self.t))

    def __add__(self, other):
        return _LinComb([(1.0, self), (1.0, other)])

    def __sub__(self, other):
        return _LinComb([(1.0, self), (-1.0, other)])

    def __rmul__(self, s):
        return _LinComb([(float(s), self)])

    def __iadd__(self, other):
        if isinstance(other, _Expr):
            tmp = self.CreateVector()
            other.eval_into(tmp)
            self.t.add_(tmp.t)
        else:
            self.t.add_(other.t)
        return self

    def __isub__(self, other):
        if isinstance(other, _Expr):
            tmp = self.CreateVector()
            other.eval_into(tmp)
            self.t.sub_(tmp.t)
        else:
            self.t.sub_(other.t)
        return self

    def __imul__(self, s):
        self.t.mul_(float(s))
        return self


class _Expr:
    def Evaluate(self):
        """The expression's value as a new vector ((inv * f).Evaluate())."""
        y = BaseVector(data=self._template())
        self.eval_into(y)
        return y

    def eval_into(self, y):
        raise NotImplementedError


class _LinComb(_Expr):
    def __init__(self, terms):
        self.terms = terms

    def __add__(self, other):
        if isinstance(other, _LinComb):
            return _LinComb(self.terms + other.terms)
        return _LinComb(self.terms + [(1.0, other)])

    def __sub__(self, other):
        if isinstance(other, _LinComb):
            return _LinComb(self.terms + [(-s, v) for s, v in other.terms])
        return _LinComb(self.terms + [(-1.0, other)])

    def _template(self):
        for _, v in self.terms:
            if isinstance(v, BaseVector):
                return torch.zeros_like(v.t)
        return self.terms[0][1]._template()

    def eval_into(self, y):
        acc = torch.zeros_like(y.t)
        for s, v in self.terms:
            if isinstance(v, _Expr):
                tmp = y.CreateVector()
                v.eval_into(tmp)
                acc.add_(tmp.t, alpha=s)
            else:
                acc.add_(v.t, alpha=s)
        y.t.copy_(acc)


class _MatVec(_Expr):
    def __init__(self, mat, x, s=1.0):
        self.mat, self.x, self.s = mat, x, s

    def _template(self):
        return torch.zeros(self.mat.height, dtype=self.x.t.dtype, device=self.x.t.device)

    def __rmul__(self, s):
        return _MatVec(self.mat, self.x, self.s * float(s))

    def __add__(self, other):
        return _LinComb([(1.0, self), (1.0, other)])

    def __radd__(self, other):
        return _LinComb([(1.0, other), (1.0, self)])

    def __rsub__(self, other):
        return _LinComb([(1.0, other), (-1.0, self)])

    def eval_into(self, y):
        self.mat.MultScale(self.s, self.x, y)


def _as_vec(x):
    return x if isinstance(x, BaseVector) else BaseVector(data=x)


class BaseMatrix:
    """BaseMatrix Mult / MultAdd (linalg/basematrix.hpp:117-126) on a gh1 operator."""

    def __init__(self, ctx, h, height, fes=None):
        self.ctx, self.h, self.height, self.width, self.fes = ctx, h, int(height), int(height), fes

    def Info(self):
        """kind, nrows, ne, order and (hex matrix-free) the apply variant per precision."""
        a = (ctypes.c_int64 * 6)()
        self.ctx.check(self.ctx.lib.gh1_op_info(self.h, a))
        return {"kind": a[0], "nrows": a[1], "ne": a[2], "order": a[3], "hex_variant_fp64": a[4],
                "hex_variant_fp32": a[5]}

    def __mul__(self, x):
        return _MatVec(self, _as_vec(x))

    def CreateVector(self, colvector=False):
        return BaseVector(self.height)

    CreateRowVector = CreateVector
    CreateColVector = CreateVector

    def _apply(self, s, x, y, acc):
        x, y = _as_vec(x), _as_vec(y)
        if x.t.dtype != y.t.dtype:
            raise TypeError("x and y must have the same precision")
        prec = _lib.GH1_F64 if x.t.dtype == torch.float64 else _lib.GH1_F32
        if not (x.t.is_cuda and y.t.is_cuda and x.t.is_contiguous() and y.t.is_contiguous()):
            raise TypeError("vectors must be contiguous CUDA tensors")
        if x.t.numel() != self.width or y.t.numel() != self.height:
            raise ValueError("vector size does not match the matrix")
        self.ctx.sync_stream()
        self.ctx.check(self.ctx.lib.gh1_op_apply(self.h, float(s), _ptr(x.t), _ptr(y.t), prec, int(acc)))

    def Mult(self, x, y):
        self._apply(1.0, x, y, 0)

    def MultScale(self, s, x, y):
        self._apply(s, x, y, 0)

    def MultAdd(self, s, x, y):
        self._apply(s, x, y, 1)

    # The operators of the Laplace / mass / tensor forms, the Jacobi diagonal and
    # the projectors are symmetric (sum_e B^T G B with a symmetric G), so their
    # transpose products apply the operator itself.  A generic B^T D B form with
    # a non-symmetric D (convection b.grad(u) v, for example) carries a factory
    # `_transposer` for the operator of the transposed form, D^T (built on first use).
    def _transpose_op(self):
        back = getattr(self, "_transpose_of", None)  # this is the transposed operator of another
        if back is not None and back() is not None:
            return back()
        f = getattr(self, "_transposer", None)
        if f is None:
            return self
        if getattr(self, "_transposed", None) is None:
            self._transposed = f()
            self._transposed._transpose_of = weakref.ref(self)
        return self._transposed

    def MultTrans(self, value, x, y):
        """y = A^T x.  As in the reference binding (linalg/python_linalg.cpp:1074),
        y is cleared and A^T x added; `value` is accepted and not applied."""
        self._transpose_op()._apply(1.0, x, y, 0)

    def MultTransAdd(self, value, x, y):
        """y += value * A^T x (linalg/python_linalg.cpp:1075)."""
        self._transpose_op()._apply(value, x, y, 1)

    @property
    def T(self):
        """The transpose: this operator itself where it is symmetric, else the
        operator of the transposed form."""
        return self._transpose_op()

    def CreateDeviceMatrix(self):
        """The operator already lives on the device (BaseMatrix.CreateDeviceMatrix)."""
        return self

    def GetOperatorInfo(self):
        i = self.Info()
        kind = {0: "SparseMatrix (CSR)", 1: "BilinearFormApplication (matrix-free)", 2: "BlockMatrix"}.get(i["kind"], "?")
        return "%s, h = %d, w = %d, elements %d, order %d\n" % (kind, self.height, self.width, i["ne"], i["order"])

    @property
    def shape(self):
        return (self.height, self.width)

    def CreateSmoother(self, freedofs=None):
        return JacobiPrecond(self, freedofs)

    def CreateBlockSmoother(self, blocks, **kwargs):
        """BlockJacobiPrecond of an assembled matrix over SmoothingBlocks."""
        if not isinstance(self, SparseMatrix):
            raise NotImplementedError("the block smoother needs the assembled matrix (BilinearForm without nonassemble)")
        return BlockJacobiPrecond(self, blocks)

    def Inverse(self, freedofs=None, inverse=None, tol=1e-12, maxsteps=100000):
        """A^{-1} on the free DOFs, for a.mat.Inverse(fes.FreeDofs()).  The
        reference factorizes (sparsecholesky, umfpack, pardiso ...); this path has
        no sparse direct solver, so every `inverse` name gives the same operator:
        FP64 Jacobi-PCG on the GPU to `tol` (relative preconditioned residual,
        the default of solvers.CG), raising if it does not get there.  Rows of non-free DOFs are zero, as in
        the reference.  freedofs=None: the space's free DOFs."""
        if inverse not in _INVERSE_NAMES:
            raise ValueError("unknown inverse %r" % (inverse,))
        if inverse == "sparsecholesky" and isinstance(self, SparseMatrix):
            fd = np.ones(self.height, dtype=bool) if freedofs is None else np.asarray(freedofs, dtype=bool)
            if int(fd.sum()) <= ExactInverse.MAX_FREE:
                return ExactInverse(self, fd)
        return InverseOperator(self, freedofs, tol, maxsteps)

    def __del__(self):
        try:
            self.ctx.lib.gh1_op_free(self.h)
        except Exception:
            pass


_INVERSE_NAMES = (None, "", "cg", "sparsecholesky", "umfpack", "pardiso", "pardisospd", "mumps", "masterinverse")


class InverseOperator:
    """The operator BaseMatrix.Inverse returns: each product is one FP64
    Jacobi-PCG solve on the GPU from a zero start.  Symmetric, like A."""

    def __init__(self, mat, freedofs=None, tol=1e-12, maxsteps=100000):
        self.mat, self.height, self.width = mat, mat.height, mat.width
        self.pre = mat.CreateSmoother(freedofs)
        self.tol, self.maxsteps = float(tol), int(maxsteps)
        self.iterations = 0

    def Mult(self, x, y):
        from .solvers import CGSolver
        solver = CGSolver(mat=self.mat, pre=self.pre, tol=self.tol, maxiter=self.maxsteps)
        solver.Solve(rhs=x, sol=y, initialize=True)
        self.iterations = solver.iterations
        if solver.result.status != 0:
            raise _lib.GH1Error(solver.result.status, "Inverse: CG stopped after %d iterations above tol %g"
                                % (solver.iterations, self.tol))

    def MultScale(self, s, x, y):
        self.Mult(x, y)
        if s != 1.0:
            _as_vec(y).t.mul_(s)

    def MultAdd(self, s, x, y):
        y = _as_vec(y)
        tmp = y.CreateVector()
        self.Mult(x, tmp)
        y.t.add_(tmp.t, alpha=s)

    def MultTrans(self, value, x, y):
        self.Mult(x, y)

    def MultTransAdd(self, value, x, y):
        self.MultAdd(value, x, y)

    @property
    def T(self):
        return self

    @property
    def shape(self):
        return (self.height, self.width)

    def CreateVector(self, colvector=False):
        return self.mat.CreateVector()

    def CreateDeviceMatrix(self):
        return self

    def GetOperatorInfo(self):
        return "Inverse by CG (tol %g) of: %s" % (self.tol, self.mat.GetOperatorInfo())

    def __mul__(self, x):
        return _MatVec(self, _as_vec(x))


class SparseMatrix(BaseMatrix):
    """Assembled CSR matrix on the GPU (SparseMatrix<double>)."""

    def __init__(self, ctx, h, fes=None):
        info = np.zeros(2, dtype=np.int64)
        ctx.check(ctx.lib.gh1_csr_info(h, _np_ptr(info)))
        super().__init__(ctx, h, info[0], fes)
        self.nze = int(info[1])

    def CSR(self):
        """(rowptr int64, colind int32, vals float64) copied to the host."""
        rp = np.zeros(self.height + 1, dtype=np.int64)
        ci = np.zeros(self.nze, dtype=np.int32)
        va = np.zeros(self.nze, dtype=np.float64)
        self.ctx.check(self.ctx.lib.gh1_csr_export(self.h, _np_ptr(rp), _np_ptr(ci), _np_ptr(va), _lib.GH1_MEM_HOST))
        return rp, ci, va

    def __getitem__(self, ij):
        i, j = ij
        rp, ci, va = self.CSR()
        row = ci[rp[i]:rp[i + 1]]
        k = np.searchsorted(row, j)
        return float(va[rp[i] + k]) if k < len(row) and row[k] == j else 0.0

    @staticmethod
    def FromCSR(rowptr, colind, vals, device=0):
        ctx = context(device)
        rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
        colind = np.ascontiguousarray(colind, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        h = ctypes.c_void_p()
        ctx.check(ctx.lib.gh1_csr_import(ctx.h, len(rowptr) - 1, len(colind), _np_ptr(rowptr), _np_ptr(colind),
                                         _np_ptr(vals), _lib.GH1_MEM_HOST, ctypes.byref(h)))
        return SparseMatrix(ctx, h)


class BilinearFormApplication(BaseMatrix):
    """Matrix-free operator: sum-factorized on hexes, element-wise on tets."""


class BlockMatrix(BaseMatrix):
    """diag(A, ..., A): the VectorH1 form of a scalar operator A (one block per
    component).  Keeps A alive: the block operator borrows it."""

    def __init__(self, ctx, h, fes, inner):
        super().__init__(ctx, h, fes.ndof, fes)
        self.inner = inner


class _PreBase(BaseMatrix):
    """A gh1 preconditioner handle used as an operator (Mult), summed with `+`
    (the reference's SumMatrix) and passed to CGSolver."""

    def _apply(self, s, x, y, acc):
        x, y = _as_vec(x), _as_vec(y)
        if x.t.dtype != y.t.dtype or x.t.numel() != self.height or y.t.numel() != self.height:
            raise ValueError("vectors must match the preconditioner in size and precision")
        prec = _lib.GH1_F64 if x.t.dtype == torch.float64 else _lib.GH1_F32
        self.ctx.sync_stream()
        self.ctx.check(self.ctx.lib.gh1_pre_apply(self.h, float(s), _ptr(x.t), _ptr(y.t), prec, int(acc)))

    def __add__(self, other):
        if isinstance(other, _EmbComposed):
            other = other.solver()
        if not isinstance(other, _PreBase):
            return NotImplemented
        return SumPrecond(self, other)

    __radd__ = __add__

    def Info(self):  # the handle is a preconditioner, not an operator
        return {"kind": type(self).__name__, "nrows": self.height}

    def Inverse(self, *args, **kwargs):
        raise NotImplementedError("Inverse of a preconditioner")

    def __del__(self):
        try:
            self.ctx.lib.gh1_pre_free(self.h)
        except Exception:
            pass


class SmoothingBlocks:
    """The Table of DOF blocks of CreateSmoothingBlocks: len(), blocks[i] (a
    list of DOFs), iteration; offsets / dofs as arrays."""

    def __init__(self, offsets, dofs):
        self.offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        self.dofs = np.ascontiguousarray(dofs, dtype=np.int32)

    def __len__(self):
        return len(self.offsets) - 1

    def __getitem__(self, i):
        return self.dofs[self.offsets[i]:self.offsets[i + 1]].tolist()

    def __iter__(self):
        for i in range(len(self)):
            yield self[i]


class BlockJacobiPrecond(_PreBase):
    """BlockJacobiPrecond (linalg/blockjacobi.cpp; device DevBlockJacobiMatrix,
    ngscuda/dev_blockjacobi.cpp:49-137): sum_b E_b A_b^{-1} E_b^T."""

    def __init__(self, mat, blocks):
        if not isinstance(blocks, SmoothingBlocks):
            rows = [np.asarray(b, dtype=np.int32) for b in blocks]
            off = np.concatenate([[0], np.cumsum([len(b) for b in rows])]).astype(np.int64)
            blocks = SmoothingBlocks(off, np.concatenate(rows) if rows else np.zeros(0, dtype=np.int32))
        h = ctypes.c_void_p()
        mat.ctx.sync_stream()
        mat.ctx.check(mat.ctx.lib.gh1_blockjacobi_create(mat.h, len(blocks), _np_ptr(blocks.offsets),
                                                          _np_ptr(blocks.dofs), _lib.GH1_MEM_HOST, ctypes.byref(h)))
        self.ctx, self.h, self.height, self.width, self.fes = mat.ctx, h, mat.height, mat.height, mat.fes
        self.blocks, self.mat = blocks, mat

    def GetOperatorInfo(self):
        return "BlockJacobiPrecond (%d blocks), h = %d, w = %d\n" % (len(self.blocks), self.height, self.width)


class ExactInverse(_PreBase):
    """A^{-1} on the free DOFs of an assembled matrix, inverted on the GPU: the
    role of Inverse(inverse="sparsecholesky") for matrices with up to MAX_FREE
    free DOFs (larger ones get the Jacobi-PCG InverseOperator).  With `nfine`,
    the inverse of a low-order matrix embedded into the first DOFs of a larger
    space (loemb @ loinv @ loemb.T)."""
    MAX_FREE = 8192

    def __init__(self, mat, freedofs, nfine=None):
        fd = np.ascontiguousarray(np.asarray(freedofs, dtype=bool).astype(np.uint8))
        if fd.shape != (mat.height,):
            raise ValueError("freedofs size does not match the matrix")
        n = mat.height if nfine is None else int(nfine)
        h = ctypes.c_void_p()
        mat.ctx.sync_stream()
        mat.ctx.check(mat.ctx.lib.gh1_coarse_create(mat.h, n, None, _np_ptr(fd), _lib.GH1_MEM_HOST, ctypes.byref(h)))
        self.ctx, self.h, self.height, self.width, self.fes = mat.ctx, h, n, n, mat.fes
        self.mat, self._fd = mat, fd

    def GetOperatorInfo(self):
        return "ExactInverse (dense, %d free DOFs), h = %d, w = %d\n" % (int(self._fd.sum()), self.height, self.width)


class SumPrecond(_PreBase):
    """a + b of two preconditioners (SumMatrix); keeps both alive."""

    def __init__(self, a, b):
        if a.height != b.height:
            raise ValueError("the two preconditioners differ in size")
        h = ctypes.c_void_p()
        a.ctx.check(a.ctx.lib.gh1_pre_sum(a.h, b.h, ctypes.byref(h)))
        self.ctx, self.h, self.height, self.width, self.fes = a.ctx, h, a.height, a.height, a.fes
        self.a, self.b = a, b

    def GetOperatorInfo(self):
        return "SumMatrix, h = %d, w = %d\n  %s  %s" % (self.height, self.width, self.a.GetOperatorInfo(),
                                                         self.b.GetOperatorInfo())


class _Embedding:
    """fes.loembedding: the low-order space's DOFs are the first DOFs of the
    high-order space (identity there); E @ inv @ E.T is the embedded solve."""

    def __init__(self, fes, transposed=False):
        self.fes, self.transposed = fes, transposed

    @property
    def T(self):
        return _Embedding(self.fes, not self.transposed)

    def __matmul__(self, other):
        if self.transposed:
            raise NotImplementedError("loembedding.T only on the right of loembedding @ loinv")
        return _EmbComposed(self.fes, other)


class _EmbComposed:
    """loembedding @ loinv (@ loembedding.T): becomes an ExactInverse of the
    low-order matrix acting on the vertex DOFs of the high-order space."""

    def __init__(self, fes, inner, closed=False):
        self.fes, self.inner, self.closed = fes, inner, closed
        self._solver = None

    def __matmul__(self, other):
        if not (isinstance(other, _Embedding) and other.transposed and not self.closed):
            raise NotImplementedError("loembedding @ loinv @ loembedding.T")
        return _EmbComposed(self.fes, self.inner, closed=True)

    def solver(self):
        if not self.closed:
            raise NotImplementedError("loembedding @ loinv needs @ loembedding.T")
        if self._solver is None:
            inv = self.inner
            if not isinstance(inv, ExactInverse):
                raise NotImplementedError("loinv = a.loform.mat.Inverse(inverse='sparsecholesky', freedofs=...)")
            self._solver = ExactInverse(inv.mat, inv._fd.astype(bool), nfine=self.fes.ndof)
        return self._solver

    def __add__(self, other):
        return self.solver() + other

    __radd__ = __add__

    def Mult(self, x, y):
        self.solver().Mult(x, y)

    def GetOperatorInfo(self):
        return self.solver().GetOperatorInfo()


class JacobiPrecond(_PreBase):
    """JacobiPrecond (linalg/jacobi.cpp:40-110): invdiag on free DOFs, 0 elsewhere."""

    def __init__(self, mat, freedofs=None):
        self.mat = mat
        h = ctypes.c_void_p()
        fd = None
        if freedofs is not None:
            fd = np.ascontiguousarray(np.asarray(freedofs, dtype=bool).astype(np.uint8))
            if fd.shape != (mat.height,):
                raise ValueError("freedofs size does not match the matrix")
        mat.ctx.sync_stream()
        mat.ctx.check(mat.ctx.lib.gh1_jacobi_create(mat.h, None if fd is None else _np_ptr(fd), _lib.GH1_MEM_HOST,
                                                     ctypes.byref(h)))
        self.ctx, self.h, self.height, self.width, self.fes = mat.ctx, h, mat.height, mat.height, mat.fes
        self._fd = fd

    def _apply(self, s, x, y, acc):
        x, y = _as_vec(x), _as_vec(y)
        prec = _lib.GH1_F64 if x.t.dtype == torch.float64 else _lib.GH1_F32
        self.ctx.sync_stream()
        self.ctx.check(self.ctx.lib.gh1_pre_apply(self.h, float(s), _ptr(x.t), _ptr(y.t), prec, int(acc)))

    def Info(self):  # the handle is a preconditioner, not an operator
        return {"kind": "jacobi", "nrows": self.height}

    def GetOperatorInfo(self):
        return "JacobiPrecond, h = %d, w = %d\n" % (self.height, self.width)

    def Inverse(self, *args, **kwargs):
        raise NotImplementedError("Inverse of a preconditioner")

    def __del__(self):
        try:
            self.ctx.lib.gh1_pre_free(self.h)
        except Exception:
            pass


class Projector(BaseMatrix):
    """Projector(mask, range) (linalg/diagonalmatrix.cpp:13-110): keeps the entries
    whose mask bit equals `range` and zeroes the others; .Project(vec) in place."""

    def __init__(self, mask, range=True, device=0):
        ctx = context(device)
        m = np.ascontiguousarray(np.asarray(mask, dtype=bool).astype(np.uint8))
        h = ctypes.c_void_p()
        ctx.check(ctx.lib.gh1_projector_create(ctx.h, len(m), _np_ptr(m), 1 if range else 0, _lib.GH1_MEM_HOST,
                                               ctypes.byref(h)))
        self.ctx, self.h, self.height, self.width, self.fes = ctx, h, len(m), len(m), None
        self.range = bool(range)

    def _apply(self, s, x, y, acc):
        x, y = _as_vec(x), _as_vec(y)
        if x.t.dtype != y.t.dtype or x.t.numel() != self.height or y.t.numel() != self.height:
            raise ValueError("vectors must match the projector in size and precision")
        prec = _lib.GH1_F64 if x.t.dtype == torch.float64 else _lib.GH1_F32
        self.ctx.sync_stream()
        self.ctx.check(self.ctx.lib.gh1_projector_apply(self.h, float(s), _ptr(x.t), _ptr(y.t), prec, int(acc)))

    def Info(self):  # the handle is a projector, not an operator
        return {"kind": "projector", "nrows": self.height}

    def GetOperatorInfo(self):
        return "Projector (range = %s), h = %d, w = %d\n" % (self.range, self.height, self.width)

    def Inverse(self, *args, **kwargs):
        raise NotImplementedError("Inverse of a projector")

    def Project(self, vec):
        v = _as_vec(vec)
        if v.t.numel() != self.height:
            raise ValueError("vector size does not match the projector")
        prec = _lib.GH1_F64 if v.t.dtype == torch.float64 else _lib.GH1_F32
        self.ctx.sync_stream()
        self.ctx.check(self.ctx.lib.gh1_projector_project(self.h, _ptr(v.t), prec))
        return vec

    def __del__(self):
        try:
            self.ctx.lib.gh1_projector_free(self.h)
        except Exception:
            pass


def Preconditioner(a, kind="local"):
    """Preconditioner(a, "local") = Jacobi on the free DOFs (comp/preconditioner.cpp:684-760)."""
    if kind not in ("local", "jacobi"):
        raise NotImplementedError("only the 'local' (Jacobi) preconditioner is on the H1 path")
    return JacobiPrecond(a.mat, a.fes.FreeDofs())


# ---------------------------------------------------------------------------
class BilinearForm:
    """BilinearForm(fes, nonassemble=False) with kappa grad.grad and mu u.v terms.

    nonassemble=True gives the matrix-free operator as .mat (BilinearFormApplication,
    comp/bilinearform.cpp:7549-7607); precision='fp32' adds the FP32 data used by
    the mixed-precision solver (the reference's fp32 flag, :7590-7607)."""

    # flags of the reference's BilinearForm that would change what the operator
    # is; accepted only at their default (other flags are accepted and unused)
    _FIXED_FLAGS = {"condense": False, "eliminate_internal": False, "eliminate_hidden": False,
                    "symmetric_storage": False, "diagonal": False, "hermitian": False, "nonsym": False}

    def __init__(self, fes, nonassemble=False, precision="fp64", symmetric=True, **kwargs):
        integrand = None
        if isinstance(fes, (_Product, _Sum)):  # BilinearForm(grad(u)*grad(v)*dx + ...)
            integrand, fes = fes, _space_of(fes)
        for flag, default in self._FIXED_FLAGS.items():
            if flag in kwargs and bool(kwargs[flag]) != default:
                raise NotImplementedError("BilinearForm(%s=%r) is not on the H1 path" % (flag, kwargs[flag]))
        if precision not in ("fp64", "fp32", "mixed"):
            raise ValueError("precision is 'fp64', 'fp32' or 'mixed'")
        self.fes = fes
        self._sfes = fes.scalar if isinstance(fes, VectorH1) else fes  # the space the form lives on
        self.nonassemble = bool(nonassemble)
        self.precision = precision
        self.kappa = np.zeros(fes.ne)
        self.K6 = None  # (ne, 6) sum of the tensor diffusion terms
        self.mu = None
        self._has_laplace = False
        self._terms = []       # every bilinear term, for the generic B^T D B form
        self._generic = False  # a term outside kappa grad.grad / mu u v / symmetric K
        self._form = None
        self.mat = None
        if integrand is not None:
            self += integrand

    def __iadd__(self, term):
        if isinstance(term, _Sum):
            for t in term.terms:
                self += t
            return self
        if _bdb_needed(term):
            if self._sfes is not self.fes:
                raise NotImplementedError("the generic B^T D B form is on the path for scalar H1 only")
            _bdb_parts(term)  # shape check now, values at Assemble
            self._terms.append(term)
            self._generic = True
            self._form = None
            return self
        kind, coef = term.classify(self.fes.ne)
        if kind in ("laplace", "laplace_tensor", "mass"):
            self._terms.append(term)
        if kind == "laplace":
            self.kappa = self.kappa + coef
            self._has_laplace = True
        elif kind == "laplace_tensor":
            if self._sfes is not self.fes:
                # on VectorH1, K * grad(u) is the matrix product K (du_i/dx_j),
                # which couples the components: not the block-diagonal operator
                raise NotImplementedError("a tensor diffusion term is on the path for scalar H1 only")
            self.K6 = coef if self.K6 is None else self.K6 + coef
            self._has_laplace = True
        elif kind == "mass":
            self.mu = coef if self.mu is None else self.mu + coef
        else:
            raise ValueError("a source term belongs to a LinearForm")
        self._form = None
        return self

    def _make_form(self):
        ctx = self.fes.ctx
        kappa = np.ascontiguousarray(self.kappa, dtype=np.float64)
        mu = None if self.mu is None else np.ascontiguousarray(self.mu, dtype=np.float64)
        if self._form is None and self._generic:
            # generic B^T D B: D per element, or per rule point when a coefficient
            # varies inside the elements (gh1_form_set_bdb, gh1_space_qpoints)
            sfes, ne = self._sfes, self._sfes.ne
            dev = torch.device("cuda", ctx.device)
            pts = None
            if any(_is_pointwise(f) for t in self._terms for f in t.factors):
                nq = ctypes.c_int()
                ctx.check(ctx.lib.gh1_space_qpoints(sfes.h, None, None, _lib.GH1_MEM_HOST, ctypes.byref(nq)))
                pts = torch.empty((ne, nq.value, 3), dtype=torch.float64, device=dev)
                ctx.sync_stream()
                ctx.check(ctx.lib.gh1_space_qpoints(sfes.h, None, _ptr(pts), _lib.GH1_MEM_DEVICE, None))
            D = _bdb_D(self._terms, ne, pts, dev).reshape(ne, -1, 16)
            D = (D[:, 0] if pts is None else D).contiguous()
            torch.cuda.synchronize(dev)
            h = ctypes.c_void_p()
            ctx.check(ctx.lib.gh1_form_create(sfes.h, None, None, _lib.GH1_MEM_HOST, ctypes.byref(h)))
            self._form = h
            ctx.check(ctx.lib.gh1_form_set_bdb(h, _ptr(D), 0 if pts is None else 1, _lib.GH1_MEM_DEVICE))
            # the transposed form's D, kept while it differs from D
            Dm = D.reshape(*D.shape[:-1], 4, 4)
            DT = Dm.transpose(-1, -2).reshape(D.shape).contiguous()
            sym = float((DT - D).abs().max()) <= 1e-14 * max(float(D.abs().max()), 1e-300)
            self._bdb_T = None if sym else (DT, pts is not None)
            return self._form
        if self._form is None:
            h = ctypes.c_void_p()
            ctx.check(ctx.lib.gh1_form_create(self._sfes.h, _np_ptr(kappa), None if mu is None else _np_ptr(mu),
                                              _lib.GH1_MEM_HOST, ctypes.byref(h)))
            self._form = h
            if self.K6 is not None:  # scalar terms folded in as kappa I
                K6 = np.array(self.K6, dtype=np.float64)
                K6[:, :3] += kappa[:, None]
                ctx.check(ctx.lib.gh1_form_set_tensor(h, _np_ptr(K6), _lib.GH1_MEM_HOST))
        return self._form

    def Assemble(self, reallocate=False):
        ctx = self.fes.ctx.sync_stream()
        form = self._make_form()
        h = ctypes.c_void_p()
        sfes = self._sfes
        if self.nonassemble:
            mask = 1 | (2 if self.precision in ("fp32", "mixed") else 0)
            ctx.check(ctx.lib.gh1_matfree_create(form, mask, ctypes.byref(h)))
            mat = BilinearFormApplication(ctx, h, sfes.ndof, sfes)
        else:
            ctx.check(ctx.lib.gh1_assemble_csr(form, ctypes.byref(h)))
            mat = SparseMatrix(ctx, h, sfes)
        if self._generic and getattr(self, "_bdb_T", None) is not None:
            mat._transposer = self._transposer(*self._bdb_T)
        if sfes is not self.fes:  # VectorH1: the scalar operator once per component
            hb = ctypes.c_void_p()
            ctx.check(ctx.lib.gh1_op_block_create(mat.h, self.fes.dim, ctypes.byref(hb)))
            mat = BlockMatrix(ctx, hb, self.fes, mat)
        self.mat = mat
        return self

    def _transposer(self, DT, per_point):
        """Factory of the operator of the transposed B^T D B form (D^T), of the
        same kind as this form's (matrix-free with the same precisions, or CSR)."""
        ctx, sfes, nonassemble, precision = self.fes.ctx, self._sfes, self.nonassemble, self.precision

        def make():
            ctx.sync_stream()
            hf = ctypes.c_void_p()
            ctx.check(ctx.lib.gh1_form_create(sfes.h, None, None, _lib.GH1_MEM_HOST, ctypes.byref(hf)))
            try:
                ctx.check(ctx.lib.gh1_form_set_bdb(hf, _ptr(DT), 1 if per_point else 0, _lib.GH1_MEM_DEVICE))
                h = ctypes.c_void_p()
                if nonassemble:
                    mask = 1 | (2 if precision in ("fp32", "mixed") else 0)
                    ctx.check(ctx.lib.gh1_matfree_create(hf, mask, ctypes.byref(h)))
                    return BilinearFormApplication(ctx, h, sfes.ndof, sfes)
                ctx.check(ctx.lib.gh1_assemble_csr(hf, ctypes.byref(h)))
                return SparseMatrix(ctx, h, sfes)
            finally:
                ctx.lib.gh1_form_free(hf)  # the operator keeps its form alive
        return make

    def Apply(self, x, y):
        if self.mat is None:
            self.Assemble()
        self.mat.Mult(x, y)

    @property
    def loform(self):
        """The same integrand on fes.lospace, assembled (the reference's
        low-order bilinear form of an H1 high-order space)."""
        if self._generic or self._sfes is not self.fes:
            raise NotImplementedError("the low-order form is built for scalar H1 Laplace / mass / tensor forms")
        if getattr(self, "_loform", None) is None:
            lo = BilinearForm(self.fes.lospace)
            for t in self._terms:
                lo += t
            self._loform = lo.Assemble()
        return self._loform

    def __del__(self):
        try:
            if self._form is not None:
                self.fes.ctx.lib.gh1_form_free(self._form)
        except Exception:
            pass


class LinearForm:
    """LinearForm(fes) += f * v * dx with f constant per element; order 2p.  On
    VectorH1, f is CoefficientFunction((f_1, ..., f_dim)), one value (or array per
    element) per component."""

    def __init__(self, fes):
        integrand = None
        if isinstance(fes, (_Product, _Sum)):  # LinearForm(f*v*dx + ...)
            integrand, fes = fes, _space_of(fes)
        self.fes = fes
        self._vector = isinstance(fes, VectorH1)
        self.f = np.zeros((fes.dim, fes.ne)) if self._vector else np.zeros(fes.ne)
        self.affine = np.zeros(4)  # a.x + b.y + c.z + d sources (scalar H1)
        self._mass = None
        self.vec = BaseVector(fes.ndof)
        if integrand is not None:
            self += integrand

    def __iadd__(self, term):
        if isinstance(term, _Sum):
            for t in term.terms:
                self += t
            return self
        if self._vector:
            comps = [f for f in term.factors if isinstance(f, CoefficientFunction) and isinstance(f.values, (tuple, list))]
            if len(comps) != 1 or len(comps[0].values) != self.fes.dim:
                raise ValueError("a VectorH1 source is CoefficientFunction((f_1, ..., f_%d)) * v * dx" % self.fes.dim)
            kind, coef = _Product([f for f in term.factors if f is not comps[0]]).classify(self.fes.ne)
            if kind != "source":
                raise ValueError("LinearForm takes f*v*dx")
            for c, fc in enumerate(comps[0].values):
                self.f[c] = self.f[c] + coef * CoefficientFunction(fc).element_values(self.fes.ne)
            return self
        kind, coef = term.classify(self.fes.ne)
        if kind == "source_affine":
            self.affine = self.affine + coef
            return self
        if kind != "source":
            raise ValueError("LinearForm takes f*v*dx")
        self.f = self.f + coef
        return self

    def Assemble(self):
        ctx = self.fes.ctx.sync_stream()
        if self._vector:  # component c into its DOF block
            sfes, n = self.fes.scalar, self.fes.scalar.ndof
            for c in range(self.fes.dim):
                f = np.ascontiguousarray(self.f[c], dtype=np.float64)
                ctx.check(ctx.lib.gh1_rhs_elementwise(sfes.h, _np_ptr(f), _lib.GH1_MEM_HOST,
                                                      _ptr(self.vec.t[c * n:(c + 1) * n])))
            return self
        f = np.ascontiguousarray(self.f, dtype=np.float64)
        ctx.check(ctx.lib.gh1_rhs_elementwise(self.fes.h, _np_ptr(f), _lib.GH1_MEM_HOST, _ptr(self.vec.t)))
        if np.any(self.affine != 0.0):
            _affine_source(self, _AffineCF(self.affine[:3], self.affine[3]))
        return self


def _affine_source(lf, f):
    """lf.vec += M I_h(f) for an affine f: the mass operator of lf's space
    (matrix-free, built once per LinearForm) applied to f's interpolant."""
    fes = lf.fes
    if lf._mass is None:
        u, v = fes.TnT()
        m = BilinearForm(fes, nonassemble=True)
        m += u * v * dx
        lf._mass = m.Assemble()
    fi = np.zeros(fes.ndof)
    pts = fes.mesh.raw.points
    fi[:len(pts)] = f.vertex_values(pts)
    xi = BaseVector(data=torch.tensor(fi, dtype=lf.vec.t.dtype, device=lf.vec.t.device))
    lf._mass.mat.MultAdd(1.0, xi, lf.vec)


VOL, BND = "VOL", "BND"


class GridFunction:
    def __init__(self, fes, name="gfu", vec=None):
        self.fes = fes
        self.name = name
        self.vec = BaseVector(fes.ndof) if vec is None else vec

    def __mul__(self, other):
        if not _gf_factor(other):
            return NotImplemented
        return _GFIntegrand("product", self, other)

    __rmul__ = __mul__

    def Set(self, cf, VOL_or_BND=VOL):
        """gfu.Set(f) for f affine in x, y, z or constant, on scalar H1: the
        interpolant is then f itself (vertex values, all other DOFs zero), which
        is also what the reference's projection-based Set returns for a function
        in the space.  Set(f, BND) writes only the DOFs of the boundary (all
        boundary faces, whatever the Dirichlet flag) and keeps the others, as
        used for inhomogeneous Dirichlet data."""
        if isinstance(cf, (int, float, np.floating, np.integer)):
            cf = _AffineCF((0.0, 0.0, 0.0), float(cf))
        elif isinstance(cf, CoefficientFunction) and not isinstance(cf, _AffineCF):
            v = np.asarray(cf.values, dtype=np.float64)
            if v.ndim != 0:
                raise NotImplementedError("Set takes a constant or an affine function of x, y, z")
            cf = _AffineCF((0.0, 0.0, 0.0), float(v))
        if not isinstance(cf, _AffineCF) or not isinstance(self.fes, H1):
            raise NotImplementedError("Set takes a constant or an affine function of x, y, z on H1")
        pts = self.fes.mesh.raw.points
        new = torch.zeros_like(self.vec.t)
        new[:len(pts)] = torch.as_tensor(cf.vertex_values(pts), dtype=new.dtype, device=new.device)
        if VOL_or_BND == BND:
            on = torch.as_tensor(self.fes._boundary_dofs(), device=new.device)
            new = torch.where(on, new, self.vec.t)
        elif VOL_or_BND != VOL:
            raise ValueError("VOL_or_BND is VOL or BND")
        self.vec.t.copy_(new)

    @property
    def components(self):
        """On VectorH1: one GridFunction of the scalar space per component, each
        viewing its block of this vector (no copy: writes go through), as
        GridFunction.components of a compound space."""
        if not isinstance(self.fes, VectorH1):
            raise TypeError("components are defined on VectorH1")
        n = self.fes.scalar.ndof
        return tuple(GridFunction(self.fes.scalar, "%s.%d" % (self.name, c), BaseVector(data=self.vec.t[c * n:(c + 1) * n]))
                     for c in range(self.fes.dim))


class _GFIntegrand:
    """Integrand of Integrate made of grid functions: "graddot" (grad a .
    grad b) or "product" (a * b, where a factor may be a constant or affine
    coefficient, taken as its interpolant)."""

    def __init__(self, kind, a, b):
        self.kind, self.a, self.b = kind, a, b


def _gf_factor(f):
    return isinstance(f, (GridFunction, _AffineCF, int, float, np.floating)) or (
        isinstance(f, CoefficientFunction) and np.ndim(f.values) == 0)


def Integrate(cf, mesh, element_wise=False, order=None):
    """Integrate (comp/python_comp.cpp:3703-3948) for the integrands of this
    path: grad(a) * grad(b) of two GridFunctions, element-wise (the dJ/dkappa
    contraction of the adjoint recipe, on the GPU element kernel) or summed;
    and the total of a product a * b or of a single factor, where a factor is a
    GridFunction or a constant / affine coefficient (int a b = a^T M b with the
    mass operator, exact for functions in the space).  `order` is accepted and
    unused: the rules are those of the forms (order 2p)."""
    if isinstance(cf, _GFIntegrand) and cf.kind == "graddot":
        if cf.a.fes is not cf.b.fes:
            raise ValueError("grad(a) * grad(b) needs a and b on the same space")
        per = Integrate_grad_dot(cf.a.fes, cf.a.vec, cf.b.vec)
        return per if element_wise else float(per.sum())
    if element_wise:
        raise NotImplementedError("element-wise Integrate takes grad(a) * grad(b) of GridFunctions")
    if isinstance(cf, _GFIntegrand):
        a, b = cf.a, cf.b
    elif _gf_factor(cf):
        a, b = cf, 1.0
    else:
        raise NotImplementedError("Integrate takes grad(a)*grad(b), a*b or a single factor of GridFunctions "
                                  "and constant or affine coefficients")
    fes = next((f.fes for f in (a, b) if isinstance(f, GridFunction)), None)
    if fes is None:
        raise NotImplementedError("Integrate of coefficients alone: multiply by a GridFunction of the space")
    return _mass_integral(fes, a, b)


def _space_vector(fes, f, like):
    """f as a DOF vector of fes: a GridFunction's own, else the interpolant."""
    if isinstance(f, GridFunction):
        return f.vec
    if not isinstance(f, _AffineCF):
        f = _AffineCF((0.0, 0.0, 0.0), float(np.asarray(getattr(f, "values", f), dtype=np.float64)))
    fi = torch.zeros_like(like.t)
    pts = fes.mesh.raw.points
    fi[:len(pts)] = torch.as_tensor(f.vertex_values(pts), dtype=fi.dtype, device=fi.device)
    return BaseVector(data=fi)


def _mass_integral(fes, a, b):
    """int a b = a^T M b, with the matrix-free mass operator of fes (built once
    per space)."""
    if isinstance(fes, VectorH1) and any(not isinstance(f, GridFunction) for f in (a, b)):
        # a coefficient's interpolant lives in a scalar space; on VectorH1 the
        # integral of a coefficient times a vector field is a vector
        raise NotImplementedError("Integrate of a coefficient times a GridFunction takes scalar H1 only")
    if getattr(fes, "_mass_form", None) is None:
        u, v = fes.TnT()
        m = BilinearForm(fes, nonassemble=True)
        m += u * v * dx
        fes._mass_form = m.Assemble()
    like = next(f.vec for f in (a, b) if isinstance(f, GridFunction))
    av, bv = _space_vector(fes, a, like), _space_vector(fes, b, like)
    mb = bv.CreateVector()
    fes._mass_form.mat.Mult(bv, mb)
    return av.InnerProduct(mb)


def Integrate_grad_dot(fes, u, w):
    """Element-wise int_e grad u . grad w (Integrate(..., element_wise=True)).
    u and w are DOF vectors of the scalar H1 space fes: contiguous FP64 CUDA
    tensors of length fes.ndof (the kernel reads fes.ndof doubles of each)."""
    if isinstance(fes, VectorH1):
        raise TypeError("Integrate_grad_dot takes a scalar H1 space")
    u, w = _as_vec(u), _as_vec(w)
    for t in (u.t, w.t):
        if t.dtype != torch.float64:
            raise TypeError("grad(a) * grad(b) takes FP64 vectors")
        if not (t.is_cuda and t.is_contiguous()):
            raise TypeError("grad(a) * grad(b) takes contiguous CUDA vectors")
        if t.numel() != fes.ndof:
            raise ValueError("vector length %d does not match the space (%d DOFs)" % (t.numel(), fes.ndof))
    ctx = fes.ctx.sync_stream()
    out = torch.zeros(fes.ne, dtype=torch.float64, device=u.t.device)
    ctx.check(ctx.lib.gh1_elem_grad_dot(fes.h, _ptr(u.t), _ptr(w.t), _ptr(out)))
    return out


def ShapeEval(et, order, vnums, pts, device=0):
    """Shape values and reference gradients evaluated on the GPU."""
    ctx = context(device)
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
    vn = np.ascontiguousarray(vnums, dtype=np.int32)
    n = (order + 1) * (order + 2) * (order + 3) // 6 if et == 4 else (order + 1) ** 3
    val = np.zeros((len(pts), n))
    grd = np.zeros((len(pts), n, 3))
    ctx.check(ctx.lib.gh1_shape_eval(ctx.h, et, order, _np_ptr(vn), len(pts), _np_ptr(pts), _np_ptr(val), _np_ptr(grd)))
    return val, grd


class _Globals:
    """ngsglobals: msg_level is kept and has no effect (the library prints
    nothing)."""
    msg_level = 0


ngsglobals = _Globals()


class TaskManager:
    """`with TaskManager():` of NGSolve scripts.  NGSolve's TaskManager starts its
    CPU worker threads; here the work runs on the GPU stream and the host-side
    setup threads itself, so entering and leaving does nothing."""

    def __init__(self, pajetrace=None, **kwargs):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


def SetNumThreads(n):
    """NGSolve's CPU thread count; nothing to set on the GPU path."""
    return None


def SetHeapSize(size):
    """NGSolve's LocalHeap size; the GPU path keeps no such heap."""
    return None
