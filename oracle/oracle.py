"""ctypes front end of the FP64 CPU oracle (``gh1_oracle.cpp``).

TEST INFRASTRUCTURE ONLY.  The oracle restates NGSolve's H1 assemble / apply /
CG algorithms on the CPU; the GPU results are compared with it.  Only the
tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
import this module, and only to compare against or time the reference
algorithm -- never as a product code path.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libgh1_oracle.so")
_lib = None


def build(force=False):
    """Compile the oracle with g++ -O3 -fopenmp (portable flags: x86 and Arm)."""
    src = os.path.join(_HERE, "gh1_oracle.cpp")
    if not force and os.path.exists(_SO) and os.path.getmtime(_SO) >= os.path.getmtime(src):
        return _SO
    os.makedirs(os.path.dirname(_SO), exist_ok=True)
    tmp = _SO + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c++17",
                           src, "-o", tmp])
    os.replace(tmp, _SO)
    return _SO


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_SO)
        P = ctypes.c_void_p
        i, l, d = ctypes.c_int, ctypes.c_long, ctypes.c_double
        L.orc_space_create.restype = P
        L.orc_space_create.argtypes = [i, i, P, i, P, i]
        L.orc_space_create_bnd.restype = P
        L.orc_space_create_bnd.argtypes = [i, i, P, i, P, i, l, P]
        L.orc_space_destroy.argtypes = [P]
        L.orc_space_info.argtypes = [P, P]
        L.orc_space_dofs.argtypes = [P, P]
        L.orc_space_freedofs.argtypes = [P, P]
        L.orc_space_topology.argtypes = [P, P, P]
        L.orc_graph.restype = l
        L.orc_graph.argtypes = [P]
        L.orc_graph_get.argtypes = [P, P, P]
        L.orc_assemble.argtypes = [P, P, P, P, i]
        L.orc_assemble_k6.argtypes = [P, P, P, P, i]
        L.orc_apply_mf_k6.argtypes = [P, P, P, P, P, i, i]
        L.orc_element_matrix.argtypes = [P, i, d, d, P]
        L.orc_spmv.argtypes = [l, P, P, P, d, P, P, i]
        L.orc_apply_mf.argtypes = [P, P, P, P, P, i, i]
        L.orc_apply_bdb.argtypes = [P, P, i, i, P, P, P]
        L.orc_smoothing_blocks.argtypes = [P, i, P, P, P]
        L.orc_space_set_deformation.argtypes = [P, P, P]
        L.orc_rhs_rule.argtypes = [P, P, i, P, P]
        L.orc_smoothing_blocks.restype = l
        L.orc_diag_bdb.argtypes = [P, P, i, i, P, P]
        L.orc_rhs.argtypes = [P, P, P]
        L.orc_elem_grad_dot.argtypes = [P, P, P, P]
        L.orc_shapes.argtypes = [i, i, P, i, P, P, P]
        L.orc_dubiner2d.argtypes = [i, d, d, P]
        L.orc_dubiner3d.argtypes = [i, d, d, d, P]
        L.orc_rule.argtypes = [i, i, P, P]
        L.orc_cg.argtypes = [P, l, P, P, P, P, P, P, P, P, d, i, P, P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class OracleSpace:
    """H1 space of uniform order p on a tet (et=4) or hex (et=8) mesh.
    dirichlet_faces: (nbf, 3 | 4) boundary faces whose closure is Dirichlet
    (default: the whole boundary, as freedofs() reports it)."""

    def __init__(self, points, elements, order, dirichlet_faces=None):
        self.points = np.ascontiguousarray(points, dtype=np.float64)
        self.elements = np.ascontiguousarray(elements, dtype=np.int32)
        self.et = int(self.elements.shape[1])
        self.order = int(order)
        self.ne = int(self.elements.shape[0])
        self.h = None
        if dirichlet_faces is None:
            self.h = lib().orc_space_create(self.et, len(self.points), _p(self.points), self.ne,
                                            _p(self.elements), self.order)
        else:
            fc = np.ascontiguousarray(dirichlet_faces, dtype=np.int32)
            self.h = lib().orc_space_create_bnd(self.et, len(self.points), _p(self.points), self.ne,
                                                _p(self.elements), self.order, len(fc), _p(fc))
            if not self.h:
                raise ValueError("a Dirichlet face is not a boundary face of the mesh")
        info = np.zeros(7, dtype=np.int64)
        lib().orc_space_info(self.h, _p(info))
        self.ndof, self.nloc, self.ned, self.nfa = (int(v) for v in info[:4])
        self.first_edge, self.first_face, self.first_cell = (int(v) for v in info[4:])
        self._csr = None

    def __del__(self):
        try:
            lib().orc_space_destroy(self.h)
        except Exception:
            pass

    def element_dofs(self):
        out = np.zeros((self.ne, self.nloc), dtype=np.int32)
        lib().orc_space_dofs(self.h, _p(out))
        return out

    def freedofs(self):
        out = np.zeros(self.ndof, dtype=np.uint8)
        lib().orc_space_freedofs(self.h, _p(out))
        return out

    def topology(self):
        ned = 6 if self.et == 4 else 12
        nfa = 4 if self.et == 4 else 6
        ee = np.zeros((self.ne, ned), dtype=np.int32)
        ff = np.zeros((self.ne, nfa), dtype=np.int32)
        lib().orc_space_topology(self.h, _p(ee), _p(ff))
        return ee, ff

    def graph(self):
        if self._csr is None:
            nnz = lib().orc_graph(self.h)
            rowptr = np.zeros(self.ndof + 1, dtype=np.int64)
            colind = np.zeros(nnz, dtype=np.int32)
            lib().orc_graph_get(self.h, _p(rowptr), _p(colind))
            self._csr = (rowptr, colind)
        return self._csr

    def assemble(self, kappa=None, mu=None, reverse=False, K6=None):
        """CSR of the assembled form; reverse=True sums quadrature points in the
        opposite order (the rounding noise of the algorithm).  K6 (ne, 6): the
        element-wise symmetric diffusion tensor (xx yy zz xy xz yz) in place of
        kappa."""
        rowptr, colind = self.graph()
        vals = np.zeros(len(colind), dtype=np.float64)
        k = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
        m = None if mu is None else np.ascontiguousarray(mu, dtype=np.float64)
        if K6 is not None:
            k6 = np.ascontiguousarray(K6, dtype=np.float64).reshape(self.ne, 6)
            rc = lib().orc_assemble_k6(self.h, _p(k6), _p(m), _p(vals), 1 if reverse else 0)
        else:
            rc = lib().orc_assemble(self.h, _p(k), _p(m), _p(vals), 1 if reverse else 0)
        if rc != 0:
            raise RuntimeError("illegal dnums in AddElementMatrix")
        return rowptr, colind, vals

    def element_matrix(self, e, kappa=1.0, mu=0.0):
        K = np.zeros((self.nloc, self.nloc))
        lib().orc_element_matrix(self.h, int(e), float(kappa), float(mu), _p(K))
        return K

    def apply_mf(self, x, kappa=None, mu=None, e0=0, e1=-1, K6=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.ndof)
        k = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
        m = None if mu is None else np.ascontiguousarray(mu, dtype=np.float64)
        if K6 is not None:
            k6 = np.ascontiguousarray(K6, dtype=np.float64).reshape(self.ne, 6)
            lib().orc_apply_mf_k6(self.h, _p(k6), _p(m), _p(x), _p(y), int(e0), int(e1))
        else:
            lib().orc_apply_mf(self.h, _p(k), _p(m), _p(x), _p(y), int(e0), int(e1))
        return y

    def _bdb_args(self, D, rule):
        D = np.ascontiguousarray(D, dtype=np.float64)
        per_point = 0 if D.size == self.ne * 16 else 1
        r = None if rule is None else np.ascontiguousarray(rule, dtype=np.float64).reshape(-1, 4)
        if per_point and (r is None or D.size != self.ne * len(r) * 16):
            raise ValueError("a point-wise D needs the rule it is given at, D[ne][nq][16]")
        return D, per_point, (0 if r is None else len(r)), r

    def apply_bdb(self, x, D, rule=None):
        """Generic B^T D B apply: D[ne][4][4] (or [ne][nq][4][4] at rule's points),
        rows test (v, grad v), columns trial (u, grad u), physical coordinates."""
        D, pp, nq, r = self._bdb_args(D, rule)
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.ndof)
        lib().orc_apply_bdb(self.h, _p(D), pp, nq, _p(r), _p(x), _p(y))
        return y

    def diag_bdb(self, D, rule=None):
        D, pp, nq, r = self._bdb_args(D, rule)
        d = np.zeros(self.ndof)
        lib().orc_diag_bdb(self.h, _p(D), pp, nq, _p(r), _p(d))
        return d

    def smoothing_blocks(self, blocktype=4):
        """CreateSmoothingBlocks: (offsets int64, dofs int32), rows sorted, empty rows dropped."""
        nt = np.zeros(1, dtype=np.int64)
        nb = lib().orc_smoothing_blocks(self.h, int(blocktype), _p(nt), None, None)
        off = np.zeros(nb + 1, dtype=np.int64)
        dofs = np.zeros(max(int(nt[0]), 1), dtype=np.int32)
        lib().orc_smoothing_blocks(self.h, int(blocktype), _p(nt), _p(off), _p(dofs))
        return off, dofs[:int(nt[0])]

    def rhs(self, f_elem, rule=None):
        f = np.ascontiguousarray(f_elem, dtype=np.float64)
        b = np.zeros(self.ndof)
        if rule is None:
            lib().orc_rhs(self.h, _p(f), _p(b))
        else:
            r = np.ascontiguousarray(rule, dtype=np.float64).reshape(-1, 4)
            lib().orc_rhs_rule(self.h, _p(f), len(r), _p(r), _p(b))
        return b

    def set_deformation(self, def_space, d):
        """Curved elements: d = [3 * def_space.ndof] displacement in def_space (same mesh), None removes it."""
        if d is None:
            lib().orc_space_set_deformation(self.h, None, None)
            self._def = None
            return
        d = np.ascontiguousarray(d, dtype=np.float64)
        assert d.size == 3 * def_space.ndof
        self._def = (def_space, d)  # keeps the field's space alive
        lib().orc_space_set_deformation(self.h, def_space.h, _p(d))

    def elem_grad_dot(self, u, w):
        u = np.ascontiguousarray(u, dtype=np.float64)
        w = np.ascontiguousarray(w, dtype=np.float64)
        out = np.zeros(self.ne)
        lib().orc_elem_grad_dot(self.h, _p(u), _p(w), _p(out))
        return out

    def cg(self, b, invdiag, tol=1e-10, maxit=10000, csr=None, kappa=None, mu=None, x0=None):
        """CGSolver._SolveImpl on CSR (csr=(rowptr,colind,vals)) or matrix-free."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.ndof) if x0 is None else np.array(x0, dtype=np.float64)
        hist = np.zeros(maxit + 2)
        its = np.zeros(1, dtype=np.int32)
        invdiag = np.ascontiguousarray(invdiag, dtype=np.float64)
        k = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
        m = None if mu is None else np.ascontiguousarray(mu, dtype=np.float64)
        if csr is not None:
            rp, ci, va = csr
            lib().orc_cg(self.h, self.ndof, _p(rp), _p(ci), _p(va), None, None, _p(invdiag),
                         _p(b), _p(x), tol, maxit, _p(hist), _p(its))
        else:
            lib().orc_cg(self.h, self.ndof, None, None, None, _p(k), _p(m), _p(invdiag),
                         _p(b), _p(x), tol, maxit, _p(hist), _p(its))
        n = int(its[0])
        return x, n, hist[:n].copy()


def spmv(rowptr, colind, vals, x, s=1.0):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(len(rowptr) - 1)
    lib().orc_spmv(len(rowptr) - 1, _p(rowptr), _p(colind), _p(vals), float(s), _p(x), _p(y), 0)
    return y


def shapes(et, order, vnums, pts):
    vn = np.ascontiguousarray(vnums, dtype=np.int32)
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
    n = (order + 1) * (order + 2) * (order + 3) // 6 if et == 4 else (order + 1) ** 3
    val = np.zeros((len(pts), n))
    grad = np.zeros((len(pts), n, 3))
    rc = lib().orc_shapes(et, order, _p(vn), len(pts), _p(pts), _p(val), _p(grad))
    assert rc == n
    return val, grad


def rule(et, order):
    n = lib().orc_rule(et, order, None, None)
    pts = np.zeros((n, 3))
    w = np.zeros(n)
    lib().orc_rule(et, order, _p(pts), _p(w))
    return pts, w


def dubiner2d(n, x, y):
    out = np.zeros((n + 1) * (n + 2) // 2)
    lib().orc_dubiner2d(n, x, y, _p(out))
    return out


def dubiner3d(n, x, y, z):
    out = np.zeros((n + 1) * (n + 2) * (n + 3) // 6)
    lib().orc_dubiner3d(n, x, y, z, _p(out))
    return out


def max_threads():
    return int(lib().orc_max_threads())
