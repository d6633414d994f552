"""Pins of the CPU oracle (the FP64 reference of the GPU library) against the
reference's own known answers and closed-form properties."""
import math

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from oracle import oracle as O
from ngsolve_gb300.meshes import MakeStructured3DMesh, JitterInterior, ReadVolMesh, Mesh
from tests.util import lognormal


def test_p1_mass_golden_cube_vol(cube_vol, golden):
    """tests/pytest/test_matrix.py:84-93: H1 order-1 mass a.mat[1,1] on cube.vol.gz."""
    pts, tets = cube_vol
    S = O.OracleSpace(pts, tets, 1)
    rp, ci, va = S.assemble(kappa=np.zeros(len(tets)), mu=np.ones(len(tets)))
    k = rp[1] + np.searchsorted(ci[rp[1]:rp[2]], 1)
    g = golden["p1_mass_cube_vertex1"]
    assert abs(va[k] - g["value"]) < g["tolerance"]
    assert abs(va[k] - g["value"]) < 1e-17  # exact rule: agreement to rounding


def test_dof_and_nnz_counts(golden):
    c = golden["counts"]
    m = MakeStructured3DMesh(hexes=True, nx=16)
    S = O.OracleSpace(m.points, m.elements, 3)
    rp, ci = S.graph()
    assert S.ndof == c["hex16_p3"]["ndof"] and len(ci) == c["hex16_p3"]["nnz"]
    assert int(S.freedofs().sum()) == c["hex16_p3"]["free"]
    m = MakeStructured3DMesh(hexes=False, nx=32)
    S = O.OracleSpace(m.points, m.elements, 2)
    assert S.ndof == c["kuhn32_p2"]["ndof"] and len(S.graph()[1]) == c["kuhn32_p2"]["nnz"]


@pytest.mark.parametrize("et,p", [(4, p) for p in range(1, 9)] + [(8, p) for p in range(1, 6)])
def test_element_ndof(et, p):
    """GetFE(el).ndof == len(GetDofNrs(el)) (tests/pytest/test_fespaces.py:55-100)."""
    m = MakeStructured3DMesh(hexes=(et == 8), nx=2)
    S = O.OracleSpace(m.points, m.elements, p)
    d = S.element_dofs()
    n = (p + 1) * (p + 2) * (p + 3) // 6 if et == 4 else (p + 1) ** 3
    assert d.shape[1] == n
    for e in range(S.ne):
        assert len(set(d[e])) == n


def _dubiner2d_norms(n):
    # CalcNormInv of DubinerBasisOrthoBub (fem/recursive_pol.hpp:2864-2874)
    out = []
    for i in range(n + 1):
        for j in range(n - i + 1):
            out.append(0.5 * (5 + 2 * i + 2 * j) * (4 + 2 * i + j) * (j + 1) * (2 * i + 3) * (2 * i + 4) / (i + 1))
    return np.array(out)


def _dubiner3d_norms(n):
    # CalcNormInv of DubinerBasis3DOrthoBub (fem/recursive_pol.hpp:3011-3023)
    out = []
    for i in range(n + 1):
        for j in range(n - i + 1):
            for k in range(n - i - j + 1):
                out.append(0.5 * (7 + 2 * i + 2 * j + 2 * k) * (6 + 2 * i + 2 * j + k) * (k + 1) * (5 + 2 * i + 2 * j) *
                           (4 + 2 * i + j) * (j + 1) * (2 * i + 3) * (2 * i + 4) / (i + 1))
    return np.array(out)


@pytest.mark.parametrize("n", [0, 1, 2, 3])
def test_dubiner2d_orthogonality_norms(n):
    """The triangle bubble basis is orthogonal w.r.t. the cubic bubble weight with
    the inverse norms the reference tabulates; this pins the recursions."""
    g, gw = np.polynomial.legendre.leggauss(12)
    g, gw = 0.5 * (g + 1), 0.5 * gw
    m = (n + 1) * (n + 2) // 2
    M = np.zeros((m, m))
    for a, wa in zip(g, gw):
        for b, wb in zip(g, gw):
            x, y = a, b * (1 - a)  # collapsed map of the unit triangle
            w = wa * wb * (1 - a)
            v = O.dubiner2d(n, x, y)
            M += w * x * y * (1 - x - y) * np.outer(v, v)
    d = np.diag(M)
    assert np.max(np.abs(M - np.diag(d))) < 1e-13 * d.max()
    assert np.allclose(1.0 / d, _dubiner2d_norms(n), rtol=1e-10)


@pytest.mark.parametrize("n", [0, 1, 2])
def test_dubiner3d_orthogonality_norms(n):
    g, gw = np.polynomial.legendre.leggauss(10)
    g, gw = 0.5 * (g + 1), 0.5 * gw
    m = (n + 1) * (n + 2) * (n + 3) // 6
    M = np.zeros((m, m))
    for a, wa in zip(g, gw):
        for b, wb in zip(g, gw):
            for c, wc in zip(g, gw):
                x, y, z = a, b * (1 - a), c * (1 - a) * (1 - b)
                w = wa * wb * wc * (1 - a) ** 2 * (1 - b)
                v = O.dubiner3d(n, x, y, z)
                M += w * x * y * z * (1 - x - y - z) * np.outer(v, v)
    d = np.diag(M)
    assert np.max(np.abs(M - np.diag(d))) < 1e-12 * d.max()
    assert np.allclose(1.0 / d, _dubiner3d_norms(n), rtol=1e-9)


def test_partition_of_unity_kernel():
    """A * (vertex indicator) = 0 for the Neumann Laplacian (vertex shapes sum to 1)."""
    for hexes, p in [(True, 3), (False, 4)]:
        m = JitterInterior(MakeStructured3DMesh(hexes=hexes, nx=3), 0.05, 1)
        S = O.OracleSpace(m.points, m.elements, p)
        rp, ci, va = S.assemble(kappa=lognormal(S.ne, 1.0, 3))
        A = sp.csr_matrix((va, ci, rp), shape=(S.ndof, S.ndof))
        v = np.zeros(S.ndof)
        v[:m.nv] = 1
        assert np.abs(A @ v).max() < 1e-13 * np.abs(va).max()


@pytest.mark.parametrize("p", [2, 3, 4])
def test_hex_p_exactness(p):
    """u = x(1-x)y(1-y)z(1-z) is in Q_p (p >= 2): the discrete solution is exact
    (principle of tests/pytest/test_solvers.py:58-79, error <= 1e-12)."""
    m = MakeStructured3DMesh(hexes=True, nx=3)
    S = O.OracleSpace(m.points, m.elements, p)
    # f = -Lap u is in Q_2 but not piecewise constant: assemble the load with a
    # quadrature-exact projection -- the L2 projection of u onto V_h reproduces u,
    # so solve  A x = A_f (x_u)  where x_u = M^-1 (u,v): check A-consistency
    rp, ci, va = S.assemble(kappa=np.zeros(S.ne), mu=np.ones(S.ne))
    M = sp.csr_matrix((va, ci, rp), shape=(S.ndof, S.ndof))
    # (u, v) by tensor Gauss on each element via the oracle rule
    pts, w = O.rule(8, 2 * p + 4)
    d = S.element_dofs()
    b = np.zeros(S.ndof)
    for e in range(S.ne):
        X = m.points[m.elements[e]]
        lo, hi = X.min(0), X.max(0)
        phys = lo + (hi - lo) * pts[:, [2, 1, 0]]  # hex local x is physical z (MakeStructured3DMesh order)
        u = np.prod(phys * (1 - phys), axis=1)
        val, _ = O.shapes(8, p, m.elements[e], pts)
        b[d[e]] += (w * u * np.prod(hi - lo)) @ val
    xu = spla.spsolve(M.tocsc(), b)
    # evaluate the projection at the nodes of element 0 and compare with u
    val, _ = O.shapes(8, p, m.elements[0], pts)
    X = m.points[m.elements[0]]
    lo, hi = X.min(0), X.max(0)
    phys = lo + (hi - lo) * pts[:, [2, 1, 0]]
    assert np.abs(val @ xu[d[0]] - np.prod(phys * (1 - phys), axis=1)).max() < 1e-12
    # Galerkin solve with f = -Lap u reproduces u
    rp2, ci2, va2 = S.assemble()
    A = sp.csr_matrix((va2, ci2, rp2), shape=(S.ndof, S.ndof))
    fb = np.zeros(S.ndof)
    for e in range(S.ne):
        X = m.points[m.elements[e]]
        lo, hi = X.min(0), X.max(0)
        phys = lo + (hi - lo) * pts[:, [2, 1, 0]]
        q = phys * (1 - phys)
        f = 2 * (q[:, 1] * q[:, 2] + q[:, 0] * q[:, 2] + q[:, 0] * q[:, 1])
        val, _ = O.shapes(8, p, m.elements[e], pts)
        fb[d[e]] += (w * f * np.prod(hi - lo)) @ val
    # residual of the exact solution in the Galerkin system (the solution error
    # itself is amplified by cond(A_ff) ~ 1e6..1e9 of the hierarchical basis)
    free = S.freedofs().astype(bool)
    xf = np.where(free, xu, 0.0)
    r = (A @ xf)[free] - fb[free]
    assert np.abs(r).max() < 1e-11 * np.abs(fb).max()


def test_oracle_cg_reference_rule():
    """CG iterates follow krylovspace.py: residual history = sqrt|w.d|."""
    m = MakeStructured3DMesh(hexes=True, nx=4)
    S = O.OracleSpace(m.points, m.elements, 2)
    rp, ci, va = S.assemble()
    free = S.freedofs().astype(bool)
    diag = va[[rp[i] + np.searchsorted(ci[rp[i]:rp[i + 1]], i) for i in range(S.ndof)]]
    inv = np.where(free, 1.0 / diag, 0.0)
    b = S.rhs(np.random.default_rng(1).uniform(-1, 1, S.ne))
    x, its, hist = S.cg(b, inv, tol=1e-10, maxit=500, csr=(rp, ci, va))
    assert hist[-1] <= 1e-10 * hist[0] and hist[-2] > 1e-10 * hist[0]
    A = sp.csr_matrix((va, ci, rp), shape=(S.ndof, S.ndof))
    xr = np.zeros(S.ndof)
    xr[free] = spla.spsolve(A[free][:, free].tocsc(), b[free])
    assert np.abs(x - xr).max() < 1e-8 * np.abs(xr).max()


@pytest.mark.parametrize("nblocks", [1, 3])
def test_cg_history_bound_accepts_rounding(nblocks):
    """The CG history bound of the GPU parity tests holds between two oracle CG
    runs whose matrices differ only by a 2e-16 relative rounding of each entry
    (scalar and 3-block VectorH1 systems, hex p=3 as in those tests); their
    iteration counts differ by at most one and their solutions by 1e-9."""
    from tests.util import assert_cg_history_close
    m = JitterInterior(MakeStructured3DMesh(hexes=True, nx=4), 0.1 / 4, 21)
    S = O.OracleSpace(m.points, m.elements, 3)
    rp, ci, va = S.assemble(kappa=lognormal(S.ne, 1.0, 35))
    free = S.freedofs().astype(bool)
    diag = va[[rp[i] + np.searchsorted(ci[rp[i]:rp[i + 1]], i) for i in range(S.ndof)]]
    f = np.random.default_rng(36).uniform(-1, 1, (nblocks, S.ne))
    b = np.concatenate([S.rhs(f[c]) for c in range(nblocks)])
    inv = np.tile(np.where(free, 1.0 / diag, 0.0), nblocks)
    n, nnz = S.ndof, len(va)
    brp = np.concatenate([rp[:-1] + c * nnz for c in range(nblocks)] + [[nblocks * nnz]]).astype(rp.dtype)
    bci = np.concatenate([ci + c * n for c in range(nblocks)]).astype(ci.dtype)
    runs = []
    for vals in (va, va * (1 + 2e-16 * np.random.default_rng(1).standard_normal(nnz))):
        bva = np.tile(vals, nblocks)  # held: the oracle takes a raw pointer
        x = np.zeros(nblocks * n)
        hist = np.zeros(3002)
        its = np.zeros(1, dtype=np.int32)
        O.lib().orc_cg(None, nblocks * n, O._p(brp), O._p(bci), O._p(bva), None, None, O._p(inv),
                       O._p(b), O._p(x), 1e-10, 3000, O._p(hist), O._p(its))
        runs.append((x, int(its[0]), hist[:int(its[0])]))
    (xa, ia, ha), (xb, ib, hb) = runs
    assert abs(ia - ib) <= 1
    assert_cg_history_close(hb, ha)
    assert np.abs(xa - xb).max() <= 1e-9 * np.abs(xa).max()


def test_matfree_equals_csr_oracle():
    m = JitterInterior(MakeStructured3DMesh(hexes=True, nx=3), 0.08, 2)
    S = O.OracleSpace(m.points, m.elements, 3)
    k = lognormal(S.ne, 1.0, 4)
    mu = lognormal(S.ne, 0.5, 5)
    rp, ci, va = S.assemble(kappa=k, mu=mu)
    x = np.random.default_rng(6).normal(size=S.ndof)
    y = S.apply_mf(x, kappa=k, mu=mu)
    assert np.abs(y - O.spmv(rp, ci, va, x)).max() < 1e-13 * np.abs(y).max()


def test_vol_reader_roundtrip(tmp_path):
    m = MakeStructured3DMesh(hexes=False, nx=2)
    path = tmp_path / "m.vol"
    with open(path, "w") as fh:
        fh.write("mesh3d\nvolumeelements\n%d\n" % m.ne)
        for e in m.elements:
            fh.write("1 4 %s\n" % " ".join(str(v + 1) for v in e))
        fh.write("points\n%d\n" % m.nv)
        for p in m.points:
            fh.write("%.16f %.16f %.16f\n" % tuple(p))
        fh.write("endmesh\n")
    r = ReadVolMesh(str(path))
    assert np.array_equal(r.elements, m.elements) and np.allclose(r.points, m.points)


def _spd_tensors(ne, seed):
    """Element-wise symmetric positive definite tensors as (xx yy zz xy xz yz)."""
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(ne, 3, 3))
    K = A @ A.transpose(0, 2, 1) + 0.5 * np.eye(3)
    return np.stack([K[:, 0, 0], K[:, 1, 1], K[:, 2, 2], K[:, 0, 1], K[:, 0, 2], K[:, 1, 2]], axis=1)


@pytest.mark.parametrize("hexes,p", [(True, 2), (False, 2), (True, 3)])
def test_oracle_tensor_diffusion(hexes, p):
    """(K grad u).grad v with an element-wise tensor: u = x + 2y + 3z (exact in
    the vertex functions on the unit cube) gives u^T A u = g^T K g, g = (1,2,3),
    for a constant K (this pins the placement of every off-diagonal entry);
    K = kappa I reproduces the scalar-kappa matrix; the matrix-free apply equals
    the assembled matrix; the operator is linear in K."""
    m = MakeStructured3DMesh(hexes=hexes, nx=2)
    S = O.OracleSpace(m.points, m.elements, p)
    K1 = np.array([2.0, 3.0, 5.0, 0.7, -0.4, 1.1])
    rp, ci, va = S.assemble(K6=np.tile(K1, (S.ne, 1)))
    A = sp.csr_matrix((va, ci, rp), shape=(S.ndof, S.ndof))
    u = np.zeros(S.ndof)
    P = m.points
    u[:len(P)] = P[:, 0] + 2 * P[:, 1] + 3 * P[:, 2]
    g = np.array([1.0, 2.0, 3.0])
    Km = np.array([[K1[0], K1[3], K1[4]], [K1[3], K1[1], K1[5]], [K1[4], K1[5], K1[2]]])
    assert abs(u @ (A @ u) - g @ Km @ g) < 1e-12 * abs(g @ Km @ g)
    # kappa I
    m2 = JitterInterior(MakeStructured3DMesh(hexes=hexes, nx=3), 0.08, 3)
    S2 = O.OracleSpace(m2.points, m2.elements, p)
    kap = lognormal(S2.ne, 1.0, 4)
    _, _, v_iso = S2.assemble(kappa=kap)
    _, _, v_ten = S2.assemble(K6=np.stack([kap, kap, kap, 0 * kap, 0 * kap, 0 * kap], axis=1))
    assert np.abs(v_ten - v_iso).max() <= 1e-14 * np.abs(v_iso).max()
    # matrix-free = assembled, and linearity in K
    Ka, Kb = _spd_tensors(S2.ne, 5), _spd_tensors(S2.ne, 6)
    mu = lognormal(S2.ne, 0.5, 7)
    rp2, ci2, va_a = S2.assemble(K6=Ka, mu=mu)
    x = np.random.default_rng(8).normal(size=S2.ndof)
    y = S2.apply_mf(x, K6=Ka, mu=mu)
    assert np.abs(y - O.spmv(rp2, ci2, va_a, x)).max() <= 1e-13 * np.abs(y).max()
    _, _, va_b = S2.assemble(K6=Kb)
    _, _, va_ab = S2.assemble(K6=Ka + Kb, mu=mu)
    assert np.abs(va_ab - (va_a + va_b)).max() <= 1e-13 * np.abs(va_ab).max()


@pytest.mark.parametrize("hexes", [True, False])
def test_structured_boundary_names(hexes):
    """The structured cube names its sides as the reference does: x=0 back,
    y=0 left, x=1 front, y=1 right, z=0 bottom, z=1 top (also under a mapping,
    which does not change the lattice); each side has n^2 quads or 2 n^2
    triangles, and they are exactly the faces with one adjacent element."""
    n = 3
    m = MakeStructured3DMesh(hexes=hexes, nx=n, mapping=lambda x, y, z: (2 * x, y + 0.1 * x, z))
    assert m.GetBoundaries() == ("back", "left", "front", "right", "bottom", "top")
    plain = MakeStructured3DMesh(hexes=hexes, nx=n)
    P = plain.points
    for side, (ax, v) in enumerate(((0, 0), (1, 0), (0, 1), (1, 1), (2, 0), (2, 1))):
        f = m.BoundaryFaces(m.GetBoundaries()[side])
        assert len(f) == (1 if hexes else 2) * n * n
        assert np.all(np.abs(P[f][..., ax] - v) < 1e-14)
    S = O.OracleSpace(m.points, m.elements, 1)
    allf = m.BoundaryFaces(".*")
    # every boundary face once: the whole-boundary mask equals the listed faces'
    assert np.array_equal(S.freedofs(), O.OracleSpace(m.points, m.elements, 1, dirichlet_faces=allf).freedofs())
    assert len(np.unique(np.sort(allf, axis=1), axis=0)) == len(allf) == 6 * (1 if hexes else 2) * n * n


@pytest.mark.parametrize("hexes,p", [(True, 2), (True, 4), (False, 3)])
def test_oracle_dirichlet_regions(hexes, p):
    """Dirichlet on selected sides: exactly the DOFs of the selected faces' closure
    (vertices, edges, faces, counted here from the faces themselves) are not
    free; an interior face is rejected; no face leaves every DOF free."""
    m = JitterInterior(MakeStructured3DMesh(hexes=hexes, nx=3), 0.05, 9)
    for regex in ("bottom", "left|top", "back|front|right"):
        faces = m.BoundaryFaces(regex)
        S = O.OracleSpace(m.points, m.elements, p, dirichlet_faces=faces)
        fv = faces.shape[1]
        verts = np.unique(faces)
        edges = np.unique(np.sort(np.stack([faces, np.roll(faces, -1, axis=1)], axis=2).reshape(-1, 2), axis=1),
                          axis=0)
        nfd = (p - 1) ** 2 if hexes else max(0, (p - 1) * (p - 2) // 2)
        expect = len(verts) + len(edges) * (p - 1) + len(faces) * nfd
        fd = S.freedofs().astype(bool)
        assert (~fd).sum() == expect
        assert not fd[verts].any() and fd[np.setdiff1d(np.arange(m.nv), verts)].all()
        assert fv == (4 if hexes else 3)
    assert O.OracleSpace(m.points, m.elements, p, dirichlet_faces=np.zeros((0, 4 if hexes else 3))).freedofs().all()
    interior = np.sort(m.elements[:, :3] if not hexes else m.elements[:, [0, 1, 2, 3]], axis=1)
    inner = [f for f in interior if not np.all(np.isin(f, np.unique(m.BoundaryFaces(".*"))))][:1]
    with pytest.raises(ValueError):
        O.OracleSpace(m.points, m.elements, p, dirichlet_faces=np.array(inner))


def test_vol_reader_boundary_names(tmp_path):
    """surfaceelements rows (surfnr bcnr domin domout np p1..pnp) and bcnames
    (bcnr name) give named boundary faces; a bc number without a name is
    "default"."""
    pts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.0]])
    path = tmp_path / "t.vol"
    with open(path, "w") as fh:
        fh.write("mesh3d\nsurfaceelements\n4\n")
        for bc, f in ((1, (1, 3, 2)), (1, (1, 2, 4)), (2, (1, 4, 3)), (3, (2, 3, 4))):
            fh.write(" 1 %d 1 0 3 %d %d %d\n" % ((bc,) + f))
        fh.write("volumeelements\n1\n1 4 1 2 3 4\npoints\n4\n")
        for p in pts:
            fh.write("%.16f %.16f %.16f\n" % tuple(p))
        fh.write("bcnames\n2\n1 bottom\n2 side\nendmesh\n")
    r = ReadVolMesh(str(path))
    assert r.GetBoundaries() == ("bottom", "side", "default")
    assert np.array_equal(r.BoundaryFaces("bottom"), [[0, 2, 1], [0, 1, 3]])
    assert len(r.BoundaryFaces("side|default")) == 2 and len(r.BoundaryFaces("nothing")) == 0
    S = O.OracleSpace(r.points, r.elements, 2, dirichlet_faces=r.BoundaryFaces("bottom"))
    assert S.freedofs().sum() == S.ndof - (4 + 5)  # vertices 0..3 and the edges of the two faces


def test_cube_vol_boundary_names():
    """The surface elements of the reference's cube.vol.gz (tests/pytest), read by
    ReadVolMesh into the fixture: they are exactly the tet faces with one
    adjacent element; each named side is one axis-aligned plane, the six
    planes distinct; and Dirichlet on all of them is the whole-boundary mask."""
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "cube_vol.npz"))
    m = Mesh(d["points"], d["tets"], bnd_faces=d["bnd_faces"], bnd_index=d["bnd_index"],
             bc_names=[str(n) for n in d["bc_names"]])
    assert m.GetBoundaries() == ("back", "left", "front", "right", "bottom", "top")
    F = np.sort(m.elements[:, [[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]]].reshape(-1, 3), axis=1)
    uniq, cnt = np.unique(F, axis=0, return_counts=True)
    outer = uniq[cnt == 1]
    listed = np.unique(np.sort(m.BoundaryFaces(".*"), axis=1), axis=0)
    assert len(listed) == len(m.BoundaryFaces(".*")) and np.array_equal(listed, outer)
    planes = set()
    for name in m.GetBoundaries():
        P = m.points[m.BoundaryFaces(name)].reshape(-1, 3)
        ax = int(np.argmin(np.ptp(P, axis=0)))
        assert np.ptp(P[:, ax]) < 1e-12
        planes.add((ax, round(float(P[0, ax]), 9)))
    assert len(planes) == 6
    S = O.OracleSpace(m.points, m.elements, 3)
    Sb = O.OracleSpace(m.points, m.elements, 3, dirichlet_faces=m.BoundaryFaces(".*"))
    assert np.array_equal(S.freedofs(), Sb.freedofs())


@pytest.mark.parametrize("hexes,p", [(True, 1), (True, 3), (False, 2)])
def test_affine_source_identity(hexes, p):
    """For an affine f the load vector of f*v*dx is M I_h(f) (I_h(f): f at the
    vertices, other DOFs zero).  On a jittered unit cube, with f = x:
    1_h . b = int x = 1/2 and I_h(x) . b = int x^2 = 1/3, to round-off (x^2 only
    where the rule is exact for it: x^2 |det J| has degree 4 per direction on a
    trilinear hex, beyond the 2-point rule of p=1); with f = 2x - y + 3:
    1_h . b = int f = 3.5."""
    m = JitterInterior(MakeStructured3DMesh(hexes=hexes, nx=3), 0.05, 12)
    S = O.OracleSpace(m.points, m.elements, p)
    rp, ci, va = S.assemble(kappa=np.zeros(S.ne), mu=np.ones(S.ne))
    M = sp.csr_matrix((va, ci, rp), shape=(S.ndof, S.ndof))
    ones = np.zeros(S.ndof)
    ones[:m.nv] = 1.0
    xi = np.zeros(S.ndof)
    xi[:m.nv] = m.points[:, 0]
    b = M @ xi
    assert abs(ones @ b - 0.5) < 1e-13
    if p >= 2 or not hexes:
        assert abs(xi @ b - 1.0 / 3.0) < 1e-13
    fi = np.zeros(S.ndof)
    fi[:m.nv] = 2 * m.points[:, 0] - m.points[:, 1] + 3
    assert abs(ones @ (M @ fi) - 3.5) < 1e-13


def _bdb_matrix(ne, seed, sym=False):
    """Random D per element (4x4, rows test, columns trial) with an SPD 3x3
    diffusion block, a positive reaction and convection terms."""
    rng = np.random.default_rng(seed)
    D = np.zeros((ne, 4, 4))
    L = rng.normal(size=(ne, 3, 3)) * 0.3
    D[:, 1:, 1:] = np.einsum("eij,ekj->eik", L, L) + np.eye(3)
    D[:, 0, 0] = rng.uniform(0.5, 2.0, ne)
    D[:, 0, 1:] = rng.normal(size=(ne, 3))
    D[:, 1:, 0] = D[:, 0, 1:] if sym else rng.normal(size=(ne, 3))
    return D


@pytest.mark.parametrize("hexes,p", [(True, 1), (True, 3), (False, 2), (False, 4)])
def test_oracle_bdb(hexes, p):
    """The generic B^T D B apply: D = diag(mu, K) reproduces the kappa / tensor +
    mass operator; transposing D transposes the operator; a point-wise D that
    repeats the element's matrix gives the same result; convection b = e_x on the
    interpolant of x is the load vector of f = 1 (b . grad x = 1, x is in the
    space); the diagonal matches the operator's."""
    m = JitterInterior(MakeStructured3DMesh(hexes=hexes, nx=2), 0.05, 3) if not hexes else \
        MakeStructured3DMesh(hexes=True, nx=2)
    S = O.OracleSpace(m.points, m.elements, p)
    ne = S.ne
    rng = np.random.default_rng(11)
    x = rng.normal(size=S.ndof)
    Ka = _spd_tensors(ne, 5)
    mu = lognormal(ne, 0.5, 7)
    D = np.zeros((ne, 4, 4))
    D[:, 0, 0] = mu
    D[:, 1, 1], D[:, 2, 2], D[:, 3, 3] = Ka[:, 0], Ka[:, 1], Ka[:, 2]
    D[:, 1, 2] = D[:, 2, 1] = Ka[:, 3]
    D[:, 1, 3] = D[:, 3, 1] = Ka[:, 4]
    D[:, 2, 3] = D[:, 3, 2] = Ka[:, 5]
    y_ref = S.apply_mf(x, K6=Ka, mu=mu)
    y = S.apply_bdb(x, D)
    assert np.abs(y - y_ref).max() <= 1e-13 * np.abs(y_ref).max()
    # transpose
    Dn = _bdb_matrix(ne, 12)
    z = rng.normal(size=S.ndof)
    a = z @ S.apply_bdb(x, Dn)
    b = x @ S.apply_bdb(z, np.transpose(Dn, (0, 2, 1)))
    assert abs(a - b) <= 1e-12 * max(abs(a), 1.0)
    # point-wise D at the oracle's own rule of order 2p
    pts, w = O.rule(4 if not hexes else 8, 2 * p)
    rule = np.concatenate([pts, w[:, None]], axis=1)
    Dp = np.repeat(Dn[:, None], len(w), axis=1)
    y1, y2 = S.apply_bdb(x, Dn), S.apply_bdb(x, Dp, rule=rule)
    assert np.abs(y1 - y2).max() <= 1e-13 * np.abs(y1).max()
    # convection known answer
    Dc = np.zeros((ne, 4, 4))
    Dc[:, 0, 1] = 1.0
    u = np.zeros(S.ndof)
    u[:len(m.points)] = m.points[:, 0]
    lhs = S.apply_bdb(u, Dc)
    rhs = S.rhs(np.ones(ne))
    assert np.abs(lhs - rhs).max() <= 1e-13 * np.abs(rhs).max()
    # diagonal
    d = S.diag_bdb(Dn)
    idx = rng.choice(S.ndof, 6, replace=False)
    for i in idx:
        e = np.zeros(S.ndof)
        e[i] = 1.0
        assert abs(S.apply_bdb(e, Dn)[i] - d[i]) <= 1e-13 * max(1.0, abs(d[i]))


def _tet_rules_inc():
    """The symmetric tet rules the library compiles in (csrc/tet_rules.inc):
    {degree: (points (n, 3), weights (n,))}."""
    import os
    import re
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "ngsolve_gb300", "csrc",
                        "tet_rules.inc")
    text = open(path).read()
    out = {}
    for m in re.finditer(r"TET_RULE_D(\d+)\[(\d+)\]\[4\] = \{(.*?)\};", text, re.S):
        rows = re.findall(r"\{([^{}]*)\}", m.group(3))
        arr = np.array([[float(v) for v in r.split(",") if v.strip()] for r in rows])
        assert arr.shape == (int(m.group(2)), 4)
        out[int(m.group(1))] = (arr[:, :3], arr[:, 3])
    return out


def test_tet_rules_exact():
    """Every compiled tet rule integrates all monomials x^i y^j z^k of total
    degree <= its degree exactly (i! j! k! / (i+j+k+3)!, relative 1e-14), with
    positive weights and interior points; degree 8 has 46 points."""
    rules = _tet_rules_inc()
    assert sorted(rules) == [1, 2, 5, 6, 8] and len(rules[8][1]) == 46
    for deg, (P, W) in rules.items():
        assert np.all(W > 0) and np.all(P > 0) and np.all(P.sum(1) < 1)
        for i in range(deg + 1):
            for j in range(deg + 1 - i):
                for k in range(deg + 1 - i - j):
                    ex = math.factorial(i) * math.factorial(j) * math.factorial(k) / math.factorial(i + j + k + 3)
                    got = np.sum(W * P[:, 0] ** i * P[:, 1] ** j * P[:, 2] ** k)
                    assert abs(got - ex) <= 1e-14 * ex, (deg, i, j, k)
