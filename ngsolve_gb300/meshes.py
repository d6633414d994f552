"""Mesh generators and readers for the H1 path.

``MakeStructured3DMesh`` mirrors ``ngsolve.meshes.MakeStructured3DMesh``
(python/meshes.py:273-410 of NGSolve): points are numbered with x outermost and
z innermost, hexes list their vertices as
``[base, base+1, base+(nz+1)+1, base+(nz+1), baseup, ...]`` and the tet variant
splits every cube into the six tets of the reference's Kuhn split.  Keeping the
vertex lists identical keeps the element orientation classes identical, which
fixes the orientation of every edge and face shape function.

``ReadVolMesh`` reads the ASCII netgen ``.vol`` / ``.vol.gz`` format (the
``points``, ``volumeelements``, ``surfaceelements`` and ``bcnames`` sections)
used by the reference test meshes.

Boundary faces carry a boundary-condition name, as netgen's surface elements
do, so that ``H1(mesh, dirichlet="left|top")`` can select them by regular
expression.
"""
import gzip
import re

import numpy as np

# local faces of the reference hex (vertices 0-3 bottom, 4-7 top) and tet
_HEX_FACES = np.array([[0, 3, 2, 1], [4, 5, 6, 7], [0, 1, 5, 4], [1, 2, 6, 5], [2, 3, 7, 6], [3, 0, 4, 7]])
_TET_FACES = np.array([[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]])
# names of the structured cube's sides (python/meshes.py:457-475 of NGSolve)
_CUBE_SIDES = ("back", "left", "front", "right", "bottom", "top")


class Mesh:
    """Volume mesh of one element type: ``points`` (nv,3) float64 and
    ``elements`` (ne, 4 | 8) int32 vertex lists in the reference's local order.

    Optional boundary data: ``bnd_faces`` (nbf, 3 | 4) vertex numbers of
    boundary faces, ``bnd_index`` (nbf,) 0-based index of each face's name in
    ``bc_names``."""

    def __init__(self, points, elements, bnd_faces=None, bnd_index=None, bc_names=None):
        self.points = np.ascontiguousarray(points, dtype=np.float64)
        self.elements = np.ascontiguousarray(elements, dtype=np.int32)
        if self.elements.ndim != 2 or self.elements.shape[1] not in (4, 8):
            raise ValueError("elements must be (ne,4) tets or (ne,8) hexes")
        if self.points.ndim != 2 or self.points.shape[1] != 3:
            raise ValueError("points must be (nv,3)")
        if len(self.elements) and (self.elements.min() < 0 or self.elements.max() >= len(self.points)):
            raise ValueError("element vertex index out of range")
        self._bnd = None
        self._bnd_fn = None
        self.bc_names = None
        if bnd_faces is not None:
            faces = np.ascontiguousarray(bnd_faces, dtype=np.int32)
            index = np.ascontiguousarray(bnd_index, dtype=np.int32)
            if faces.ndim != 2 or faces.shape[1] != (3 if self.et == 4 else 4) or index.shape != (len(faces),):
                raise ValueError("bnd_faces must be (nbf, %d) with one bnd_index each" % (3 if self.et == 4 else 4))
            if len(faces) and (faces.min() < 0 or faces.max() >= self.nv):
                raise ValueError("boundary face vertex index out of range")
            if bc_names is None or (len(index) and (index.min() < 0 or index.max() >= len(bc_names))):
                raise ValueError("every bnd_index needs a name in bc_names")
            self._bnd = (faces, index)
            self.bc_names = list(bc_names)

    def _boundary(self):
        if self._bnd is None and self._bnd_fn is not None:
            self._bnd = self._bnd_fn()
        return self._bnd

    def GetBoundaries(self):
        """Names of the boundary conditions (Mesh.GetBoundaries)."""
        return tuple(self.bc_names or ())

    def SelectBoundaries(self, which):
        """Which boundary conditions the FESpace "dirichlet" flag names: a
        regular expression matched in full against each name, or a list of
        1-based boundary-condition numbers.  A bool per name."""
        names = self.bc_names or []
        if isinstance(which, str):
            pat = re.compile(which)
            return np.array([pat.fullmatch(n) is not None for n in names], dtype=bool)
        nums = [int(k) for k in which]
        if any(k < 1 or k > len(names) for k in nums):
            raise ValueError("boundary-condition numbers run from 1 to %d" % len(names))
        hit = np.zeros(len(names), dtype=bool)
        hit[[k - 1 for k in nums]] = True
        return hit

    def BoundaryFaces(self, which):
        """Vertex lists of the boundary faces that `which` (a regex or a list of
        1-based boundary-condition numbers, see SelectBoundaries) selects."""
        bnd = self._boundary()
        if bnd is None:
            raise ValueError("this mesh has no named boundary faces")
        faces, index = bnd
        hit = self.SelectBoundaries(which)
        return faces[hit[index]] if len(hit) else faces[:0]

    def _with_points(self, points):
        m = Mesh(points, self.elements)
        m._bnd, m._bnd_fn, m.bc_names = self._bnd, self._bnd_fn, self.bc_names
        return m

    @property
    def et(self):
        return int(self.elements.shape[1])

    @property
    def nv(self):
        return int(len(self.points))

    @property
    def ne(self):
        return int(len(self.elements))

    def __repr__(self):
        kind = "tet" if self.et == 4 else "hex"
        return "Mesh(%d %ss, %d vertices)" % (self.ne, kind, self.nv)


_KUHN = np.array([[0, 4, 5, 6], [0, 6, 7, 4], [0, 3, 7, 6], [0, 1, 6, 5], [0, 1, 2, 6], [0, 3, 6, 2]])


def MakeStructured3DMesh(hexes=True, nx=10, ny=None, nz=None, mapping=None):
    """Structured mesh of the unit cube (optionally mapped point-wise)."""
    if nz is None:
        if ny is None:
            nz = nx
        else:
            raise ValueError("MakeStructured3DMesh: no default value for nz if nx and ny are provided")
    if ny is None:
        ny = nx
    i, j, k = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    pts = np.stack([i.ravel() / nx, j.ravel() / ny, k.ravel() / nz], axis=1)
    if mapping is not None:
        pts = np.array([mapping(*p) for p in pts], dtype=np.float64)
    ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    base = (ci * (ny + 1) * (nz + 1) + cj * (nz + 1) + ck).ravel()
    baseup = base + (ny + 1) * (nz + 1)
    pnum = np.stack([base, base + 1, base + (nz + 1) + 1, base + (nz + 1),
                     baseup, baseup + 1, baseup + (nz + 1) + 1, baseup + (nz + 1)], axis=1)
    if hexes:
        els = pnum
    else:
        els = pnum[:, _KUHN].reshape(-1, 4)
    mesh = Mesh(pts, els.astype(np.int32))
    mesh.bc_names = list(_CUBE_SIDES)
    mesh._bnd_fn = lambda: _cube_boundary(mesh.elements, nx, ny, nz)
    return mesh


def _cube_boundary(els, nx, ny, nz):
    """Boundary faces of the structured cube and the index of their side: an
    element face whose vertices all lie on one side of the lattice (the
    mapping, if any, does not change the lattice)."""
    local = _HEX_FACES if els.shape[1] == 8 else _TET_FACES
    F = els[:, local].reshape(-1, local.shape[1])
    i, r = np.divmod(F, (ny + 1) * (nz + 1))
    j, k = np.divmod(r, nz + 1)
    faces, index = [], []
    for side, (c, v) in enumerate(((i, 0), (j, 0), (i, nx), (j, ny), (k, 0), (k, nz))):
        on = np.all(c == v, axis=1)
        faces.append(F[on])
        index.append(np.full(int(on.sum()), side, dtype=np.int32))
    return np.ascontiguousarray(np.concatenate(faces), dtype=np.int32), np.concatenate(index)


def MakeHexMesh(nx=10, ny=10, nz=10, mapping=None):
    return MakeStructured3DMesh(hexes=True, nx=nx, ny=ny, nz=nz, mapping=mapping)


def JitterInterior(mesh, amplitude, seed):
    """Move every interior vertex by a seeded uniform offset in
    [-amplitude, amplitude]^3 (boundary vertices stay on the cube faces)."""
    rng = np.random.default_rng(seed)
    pts = mesh.points.copy()
    off = rng.uniform(-amplitude, amplitude, size=pts.shape)
    interior = np.all((pts > 1e-12) & (pts < 1 - 1e-12), axis=1)
    pts[interior] += off[interior]
    return mesh._with_points(pts)


def ReadVolMesh(path):
    """Points, volume elements and (when present) the named boundary faces of an
    ASCII netgen mesh file.  A surface element row is
    ``surfnr bcnr domin domout np p1 .. p_np``; ``bcnames`` rows are
    ``bcnr name``.  A bc number without a name gets the name ``default``."""
    opener = gzip.open if str(path).endswith(".gz") else open
    with opener(path, "rt") as fh:
        lines = fh.read().split("\n")
    pts, els, sels, names = None, None, None, {}
    n = len(lines)
    i = 0
    while i < n:
        tok = lines[i].strip()
        if tok == "surfaceelements":
            cnt = int(lines[i + 1].split()[0])
            rows = [lines[i + 2 + r].split() for r in range(cnt)]
            sels = [(int(row[1]), [int(v) - 1 for v in row[5:5 + int(row[4])]]) for row in rows]
            i += 2 + cnt
            continue
        if tok == "bcnames":
            cnt = int(lines[i + 1].split()[0])
            for r in range(cnt):
                nr, name = lines[i + 2 + r].split()[:2]
                names[int(nr)] = name
            i += 2 + cnt
            continue
        if tok == "volumeelements":
            cnt = int(lines[i + 1].split()[0])
            rows = [lines[i + 2 + r].split() for r in range(cnt)]
            els = [[int(v) - 1 for v in row[2:2 + int(row[1])]] for row in rows]
            i += 2 + cnt
            continue
        if tok == "points":
            cnt = int(lines[i + 1].split()[0])
            pts = [[float(v) for v in lines[i + 2 + r].split()[:3]] for r in range(cnt)]
            i += 2 + cnt
            continue
        i += 1
    if pts is None or els is None:
        raise ValueError("no points/volumeelements section in %s" % path)
    els = np.array(els, dtype=np.int32)
    fv = 3 if els.shape[1] == 4 else 4
    if not sels:
        return Mesh(np.array(pts), els)
    sels = [(bc, v) for bc, v in sels if len(v) == fv]
    bcs = sorted({bc for bc, _ in sels})
    slot = {bc: k for k, bc in enumerate(bcs)}
    return Mesh(np.array(pts), els, bnd_faces=np.array([v for _, v in sels], dtype=np.int32).reshape(-1, fv),
                bnd_index=np.array([slot[bc] for bc, _ in sels], dtype=np.int32),
                bc_names=[names.get(bc, "default") for bc in bcs])
