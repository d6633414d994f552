"""Mesh generators and readers for the H1 path.

``MakeStructured3DMesh`` mirrors ``ngsolve.meshes.MakeStructured3DMesh``
(python/meshes.py:273-410 of NGSolve): points are numbered with x outermost and
z innermost, hexes list their vertices as
``[base, base+1, base+(nz+1)+1, base+(nz+1), baseup, ...]`` and the tet variant
splits every cube into the six tets of the reference's Kuhn split.  Keeping the
vertex lists identical keeps the element orientation classes identical, which
fixes the orientation of every edge and face shape function.

``ReadVolMesh`` reads the ASCII netgen ``.vol`` / ``.vol.gz`` format (the
``volumeelements`` and ``points`` sections) used by the reference test meshes.
"""
import gzip

import numpy as np


class Mesh:
    """Volume mesh of one element type: ``points`` (nv,3) float64 and
    ``elements`` (ne, 4 | 8) int32 vertex lists in the reference's local order."""

    def __init__(self, points, elements):
        self.points = np.ascontiguousarray(points, dtype=np.float64)
        self.elements = np.ascontiguousarray(elements, dtype=np.int32)
        if self.elements.ndim != 2 or self.elements.shape[1] not in (4, 8):
            raise ValueError("elements must be (ne,4) tets or (ne,8) hexes")
        if self.points.ndim != 2 or self.points.shape[1] != 3:
            raise ValueError("points must be (nv,3)")
        if len(self.elements) and (self.elements.min() < 0 or self.elements.max() >= len(self.points)):
            raise ValueError("element vertex index out of range")

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
    return Mesh(pts, els.astype(np.int32))


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
    return Mesh(pts, mesh.elements)


def ReadVolMesh(path):
    """Volume elements and points of an ASCII netgen mesh file."""
    opener = gzip.open if str(path).endswith(".gz") else open
    with opener(path, "rt") as fh:
        lines = fh.read().split("\n")
    pts, els = None, None
    n = len(lines)
    i = 0
    while i < n:
        tok = lines[i].strip()
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
    return Mesh(np.array(pts), np.array(els, dtype=np.int32))
