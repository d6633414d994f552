"""Derive the symmetric tetrahedron quadrature rules used by libgh1 and write
``tet_rules.inc``.

The rules have the point counts NGSolve uses for its tabulated tet rules
(fem/intrule.cpp:2596-2812): degree 1 -> 1 point, 2 -> 4, 3..5 -> 14, 6 -> 24.
Each rule is built from symmetry orbits in barycentric coordinates
  S4 (1/4,1/4,1/4,1/4)        1 point
  S31(a)  (a,a,a,1-3a)          4 points
  S22(a)  (a,a,1/2-a,1/2-a)     6 points
  S211(a,b) (a,a,b,1-2a-b)     12 points
and its orbit parameters and weights are found here by solving the moment
equations  sum_q w_q x^i y^j z^k = i! j! k! / (i+j+k+3)!  for all monomials of
total degree <= d with a multi-start least-squares solve (scipy).  Only rules
with positive weights and interior points are accepted.  Run once; the output
is committed.  Usage:  python gen_tet_rules.py
"""
import itertools
import math
import os

import numpy as np
from scipy.optimize import least_squares


def orbit_points(kind, params):
    if kind == "S4":
        bary = [(0.25, 0.25, 0.25, 0.25)]
    elif kind == "S31":
        a, = params
        base = (a, a, a, 1 - 3 * a)
        bary = sorted(set(itertools.permutations(base)))
    elif kind == "S22":
        a, = params
        base = (a, a, 0.5 - a, 0.5 - a)
        bary = sorted(set(itertools.permutations(base)))
    elif kind == "S211":
        a, b = params
        base = (a, a, b, 1 - 2 * a - b)
        bary = sorted(set(itertools.permutations(base)))
    return np.array(bary)


ORBIT_SIZE = {"S4": 1, "S31": 4, "S22": 6, "S211": 12}
NPAR = {"S4": 0, "S31": 1, "S22": 1, "S211": 2}


def monomials(d):
    return [(i, j, k) for i in range(d + 1) for j in range(d + 1 - i) for k in range(d + 1 - i - j)]


def exact(i, j, k):
    return math.factorial(i) * math.factorial(j) * math.factorial(k) / math.factorial(i + j + k + 3)


def unpack(structure, v):
    pos = 0
    pts, wts = [], []
    for kind in structure:
        par = v[pos:pos + NPAR[kind]]
        pos += NPAR[kind]
        P = orbit_points(kind, par)
        pts.append(P)
        wts.append(np.full(len(P), np.nan))
    for o in range(len(structure)):
        wts[o][:] = v[pos]
        pos += 1
    return np.concatenate(pts), np.concatenate(wts)


def residual(v, structure, mons, ex):
    P, W = unpack(structure, v)
    x, y, z = P[:, 0], P[:, 1], P[:, 2]
    return np.array([np.sum(W * x ** i * y ** j * z ** k) for (i, j, k) in mons]) - ex


def solve(structure, degree, seed=0, tries=4000):
    mons = monomials(degree)
    ex = np.array([exact(*m) for m in mons])
    rng = np.random.default_rng(seed)
    npar = sum(NPAR[k] for k in structure)
    for _ in range(tries):
        v0 = np.concatenate([rng.uniform(0.01, 0.33, npar), rng.uniform(0.001, 0.03, len(structure))])
        r = least_squares(residual, v0, args=(structure, mons, ex), xtol=1e-15, ftol=1e-15, gtol=1e-15)
        if np.max(np.abs(r.fun)) > 1e-14:
            continue
        P, W = unpack(structure, r.x)
        if np.all(W > 0) and np.all(P > 1e-6) and len(np.unique(np.round(P, 12), axis=0)) == len(P):
            return P, W
    raise RuntimeError("no rule found for %s degree %d" % (structure, degree))


RULES = [
    (1, ["S4"]),
    (2, ["S31"]),
    (5, ["S31", "S31", "S22"]),
    (6, ["S31", "S31", "S31", "S211"]),
]


def main():
    out = ["// generated by gen_tet_rules.py -- symmetric tet rules on the reference tet",
           "// {(1,0,0),(0,1,0),(0,0,1),(0,0,0)}: x,y,z = barycentric lambda_0..2, weights sum to 1/6"]
    for degree, structure in RULES:
        P, W = solve(structure, degree)
        mons = monomials(degree)
        err = max(abs(np.sum(W * P[:, 0] ** i * P[:, 1] ** j * P[:, 2] ** k) - exact(i, j, k)) for i, j, k in mons)
        out.append("// degree %d, %d points, max moment error %.1e" % (degree, len(W), err))
        out.append("static const double TET_RULE_D%d[%d][4] = {" % (degree, len(W)))
        for p, w in zip(P, W):
            out.append("  {%.17g, %.17g, %.17g, %.17g}," % (p[0], p[1], p[2], w))
        out.append("};")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tet_rules.inc")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")
    print("wrote", path)


if __name__ == "__main__":
    main()
