"""Derive the symmetric tetrahedron quadrature rules used by libgh1 and write
``tet_rules.inc``.

The rules have the point counts NGSolve uses for its tabulated tet rules
(fem/intrule.cpp:2596-2812): degree 1 -> 1 point, 2 -> 4, 3..5 -> 14, 6 -> 24;
above degree 6 the reference falls back to collapsed (Duffy) tensor rules, and
so does libgh1 except at degree 7..8, where a 46-point symmetric rule found here
replaces the 216-point tensor rule (the p = 4 mass / load / B^T D B rule and the
p = 5 stiffness rule).
Each rule is built from symmetry orbits in barycentric coordinates
  S4 (1/4,1/4,1/4,1/4)        1 point
  S31(a)  (a,a,a,1-3a)          4 points
  S22(a)  (a,a,1/2-a,1/2-a)     6 points
  S211(a,b) (a,a,b,1-2a-b)     12 points
and its orbit parameters and weights are found here by solving the moment
equations  sum_q w_q x^i y^j z^k = i! j! k! / (i+j+k+3)!  for all monomials of
total degree <= d with a multi-start least-squares solve (scipy); only rules
with positive weights and interior points are accepted.  The double solution is
then refined by Gauss-Newton in 40-digit arithmetic (mpmath), so every moment
of the rounded rule is exact to double rounding relative to its own size.  Run
once; the output is committed.  Usage:  python gen_tet_rules.py
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


def residual_rel(v, structure, M, ex):
    """Moment residuals relative to the exact moments, all monomials at once."""
    P, W = unpack(structure, v)
    V = P[:, None, 0] ** M[None, :, 0] * P[:, None, 1] ** M[None, :, 1] * P[:, None, 2] ** M[None, :, 2]
    return (W @ V - ex) / ex


def solve(structure, degree, seed=0, tries=4000, relative=False):
    """Multi-start least squares.  relative=False: absolute moment residuals and
    the start ranges the rules up to degree 6 were found with; relative=True (the
    larger rules): relative residuals, weights started around the mean weight
    1/(6 npts), at most 200 evaluations per start."""
    mons = monomials(degree)
    ex = np.array([exact(*m) for m in mons])
    rng = np.random.default_rng(seed)
    npar = sum(NPAR[k] for k in structure)
    npts = sum(ORBIT_SIZE[k] for k in structure)
    for t in range(tries):
        if relative:
            v0 = np.concatenate([rng.uniform(0.02, 0.32, npar), rng.uniform(0.2, 3.0, len(structure)) / (6 * npts)])
            r = least_squares(residual_rel, v0, args=(structure, np.array(mons), ex), xtol=1e-15, ftol=1e-15,
                              gtol=1e-15, max_nfev=200)
            if np.max(np.abs(r.fun)) > 1e-11:
                continue
        else:
            v0 = np.concatenate([rng.uniform(0.01, 0.33, npar), rng.uniform(0.001, 0.03, len(structure))])
            r = least_squares(residual, v0, args=(structure, mons, ex), xtol=1e-15, ftol=1e-15, gtol=1e-15)
            if np.max(np.abs(r.fun)) > 1e-14:
                continue
        P, W = unpack(structure, r.x)
        if np.all(W > 0) and np.all(P > 1e-6) and len(np.unique(np.round(P, 12), axis=0)) == len(P):
            print("degree %d: %d points after %d starts" % (degree, len(W), t + 1), flush=True)
            return P, W
    raise RuntimeError("no rule found for %s degree %d" % (structure, degree))


def refine_mp(structure, degree, v0, dps=40, iters=8, fixed=None):
    """Gauss-Newton on the moment equations in mpmath (dps digits) from the
    double-precision solution: the rounded rule then has moments exact to
    double rounding relative to each moment (not only in absolute terms).
    fixed: index of an unknown held at its start value (structures with one
    unknown more than independent moment conditions form a one-parameter
    family; fixing one unknown picks the member the double solve found)."""
    import mpmath as mp
    mp.mp.dps = dps
    mons = monomials(degree)
    exact_mp = [mp.factorial(i) * mp.factorial(j) * mp.factorial(k) / mp.factorial(i + j + k + 3) for i, j, k in mons]

    def orbit_mp(kind, par):
        if kind == "S4":
            base = (mp.mpf(1) / 4,) * 4
        elif kind == "S31":
            a = par[0]
            base = (a, a, a, 1 - 3 * a)
        elif kind == "S22":
            a = par[0]
            base = (a, a, mp.mpf(1) / 2 - a, mp.mpf(1) / 2 - a)
        else:
            a, b = par
            base = (a, a, b, 1 - 2 * a - b)
        perms = sorted(set(itertools.permutations(range(4))))
        pts = {}
        for pm in perms:
            key = tuple(round(float(base[q]), 9) for q in pm)
            if key not in pts:
                pts[key] = tuple(base[q] for q in pm)
        return [pts[k] for k in sorted(pts)]

    def resid(v):
        pos = 0
        P, W = [], []
        pars = []
        for kind in structure:
            pars.append(v[pos:pos + NPAR[kind]])
            pos += NPAR[kind]
        for o, kind in enumerate(structure):
            pts = orbit_mp(kind, pars[o])
            P += pts
            W += [v[pos + o]] * len(pts)
        return [sum(w * p[0] ** i * p[1] ** j * p[2] ** k for p, w in zip(P, W)) - ex
                for (i, j, k), ex in zip(mons, exact_mp)], P, W

    v = [mp.mpf(float(t)) for t in v0]
    for _ in range(iters):
        r, _, _ = resid(v)
        h = mp.mpf(10) ** (-dps // 2)
        free = [c for c in range(len(v)) if c != fixed]
        J = mp.matrix(len(r), len(free))
        for cc, c in enumerate(free):
            vp = list(v)
            vp[c] += h
            rp, _, _ = resid(vp)
            for rr in range(len(r)):
                J[rr, cc] = (rp[rr] - r[rr]) / h
        JT = J.T
        delta = mp.lu_solve(JT * J, -(JT * mp.matrix(r)))
        for cc, c in enumerate(free):
            v[c] = v[c] + delta[cc]
    r, P, W = resid(v)
    return np.array([[float(c) for c in p[:3]] for p in P]), np.array([float(w) for w in W]), max(abs(x) for x in r)


def solve_refined(structure, degree, seed=0, relative=False):
    P, W = solve(structure, degree, seed=seed, relative=relative)
    # recover the orbit parameters from the double solution (one point per orbit)
    v0 = []
    idx = 0
    for kind in structure:
        n = ORBIT_SIZE[kind]
        block = P[idx:idx + n]
        # barycentric coordinates of the orbit's points (unpack returns all four)
        bary = block if block.shape[1] == 4 else np.column_stack([block, 1 - block.sum(1)])
        if kind == "S31":
            vals, cnt = np.unique(np.round(bary[0], 12), return_counts=True)
            v0.append(vals[np.argmax(cnt)])
        elif kind == "S22":
            v0.append(min(bary[0]))
        elif kind == "S211":
            vals, cnt = np.unique(np.round(bary[0], 12), return_counts=True)
            a = vals[np.argmax(cnt)]
            others = [x for x in bary[0] if abs(x - a) > 1e-9]
            v0 += [a, others[0]]
        idx += n
    idx = 0
    for kind in structure:
        v0.append(W[idx])
        idx += ORBIT_SIZE[kind]
    # one unknown more than the invariant moment conditions (a one-parameter
    # family): hold the unknown whose removal keeps the Jacobian best conditioned
    fixed = None
    mons = monomials(degree)
    M = np.array(mons)
    ex = np.array([exact(*m) for m in mons])
    v0a = np.array(v0, dtype=float)
    h = 1e-7
    J = np.column_stack([(residual_rel(v0a + h * np.eye(len(v0a))[c], structure, M, ex) -
                          residual_rel(v0a - h * np.eye(len(v0a))[c], structure, M, ex)) / (2 * h)
                         for c in range(len(v0a))])
    if np.linalg.matrix_rank(J, tol=1e-8 * np.linalg.norm(J, 2)) < len(v0a):
        conds = [np.linalg.cond(np.delete(J, c, axis=1)) for c in range(len(v0a))]
        fixed = int(np.argmin(conds))
    Pm, Wm, res = refine_mp(structure, degree, v0, fixed=fixed)
    return Pm, Wm, res


# (degree, orbit structure, start seed, relative residuals)
RULES = [
    (1, ["S4"], 0, False),
    (2, ["S31"], 0, False),
    (5, ["S31", "S31", "S22"], 0, False),
    (6, ["S31", "S31", "S31", "S211"], 0, False),
    (8, ["S31", "S31", "S31", "S31", "S22", "S211", "S211"], 1, True),
]


def main():
    out = ["// generated by gen_tet_rules.py -- symmetric tet rules on the reference tet",
           "// {(1,0,0),(0,1,0),(0,0,1),(0,0,0)}: x,y,z = barycentric lambda_0..2, weights sum to 1/6"]
    for degree, structure, seed, relative in RULES:
        P, W, res_mp = solve_refined(structure, degree, seed=seed, relative=relative)
        mons = monomials(degree)
        err = max(abs(np.sum(W * P[:, 0] ** i * P[:, 1] ** j * P[:, 2] ** k) - exact(i, j, k)) / exact(i, j, k)
                  for i, j, k in mons)
        out.append("// degree %d, %d points, max relative moment error in double %.1e (40-digit residual %.1e)"
                   % (degree, len(W), err, float(res_mp)))
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
