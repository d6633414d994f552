"""solvers.CG / CGSolver on the GPU (python/krylovspace.py:222-337 of NGSolve).

The whole iteration runs on the device (libgh1 gh1_cg): the same algorithm and
stopping rule as CGSolver._SolveImpl, with `mode="mixed"` adding FP32 inner
solves inside FP64 iterative refinement.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .comp import BaseVector, _as_vec, _ptr


class CGSolver:
    """CGSolver(mat, pre, tol, maxiter, ...) -- .Solve(rhs, sol), .iterations,
    .residuals (residual history of the stop rule)."""
    name = "CG"

    def __init__(self, mat, pre=None, freedofs=None, tol=None, maxiter=100, atol=None, callback=None,
                 printrates=False, mode="fp64", stop_rule="precond", inner_tol=0.0, max_outer=0,
                 check_every=0, conjugate=False, maxsteps=None, plotrates=False, callback_sol=None,
                 abstol=None, printing=False):
        # the keywords of the reference's CGSolver / LinearSolver
        # (python/krylovspace.py:60-75, 240-255); a misspelt or unknown keyword
        # is a TypeError, as with any Python signature
        if atol is not None or abstol is not None:
            raise NotImplementedError("atol: the GPU solver supports the relative tolerance only")
        if callback_sol is not None:
            raise NotImplementedError("callback_sol: the iterates stay on the device inside one solve")
        if mode not in ("fp64", "mixed"):
            raise ValueError("mode is 'fp64' or 'mixed'")
        if stop_rule not in ("precond", "true"):
            raise ValueError("stop_rule is 'precond' or 'true'")
        printrates = printrates or printing
        if pre is None and freedofs is not None:
            pre = mat.CreateSmoother(freedofs)
        if maxsteps is not None:
            maxiter = maxsteps
        self.mat, self.pre = mat, pre
        self.tol = 1e-12 if tol is None else float(tol)
        self.maxiter = int(maxiter)
        self.callback = callback
        self.printrates = printrates
        self.mode = mode
        self.stop_rule = stop_rule
        self.inner_tol = inner_tol
        self.max_outer = max_outer
        self.check_every = check_every
        self.residuals = []
        self.iterations = 0
        self.result = None

    @property
    def errors(self):
        return self.residuals

    def Solve(self, rhs, sol=None, initialize=True):
        rhs = _as_vec(rhs)
        if sol is None:
            sol = rhs.CreateVector()
            initialize = True
        sol = _as_vec(sol)
        if rhs.t.dtype != torch.float64 or sol.t.dtype != torch.float64:
            raise TypeError("CG works on FP64 vectors (mixed mode keeps FP32 internally)")
        ctx = self.mat.ctx.sync_stream()
        hist = np.zeros(self.maxiter + 2)
        o = _lib.CGOpts()
        o.tol = self.tol
        o.maxit = self.maxiter
        o.mode = _lib.GH1_CG_MIXED if self.mode == "mixed" else _lib.GH1_CG_FP64
        o.stop_rule = _lib.GH1_STOP_TRUE if self.stop_rule == "true" else _lib.GH1_STOP_PRECOND
        o.initialize = 1 if initialize else 0
        o.inner_tol = float(self.inner_tol)
        o.max_outer = int(self.max_outer)
        o.check_every = int(self.check_every)
        o.res_hist = hist.ctypes.data
        r = _lib.CGResult()
        rc = ctx.lib.gh1_cg(self.mat.h, None if self.pre is None else self.pre.h, _ptr(rhs.t), _ptr(sol.t),
                            ctypes.byref(o), ctypes.byref(r))
        if rc not in (_lib.GH1_OK, 6, 7):
            ctx.check(rc)
        self.result = r
        self.iterations = r.iterations
        n_hist = (r.outer + 1) if self.mode == "mixed" else r.iterations
        self.residuals = list(hist[:max(0, min(n_hist, len(hist)))])
        if self.printrates:
            print("%s %sconverged in %d iterations to residual %g (true relative residual %g)" %
                  (self.name, "" if r.status == 0 else "NOT ", r.iterations, r.final_res, r.true_relres))
        if self.callback is not None:
            for k, v in enumerate(self.residuals[1:], start=2):
                self.callback(k, v)
        self.sol = sol
        return sol

    def Mult(self, x, y):
        self.Solve(rhs=x, sol=y, initialize=True)

    # the solver as an operator: inv * f runs one solve (KrylovSpaceSolver)
    @property
    def height(self):
        return self.mat.height

    @property
    def width(self):
        return self.mat.width

    def MultScale(self, s, x, y):
        self.Mult(x, y)
        if s != 1.0:
            _as_vec(y).t.mul_(s)

    def MultAdd(self, s, x, y):
        y = _as_vec(y)
        tmp = y.CreateVector()
        self.Mult(x, tmp)
        y.t.add_(tmp.t, alpha=s)

    def __mul__(self, x):
        from .comp import _MatVec
        return _MatVec(self, _as_vec(x))

    def GetSteps(self):
        return self.iterations

    def CreateVector(self, colvector=False):
        return self.mat.CreateVector()

    def CreateDeviceMatrix(self):
        return self

    def GetOperatorInfo(self):
        return "CGSolver (tol %g, maxiter %d) of: %s" % (self.tol, self.maxiter, self.mat.GetOperatorInfo())


def CG(mat, rhs, pre=None, sol=None, tol=1e-12, maxsteps=100, printrates=True, plotrates=False, initialize=True,
       conjugate=False, callback=None, **kwargs):
    """preconditioned conjugate gradient method (signature of ngsolve.solvers.CG,
    python/krylovspace.py:293-338).  Further keywords go to CGSolver, which
    raises TypeError on a keyword it does not know."""
    solver = CGSolver(mat=mat, pre=pre, tol=tol, maxiter=maxsteps, callback=callback, printrates=printrates,
                      plotrates=plotrates, conjugate=conjugate, **kwargs)
    solver.Solve(rhs=rhs, sol=sol, initialize=initialize)
    CG.last_solver = solver
    return solver.sol


class BatchCG:
    """Batched mixed-precision CG over many independent hex problems.

    forms: list of BilinearForm (hex meshes, kappa/mu per element); nrhs: right-hand
    sides per problem.  Solve(rhs_list, tol) takes per problem a (nrhs, ndof)
    FP64 CUDA tensor and returns the solutions in the same layout; `results` holds
    one CGResult per (problem, rhs).

    A form on VectorH1 (dim components) is solved as its scalar form with
    nrhs * dim right-hand sides: the (nrhs, dim * n) tensor is, in memory, the
    (nrhs * dim, n) one.  Each component then stops on its own relative residual
    (result index rhs * dim + component); at most 16 scalar right-hand sides per
    problem."""

    def __init__(self, forms, nrhs):
        if len(forms) != len(nrhs):
            raise ValueError("one rhs count per form")
        self.forms = list(forms)
        self.nrhs = [int(r) for r in nrhs]
        self._ncomp = [getattr(f.fes, "dim", 1) if f._sfes is not f.fes else 1 for f in self.forms]
        ctx = self.forms[0].fes.ctx.sync_stream()
        self.ctx = ctx
        handles = (ctypes.c_void_p * len(forms))(*[f._make_form().value for f in self.forms])
        counts = (ctypes.c_int * len(forms))(*[r * c for r, c in zip(self.nrhs, self._ncomp)])
        h = ctypes.c_void_p()
        ctx.check(ctx.lib.gh1_batch_create(ctx.h, len(forms), handles, counts, ctypes.byref(h)))
        self.h = h
        self.results = []

    def Solve(self, rhs, tol=1e-10, maxit=5000, inner_tol=0.0, max_outer=0, check_every=0, sol=None):
        ctx = self.ctx.sync_stream()
        if len(rhs) != len(self.forms):
            raise ValueError("one rhs tensor per problem")
        xs = sol if sol is not None else [torch.zeros_like(b) for b in rhs]
        for b, x, f, r in zip(rhs, xs, self.forms, self.nrhs):
            if b.shape != (r, f.fes.ndof) or b.dtype != torch.float64 or not b.is_cuda or not b.is_contiguous():
                raise ValueError("rhs of a problem must be a contiguous (nrhs, ndof) float64 CUDA tensor")
        bp = (ctypes.c_void_p * len(rhs))(*[b.data_ptr() for b in rhs])
        xp = (ctypes.c_void_p * len(xs))(*[x.data_ptr() for x in xs])
        o = _lib.CGOpts()
        o.tol, o.maxit, o.mode, o.stop_rule, o.initialize = float(tol), int(maxit), _lib.GH1_CG_MIXED, _lib.GH1_STOP_TRUE, 1
        o.inner_tol, o.max_outer, o.check_every = float(inner_tol), int(max_outer), int(check_every)
        res = (_lib.CGResult * sum(r * c for r, c in zip(self.nrhs, self._ncomp)))()
        rc = ctx.lib.gh1_batch_solve(self.h, bp, xp, ctypes.byref(o), res)
        if rc not in (_lib.GH1_OK, 6, 7):
            ctx.check(rc)
        self.status = rc
        self.results = list(res)
        return xs

    def __del__(self):
        try:
            self.ctx.lib.gh1_batch_free(self.h)
        except Exception:
            pass
