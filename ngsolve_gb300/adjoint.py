"""Adjoint gradient of J(kappa) = 1/2 int (u(kappa) - u_target)^2 dx for the
per-element diffusion coefficient kappa, with A(kappa) u = f, zero Dirichlet.

dJ/dkappa_e = - int_e grad u . grad lambda,   A lambda = M (u - u_target):
the recipe of the reference's optimisation tutorial
(docs/i-tutorials/unit-7-optimization/05_Topological_Derivative_Transmission.ipynb,
cells 6, 10, 14) with Integrate(..., element_wise=True) for the contraction
(comp/python_comp.cpp:3703-3948).  Both solves and the element contraction run
in libgh1 (gh1_adjoint_grad); `AdjointJ` exposes it as a torch.autograd.Function.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .comp import _np_ptr, _ptr


class AdjointProblem:
    """Holds the space, the assembled source f and the target u_target."""

    def __init__(self, fes, f_vec, u_target, tol=1e-12):
        self.fes = fes
        self.f = f_vec if isinstance(f_vec, torch.Tensor) else f_vec.t
        self.u_target = u_target if isinstance(u_target, torch.Tensor) else u_target.t
        self.tol = float(tol)
        ctx = fes.ctx
        h = ctypes.c_void_p()
        ones = np.ones(fes.ne)
        ctx.check(ctx.lib.gh1_form_create(fes.h, _np_ptr(ones), None, _lib.GH1_MEM_HOST, ctypes.byref(h)))
        self.form = h
        self.u = torch.zeros(fes.ndof, dtype=torch.float64, device=self.f.device)
        self.lam = torch.zeros_like(self.u)

    def evaluate(self, kappa):
        """J and dJ/dkappa (device tensor) for per-element kappa (array or tensor)."""
        ctx = self.fes.ctx.sync_stream()
        k = np.ascontiguousarray(torch.as_tensor(kappa).detach().cpu().numpy(), dtype=np.float64)
        if k.shape != (self.fes.ne,):
            raise ValueError("kappa needs one value per element")
        ctx.check(ctx.lib.gh1_form_set_coefs(self.form, _np_ptr(k), None, _lib.GH1_MEM_HOST))
        g = torch.zeros(self.fes.ne, dtype=torch.float64, device=self.f.device)
        J = ctypes.c_double()
        ctx.check(ctx.lib.gh1_adjoint_grad(self.form, _ptr(self.f), _ptr(self.u_target), self.tol, _ptr(self.u),
                                           _ptr(self.lam), _ptr(g), ctypes.byref(J)))
        return J.value, g

    def __del__(self):
        try:
            self.fes.ctx.lib.gh1_form_free(self.form)
        except Exception:
            pass


class AdjointJ(torch.autograd.Function):
    """J = AdjointJ.apply(kappa, problem); J.backward() fills kappa.grad."""

    @staticmethod
    def forward(ctx, kappa, problem):
        J, g = problem.evaluate(kappa)
        ctx.save_for_backward(g.to(kappa.device))
        return torch.tensor(J, dtype=torch.float64, device=kappa.device)

    @staticmethod
    def backward(ctx, gJ):
        (g,) = ctx.saved_tensors
        return gJ * g, None
