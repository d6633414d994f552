"""ngsolve_gb300 -- GB300-native engine for NGSolve's high-order H1 operator path.

The numerical work runs in libgh1.so (CUDA, sm_103a; C ABI in include/gh1.h).
This package mirrors the reference's Python objects on that path.
"""
from . import _lib
from .meshes import MakeStructured3DMesh, MakeHexMesh, JitterInterior, ReadVolMesh
from .comp import (Mesh, H1, VectorH1, InnerProduct, Norm, BilinearForm, LinearForm, GridFunction, CoefficientFunction, grad, dx,
                   BaseVector, BaseMatrix, SparseMatrix, BilinearFormApplication, BlockMatrix, JacobiPrecond,
                   Preconditioner,
                   Projector, Integrate_grad_dot, ShapeEval, context, TaskManager, SetNumThreads, SetHeapSize, ngsglobals, x, y, z, VOL, BND, Integrate)
from . import solvers
from .solvers import CGSolver
from .adjoint import AdjointProblem, AdjointJ

__all__ = ["MakeStructured3DMesh", "MakeHexMesh", "JitterInterior", "ReadVolMesh", "Mesh", "H1", "VectorH1",
           "InnerProduct", "Norm", "BilinearForm",
           "LinearForm", "GridFunction", "CoefficientFunction", "grad", "dx", "BaseVector", "BaseMatrix",
           "SparseMatrix", "BilinearFormApplication", "BlockMatrix", "JacobiPrecond", "Preconditioner", "Projector", "Integrate_grad_dot",
           "ShapeEval", "context", "solvers", "AdjointProblem", "AdjointJ", "TaskManager", "SetNumThreads",
           "SetHeapSize", "ngsglobals", "CGSolver", "x", "y", "z", "VOL", "BND", "Integrate"]
