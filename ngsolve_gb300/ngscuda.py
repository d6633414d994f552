"""Stand-in for ``ngsolve.ngscuda``: scripts that import it keep working.

In NGSolve this module registers the CUDA device matrices and vectors behind
CreateDeviceMatrix / CreateDeviceVector.  Every operator and vector of this
package already lives on the GPU, so those calls return the operator itself
or a device copy, and there is nothing to register.
"""
__all__ = []
