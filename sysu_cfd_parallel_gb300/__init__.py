"""GB300-native SIMPLE solve of Cycas2Parallel (Meiyim/SYSU_CFD_Parallel).

The hot path -- gradients, boundary conditions, momentum / pressure-correction / k-epsilon
assembly, Rhie-Chow fluxes and the GMRES solves the reference hands to PETSc -- is
hand-written sm_103a CUDA in ``libcycasgpu.so`` behind the C ABI of ``include/cycasgpu.h``.
This package holds the build recipe, the ctypes binding and a thin host mirror of the
reference's ``NavierStokesSolver``.
"""
from . import build, capi, meshgen  # noqa: F401
from .solver import Case, ConvergeError, NavierStokesSolver, csr_solve  # noqa: F401

__all__ = ["build", "capi", "meshgen", "Case", "ConvergeError", "NavierStokesSolver", "csr_solve"]
