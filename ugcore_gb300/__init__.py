"""ugcore_gb300 -- GB300-native (sm_103a) FV1 assembly + geometric-multigrid
Krylov solve for UG4/ugcore, behind a C ABI (include/ug4gb.h, libug4gb.so).

The Python layer mirrors ugcore's object model (algebra.py) and hosts the
adjoint autograd binding (adjoint.py).  Every numerical step runs in the
CUDA library; importing works without a GPU, but creating a Context needs one
and there is no CPU fallback.
"""
from ._lib import UG4GBError, exported_symbols, LIB_PATH  # noqa: F401
from .algebra import (AssembledOperator, BiCGStab, CG, Context, DomainDiscretization, GaussSeidel,  # noqa: F401
                      GeometricMultiGrid, GPUSparseMatrix, GPUVector, Jacobi, NewtonSolver, StandardLineSearch, StdConvCheck,
                      StructuredHierarchy, SymmetricGaussSeidel, ThetaTimeStep, UnstructuredHierarchy, ILU, StdTransfer, DofPermutation,
                      BackwardGaussSeidel, LU, BaseSmoothing)

__all__ = ["UG4GBError", "Context", "StructuredHierarchy", "GPUVector", "GPUSparseMatrix", "DomainDiscretization",
           "GeometricMultiGrid", "Jacobi", "GaussSeidel", "StdConvCheck", "CG", "BiCGStab", "ThetaTimeStep",
           "AssembledOperator", "NewtonSolver", "StandardLineSearch", "UnstructuredHierarchy", "SymmetricGaussSeidel", "BackwardGaussSeidel", "LU", "BaseSmoothing", "ILU", "StdTransfer", "DofPermutation",
           "exported_symbols"]
