"""cholespy_gb300: GB300-native (sm_103a) sparse Cholesky solves.

Drop-in for cholespy's Python API (``CholeskySolverF``, ``CholeskySolverD``,
``MatrixType``; reference src/cholespy/__init__.py and src/main.cpp). The
factorisation runs on the host; the level analysis and the triangular solves
run in hand-written CUDA kernels behind the C ABI of ``include/gbchol.h``.
"""
from .batch import BatchSolver
from .solver import CholeskySolverD, CholeskySolverF, MatrixType, RefineResult, SolverInfo

__version__ = "0.1.0"

__all__ = ["CholeskySolverF", "CholeskySolverD", "MatrixType", "RefineResult", "SolverInfo",
           "BatchSolver"]
