"""The reference package's import name, for drop-in use.

``from cholespy import CholeskySolverF, CholeskySolverD, MatrixType`` (as in
rgl-epfl/cholespy, src/cholespy/__init__.py and src/main.cpp:118-124) gives
this build's solvers from ``cholespy_gb300`` unchanged: code written for the
reference runs without edits.
"""
from cholespy_gb300 import CholeskySolverD, CholeskySolverF, MatrixType, __version__

__all__ = ["CholeskySolverF", "CholeskySolverD", "MatrixType", "__version__"]
