"""Differentiable solves: a ``torch.autograd.Function`` around the GB300 solve.

    ds = DifferentiableSolver(n, ii, jj, values, MatrixType.COO)   # values: requires_grad
    x = ds(b)                 # x = A^{-1} b, differentiable w.r.t. b and values
    loss.backward()           # backward solve on the same factor + sparse gradient kernel

Backward: grad_b = A^{-1} grad_x reuses the factor (A is symmetric), and a
hand-written kernel forms the gradient on A's stored entries from grad_b and
x (gbchol_grad_values). ``symmetric=True`` (default) gives the gradient for
A treated as a symmetric matrix: -1/2 (gb_i x_j + gb_j x_i) on each stored
off-diagonal entry, -gb_i x_i on the diagonal, i.e. the derivative of the
solve of sym(A) = (A + A^T)/2, which equals A for symmetric input.
``symmetric=False`` gives the exact derivative of the reference's forward,
which reads only the lower triangle (entries above the diagonal get 0).
The factor is fixed at construction: after changing ``values`` build a new
solver, as with the reference. No counterpart in the reference.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _ffi
from .solver import CholeskySolverD, CholeskySolverF, MatrixType, _host_vector


def _coo_indices(n, ii, jj, type):
    """(rows, cols) of every stored entry, in the order of the values array."""
    ii = _host_vector(ii, np.int32, "ii")
    jj = _host_vector(jj, np.int32, "jj")
    if type == MatrixType.COO:
        return ii, jj
    counts = np.diff(ii.astype(np.int64))
    owner = np.repeat(np.arange(n, dtype=np.int32), counts)
    if type == MatrixType.CSR:
        return owner, jj
    return jj, owner  # CSC: jj holds rows, owner the column


def _make_function():
    import torch

    class CholeskySolveFunction(torch.autograd.Function):
        @staticmethod
        def forward(ctx, values, b, owner):
            x = torch.empty_like(b)
            owner.solver.solve(b, x)
            ctx.owner = owner
            ctx.save_for_backward(x)
            return x

        @staticmethod
        def backward(ctx, grad_x):
            owner = ctx.owner
            (x,) = ctx.saved_tensors
            grad_x = grad_x.contiguous()
            gb = torch.empty_like(grad_x)
            owner.solver.solve(grad_x, gb)
            grad_vals = None
            if ctx.needs_input_grad[0]:
                grad_vals = torch.empty(owner.nnz, dtype=owner.values_dtype, device=x.device)
                nrhs = x.shape[1] if x.dim() == 2 else 1
                prec = 0 if x.dtype == torch.float32 else 1
                out_prec = 0 if owner.values_dtype == torch.float32 else 1
                stream = torch.cuda.current_stream(x.device).cuda_stream
                _ffi.check(_ffi.lib().gbchol_grad_values(
                    prec, owner.nnz, nrhs, C.c_void_p(owner.rows.data_ptr()),
                    C.c_void_p(owner.cols.data_ptr()), C.c_void_p(gb.data_ptr()),
                    C.c_void_p(x.data_ptr()), C.c_void_p(grad_vals.data_ptr()), out_prec,
                    1 if owner.symmetric else 0, C.c_void_p(stream)))
            return grad_vals, gb, None

    return CholeskySolveFunction


_FN = None


class DifferentiableSolver:
    """x = A^{-1} b with gradients for b and for A's stored values.

    ``values`` is a CUDA tensor (float64 unless given otherwise) and may
    require grad; ``precision`` picks the solver ("float": CholeskySolverF,
    "double": CholeskySolverD)."""

    def __init__(self, n_rows, ii, jj, values, type, precision="float", symmetric=True):
        import torch
        global _FN
        if _FN is None:
            _FN = _make_function()
        type = MatrixType(int(type))
        if values.device.type != "cuda":
            raise ValueError("DifferentiableSolver runs on the GPU: pass CUDA tensors.")
        cls = CholeskySolverF if precision == "float" else CholeskySolverD
        self.solver = cls(n_rows, ii, jj, values.detach(), type)
        rows, cols = _coo_indices(n_rows, ii, jj, type)
        dev = values.device
        self.rows = torch.as_tensor(rows, device=dev)
        self.cols = torch.as_tensor(cols, device=dev)
        self.nnz = int(len(rows))
        self.values = values
        self.values_dtype = values.dtype
        self.symmetric = bool(symmetric)
        self.dtype = torch.float32 if precision == "float" else torch.float64

    def __call__(self, b):
        if b.dtype != self.dtype:
            raise TypeError(f"b must be {self.dtype}.")
        return _FN.apply(self.values, b.contiguous(), self)
