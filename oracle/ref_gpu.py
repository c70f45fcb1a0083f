"""ORACLE — test infrastructure only: ctypes wrapper of oracle/ref_gpu.cpp,
which runs the reference's own GPU kernels (compiled from source) with the
reference's host protocol on a given factor."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import ref_build

_lib = None


def available() -> bool:
    return ref_build.CUBIN.exists() and ref_build.LAUNCHER.exists()


def lib():
    global _lib
    if _lib is None:
        ref_build.build_if_present()
        L = C.CDLL(str(ref_build.LAUNCHER))
        P, I32, U64 = C.c_void_p, C.c_int32, C.c_uint64
        L.refgpu_create.restype = C.c_int
        L.refgpu_create.argtypes = [C.c_char_p, I32, P, P, P, P, I32, C.POINTER(P)]
        L.refgpu_levels.restype = C.c_int
        L.refgpu_levels.argtypes = [P, I32, I32, P, P, C.POINTER(I32)]
        L.refgpu_solve.restype = C.c_int
        L.refgpu_solve.argtypes = [P, I32, U64, U64, U64]
        L.refgpu_destroy.restype = None
        L.refgpu_destroy.argtypes = [P]
        L.refgpu_last_error.restype = C.c_char_p
        L.refgpu_sync.restype = C.c_int
        L.refgpu_sync.argtypes = [C.c_double]
        _lib = L
    return _lib


class RefGpuSolver:
    """The reference's GPU analysis + solve on the factor (perm, L in CSC)."""

    def __init__(self, perm, colptr, rowidx, vals, double: bool):
        L = lib()
        self._keep = [np.ascontiguousarray(perm, np.int32), np.ascontiguousarray(colptr, np.int32),
                      np.ascontiguousarray(rowidx, np.int32), np.ascontiguousarray(vals, np.float64)]
        self.n = len(self._keep[0])
        h = C.c_void_p()
        rc = L.refgpu_create(str(ref_build.CUBIN).encode(), self.n,
                             *[a.ctypes.data for a in self._keep], 1 if double else 0, C.byref(h))
        if rc != 0:
            raise RuntimeError(L.refgpu_last_error().decode())
        self._h = h

    def levels(self, lower=True, kernel=True):
        """(row_levels, order, max_lvl): the reference analysis kernel's output
        (kernel=True) or the sequential definition it computes (kernel=False)."""
        lev = np.zeros(self.n, np.int32)
        order = np.zeros(self.n, np.int32)
        mx = C.c_int32()
        lib().refgpu_levels(self._h, 1 if lower else 0, 0 if kernel else 1, lev.ctypes.data,
                            order.ctypes.data, C.byref(mx))
        return lev, order, mx.value

    def solve(self, b, x, stream=0):
        """b, x: torch CUDA tensors (n, nrhs) row-major; asynchronous."""
        nrhs = b.shape[1] if b.dim() == 2 else 1
        rc = lib().refgpu_solve(self._h, nrhs, b.data_ptr(), x.data_ptr(), stream)
        if rc != 0:
            raise RuntimeError(lib().refgpu_last_error().decode())

    def close(self):
        if getattr(self, "_h", None):
            lib().refgpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
