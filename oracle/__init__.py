"""ORACLE — test infrastructure only (the checker, never the product).

ctypes wrapper around ``oracle/oracle.c``, the CPU restatement of the
reference's solve path (see the header of oracle.c for the file:line of the
reference each function follows). Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline legs of ``bench.py`` import this package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "oracle.c"
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
_lib = None


def build(force: bool = False) -> Path:
    """Compile oracle.c with gcc (no fused contractions beyond explicit fma)."""
    BUILD.mkdir(exist_ok=True)
    stamp = BUILD / "liboracle.stamp"
    key = f"{SRC.stat().st_mtime_ns}:{SRC.stat().st_size}:{os.uname().machine}"
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == key:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run(["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
                    str(SRC), "-o", str(tmp), "-lm"], check=True)
    os.replace(tmp, LIB)
    stamp.write_text(key)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P, I32, I64 = C.c_void_p, C.c_int32, C.c_int64
        L.oracle_build_csc.restype = I64
        L.oracle_build_csc.argtypes = [I32, I64, P, P, P, I32, P, P, P]
        L.oracle_levels.restype = None
        L.oracle_levels.argtypes = [I32, P, P, I32, P, P, P]
        for suf in ("f32", "f64"):
            getattr(L, f"oracle_lower_{suf}").restype = None
            getattr(L, f"oracle_lower_{suf}").argtypes = [I32, I32, P, P, P, P, P, P, P]
            getattr(L, f"oracle_upper_{suf}").restype = None
            getattr(L, f"oracle_upper_{suf}").argtypes = [I32, I32, P, P, P, P, P, P, P]
        L.oracle_chol_symbolic.restype = I64
        L.oracle_chol_symbolic.argtypes = [I32, P, P, P, P, P]
        L.oracle_chol_numeric.restype = I32
        L.oracle_chol_numeric.argtypes = [I32, P, P, P, P, P, P, P]
        L.oracle_cpu_solve.restype = None
        L.oracle_cpu_solve.argtypes = [I32, I32, P, P, P, P, P, P, I32]
        _lib = L
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def build_csc(n, ii, jj, x, fmt):
    """(colptr, rowidx, vals): sorted, duplicates summed (cholesky_solver.cpp:8-149)."""
    ii, jj, x = _c(ii, np.int32), _c(jj, np.int32), _c(x, np.float64)
    nnz = len(x)
    colptr = np.zeros(n + 1, np.int32)
    rowidx = np.zeros(max(nnz, 1), np.int32)
    vals = np.zeros(max(nnz, 1), np.float64)
    w = lib().oracle_build_csc(n, nnz, _p(ii), _p(jj), _p(x), int(fmt), _p(colptr), _p(rowidx), _p(vals))
    if w < 0:
        raise ValueError("index out of range")
    return colptr, rowidx[:w].copy(), vals[:w].copy()


def levels(rowptr, cols, lower):
    """(row_levels, order, max_lvl) as analysis_lower/upper + the counting sort."""
    rowptr, cols = _c(rowptr, np.int32), _c(cols, np.int32)
    n = len(rowptr) - 1
    lev = np.zeros(max(n, 1), np.int32)
    order = np.zeros(max(n, 1), np.int32)
    mx = C.c_int32(0)
    lib().oracle_levels(n, _p(rowptr), _p(cols), 1 if lower else 0, _p(lev), _p(order), C.byref(mx))
    return lev[:n], order[:n], int(mx.value)


def csr_of_lower(colptr, rowidx, vals):
    """CSR of L (columns ascending, diagonal last) from the CSC of L."""
    import scipy.sparse as sp
    n = len(colptr) - 1
    m = sp.csc_matrix((vals, rowidx, colptr), shape=(n, n)).tocsr()
    m.sort_indices()
    return m.indptr.astype(np.int32), m.indices.astype(np.int32), m.data


def solve_lower(rowptr, cols, vals, order, perm, b):
    """The reference's lower sweep on the CPU; b is (n, nrhs) row-major."""
    b = np.ascontiguousarray(b)
    dt = b.dtype
    suf = "f32" if dt == np.float32 else "f64"
    n, nrhs = b.shape
    tmp = np.zeros_like(b)
    v = _c(vals, dt)
    getattr(lib(), f"oracle_lower_{suf}")(n, nrhs, _p(_c(rowptr, np.int32)), _p(_c(cols, np.int32)),
                                          _p(v), _p(_c(order, np.int32)), _p(_c(perm, np.int32)),
                                          _p(b), _p(tmp))
    return tmp


def solve_upper(rowptr, cols, vals, order, perm, tmp):
    """The reference's upper sweep on the CPU; returns (tmp, out)."""
    tmp = np.ascontiguousarray(tmp).copy()
    dt = tmp.dtype
    suf = "f32" if dt == np.float32 else "f64"
    n, nrhs = tmp.shape
    out = np.zeros_like(tmp)
    v = _c(vals, dt)
    getattr(lib(), f"oracle_upper_{suf}")(n, nrhs, _p(_c(rowptr, np.int32)), _p(_c(cols, np.int32)),
                                          _p(v), _p(_c(order, np.int32)), _p(_c(perm, np.int32)),
                                          _p(tmp), _p(out))
    return tmp, out


def reference_solve(perm, colptr, rowidx, lvals, b, dtype):
    """The reference's full GPU solve (analysis + lower + upper sweeps),
    executed on the CPU in `dtype` on the given factor (L in CSC)."""
    lrp, lci, lv = csr_of_lower(colptr, rowidx, lvals)
    lev_l, ord_l, _ = levels(lrp, lci, True)
    lev_u, ord_u, _ = levels(colptr, rowidx, False)
    b2 = np.ascontiguousarray(b, dtype=dtype).reshape(len(perm), -1)
    tmp = solve_lower(lrp, lci, lv.astype(dtype), ord_l, perm, b2)
    _, out = solve_upper(colptr, rowidx, np.asarray(lvals).astype(dtype), ord_u, perm, tmp)
    return out.reshape(np.shape(b))


def cholesky(n, colptr, rowidx, vals, perm):
    """Up-looking simplicial LL^T of P A P^T (A's lower triangle used).
    Returns (Lp, Li, Lx) or raises ValueError if not positive definite."""
    Ap, Ai, Ax = _c(colptr, np.int32), _c(rowidx, np.int32), _c(vals, np.float64)
    perm = _c(perm, np.int32)
    Lp = np.zeros(n + 1, np.int32)
    nz = lib().oracle_chol_symbolic(n, _p(Ap), _p(Ai), _p(Ax), _p(perm), _p(Lp))
    Li = np.zeros(max(nz, 1), np.int32)
    Lx = np.zeros(max(nz, 1), np.float64)
    rc = lib().oracle_chol_numeric(n, _p(Ap), _p(Ai), _p(Ax), _p(perm), _p(Lp), _p(Li), _p(Lx))
    if rc != 0:
        raise ValueError("Matrix is not positive definite!")
    return Lp, Li[:nz], Lx[:nz]


def cpu_solve(perm, Lp, Li, Lx, b, threads=1):
    """x = P^T L^-T L^-1 P b in FP64 (cholmod_solve(CHOLMOD_A) semantics)."""
    b = np.ascontiguousarray(b, dtype=np.float64)
    shape = b.shape
    b2 = b.reshape(shape[0], -1)
    x = np.zeros_like(b2)
    lib().oracle_cpu_solve(len(perm), b2.shape[1], _p(_c(perm, np.int32)), _p(_c(Lp, np.int32)),
                           _p(_c(Li, np.int32)), _p(_c(Lx, np.float64)), _p(b2), _p(x), int(threads))
    return x.reshape(shape)
