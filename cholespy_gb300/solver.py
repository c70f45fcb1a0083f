"""Drop-in ``CholeskySolverF`` / ``CholeskySolverD`` / ``MatrixType``.

Mirrors the reference's nanobind module (src/main.cpp:16-136): the same
constructor ``(n_rows, ii, jj, x, type)`` and ``solve(b, x)``, the same
argument checks and error messages, and the same asynchronous in-place write
of ``x``. Arrays may be torch tensors, NumPy arrays or anything exporting
DLPack / ``__cuda_array_interface__`` (CuPy, JAX, ...). A solver built from
CUDA arrays solves on the GB300 through the gbchol C ABI and lives on the
CUDA device of those arrays (the reference always uses device 0,
src/cuda_driver.cpp:124). A solver built from CPU arrays solves CPU arrays
on the host cores (gbchol_factor_solve, the reference's solve_cpu path,
src/main.cpp:68-70, 83-91); the two never stand in for each other.

Extensions beyond the reference (keyword-only, off by default):
``CholeskySolverD(..., refine=True)`` keeps an FP32 factor plus the FP64
matrix and makes ``solve`` an FP32 solve with FP64-residual iterative
refinement to ``tol`` (default 1e-10); ``solve_refined`` returns its
statistics.
"""
from __future__ import annotations

import ctypes as C
import enum
import math
import os
from dataclasses import dataclass

import numpy as np

from . import _ffi


class MatrixType(enum.IntEnum):
    """Sparse input format (src/cholesky_solver.h:8-12, src/main.cpp:118-121)."""

    CSC = 0
    CSR = 1
    COO = 2


@dataclass
class SolverInfo:
    n: int
    device: int
    nnz_a: int
    nnz_l: int
    levels_lower: int
    levels_upper: int
    n_supernodes: int
    max_supernode: int
    factor_flops: float
    factor_seconds: float
    analysis_seconds: float
    top_rows: int = 0
    top_units: int = 0
    top_blocks: int = 0
    launches_per_solve: int = 0


@dataclass
class RefineResult:
    iterations: int
    converged: bool
    max_rel_residual: float


def _refine_result(iterations: int, converged: bool, max_rel: float, tol: float) -> RefineResult:
    """Stats of a refined solve as returned to the caller. A residual that is
    not finite, or above tol, is never reported as converged, whatever the
    device flag says."""
    ok = bool(converged) and math.isfinite(max_rel) and max_rel <= tol
    return RefineResult(int(iterations), ok, float(max_rel))


def _torch():
    import torch
    return torch


def _device_of(a):
    """('cuda', index) or ('cpu', 0) for a torch tensor / array-like."""
    try:
        torch = _torch()
        if isinstance(a, torch.Tensor):
            return (a.device.type, a.device.index or 0)
    except ImportError:  # pragma: no cover - torch is a hard dependency here
        pass
    if isinstance(a, np.ndarray):
        return ("cpu", 0)
    if hasattr(a, "__cuda_array_interface__"):
        return ("cuda", _cuda_index_of(a))
    if hasattr(a, "__dlpack_device__"):
        dev_type, dev_id = a.__dlpack_device__()
        if int(dev_type) in (2, 13):  # kDLCUDA, kDLCUDAManaged
            return ("cuda", int(dev_id))
        if int(dev_type) == 1:
            return ("cpu", 0)
        return ("other", int(dev_id))
    return ("cpu", 0)


def _cuda_index_of(a):
    torch = _torch()
    return torch.as_tensor(a, device="cuda").device.index or 0


def _as_torch(a):
    """Zero-copy torch view of an array-like (DLPack / CUDA array interface)."""
    torch = _torch()
    if isinstance(a, torch.Tensor):
        return a
    if isinstance(a, np.ndarray):
        return torch.from_numpy(a)
    if hasattr(a, "__dlpack__"):
        return torch.from_dlpack(a)
    if hasattr(a, "__cuda_array_interface__"):
        return torch.as_tensor(a, device="cuda")
    return torch.as_tensor(np.asarray(a))


def _check_shapes(n_rows, ii, jj, x, type):
    """Shape checks of src/main.cpp:28-43 (same messages); returns len(x)."""
    ni, nj, nx = _len(ii), _len(jj), _len(x)
    if type == MatrixType.COO:
        if ni != nj:
            raise ValueError("Sparse COO matrix: the two index arrays should have the same size.")
        if ni != nx:
            raise ValueError("Sparse COO matrix: the index and data arrays should have the same size.")
    elif type == MatrixType.CSR:
        if nj != nx:
            raise ValueError("Sparse CSR matrix: the column index and data arrays should have the same size.")
        if ni != n_rows + 1:
            raise ValueError("Sparse CSR matrix: Invalid size for row pointer array.")
    else:
        if nj != nx:
            raise ValueError("Sparse CSC matrix: the row index and data arrays should have the same size.")
        if ni != n_rows + 1:
            raise ValueError("Sparse CSC matrix: Invalid size for column pointer array.")
    return nx


def _host_vector(a, dtype, name):
    """1-D host copy of a constructor argument, as the reference's D2H copies
    (src/main.cpp:55-61)."""
    t = _as_torch(a)
    if t.dim() != 1:
        raise ValueError(f"{name} must be a 1-D array.")
    arr = t.detach().cpu().numpy()
    if dtype == np.int32:
        if not np.issubdtype(arr.dtype, np.integer):
            raise TypeError(f"{name} must be an integer array.")
        if arr.size and (arr.min() < np.iinfo(np.int32).min or arr.max() > np.iinfo(np.int32).max):
            raise ValueError(f"{name}: index does not fit in int32.")
    return np.ascontiguousarray(arr, dtype=dtype)


def _device_vector(a, dtype, device, name):
    """1-D contiguous CUDA tensor of `dtype` on `device` from a CUDA array (the
    reference's constructor takes int32 indices and float64 values)."""
    torch = _torch()
    t = _as_torch(a).detach()
    if t.dim() != 1:
        raise ValueError(f"{name} must be a 1-D array.")
    if dtype == torch.int32:
        if t.is_floating_point() or t.is_complex() or t.dtype == torch.bool:
            raise TypeError(f"{name} must be an integer array.")
        if t.numel() and t.dtype != torch.int32 and (int(t.min()) < -2**31 or int(t.max()) > 2**31 - 1):
            raise ValueError(f"{name}: index does not fit in int32.")
    return t.to(device=torch.device("cuda", device), dtype=dtype).contiguous()


def _ptr(arr: np.ndarray):
    return C.c_void_p(arr.ctypes.data) if arr.size else C.c_void_p(0)


class _CholeskySolver:
    _precision = 0
    _torch_dtype_name = "float32"

    def __init__(self, n_rows, ii, jj, x, type, *, refine=False, tol=1e-10, max_iter=10):
        lib = _ffi.lib()
        self._h = None
        self._fh = None
        self._cpu = False
        n_rows = int(n_rows)
        if n_rows < 0 or n_rows > np.iinfo(np.uint32).max:
            raise ValueError("n_rows out of range.")
        type = MatrixType(int(type))
        nx = _check_shapes(n_rows, ii, jj, x, type)
        devs = {_device_of(a)[0] for a in (ii, jj, x)}
        if len(devs) != 1:
            raise ValueError("All input tensors should be on the same device!")
        dev_type = devs.pop()
        if dev_type != "cuda" and dev_type != "cpu":
            raise ValueError("Unsupported input device! Only CPU and CUDA arrays are supported.")
        if dev_type == "cpu":
            self._init_cpu(n_rows, nx, ii, jj, x, type)
            return
        device = _device_of(x)[1]
        self._device = device
        self._refine = bool(refine) and self._precision == 1
        self._tol = float(tol)
        self._max_iter = int(max_iter)
        store = _ffi.STORE_F32 if self._precision == 0 else _ffi.STORE_F64
        if self._refine:
            store = _ffi.STORE_F32 | _ffi.STORE_F64 | _ffi.STORE_A64
        torch = _torch()
        h = C.c_void_p()
        if os.environ.get("GBCHOL_HOST_PREP") == "1":  # the host conversion (gbchol_create)
            hi = _host_vector(ii, np.int32, "ii")
            hj = _host_vector(jj, np.int32, "jj")
            hx = _host_vector(x, np.float64, "x")
            with torch.cuda.device(device):
                st = lib.gbchol_create(n_rows, int(nx), _ptr(hi), _ptr(hj), _ptr(hx), int(type),
                                       store, C.byref(h))
        else:
            # the input conversion on the GPU (gbchol_create_device)
            with torch.cuda.device(device):
                di = _device_vector(ii, torch.int32, device, "ii")
                dj = _device_vector(jj, torch.int32, device, "jj")
                dx = _device_vector(x, torch.float64, device, "x")
                torch.cuda.current_stream(device).synchronize()
                st = lib.gbchol_create_device(n_rows, int(nx), C.c_void_p(di.data_ptr() if di.numel() else 0),
                                              C.c_void_p(dj.data_ptr() if dj.numel() else 0),
                                              C.c_void_p(dx.data_ptr() if dx.numel() else 0), int(type), store,
                                              C.byref(h))
        _ffi.check(st)
        self._h = h
        self._n = n_rows

    def _init_cpu(self, n_rows, nx, ii, jj, x, type):
        # CPU arrays: factorise on the host and keep the factor there; solves
        # take CPU arrays only (src/main.cpp:68-70, cholesky_solver.cpp:435-463)
        self._cpu = True
        self._device = None
        self._refine = False
        self._tol = 1e-10
        self._max_iter = 10
        hi = _host_vector(ii, np.int32, "ii")
        hj = _host_vector(jj, np.int32, "jj")
        hx = _host_vector(x, np.float64, "x")
        fh = C.c_void_p()
        st = _ffi.lib().gbchol_factorize(n_rows, int(nx), _ptr(hi), _ptr(hj), _ptr(hx), int(type), 0,
                                         C.byref(fh))
        _ffi.check(st)
        self._fh = fh
        self._n = n_rows
        # build the host solve's structure now (a zero-RHS solve), so that the
        # first solve is not slower than the others
        _ffi.check(_ffi.lib().gbchol_factor_solve(fh, self._precision, 0, None, None, 0))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _ffi.lib().gbchol_destroy(h)
            except Exception:
                pass
            self._h = None
        fh = getattr(self, "_fh", None)
        if fh:
            try:
                _ffi.lib().gbchol_factor_free(fh)
            except Exception:
                pass
            self._fh = None

    @property
    def is_cpu(self):
        """True for a solver built from CPU arrays (it solves CPU arrays)."""
        return self._cpu

    def _gpu_only(self, what):
        if self._cpu:
            raise RuntimeError(f"{what} needs a solver built from CUDA arrays.")

    # -- checks of src/main.cpp:83-100 --------------------------------------
    def _prepare(self, b, x, dtype):
        torch = _torch()
        tb, tx = _as_torch(b), _as_torch(x)
        if tb.dim() != 1 and tb.dim() != 2:
            raise ValueError("Expected 1D or 2D tensors as input.")
        if tb.shape[0] != tx.shape[0] or (tb.dim() == 2 and (tx.dim() != 2 or tb.shape[1] != tx.shape[1])):
            raise ValueError("x and b should have the same dimensions.")
        db, dx = _device_of(b), _device_of(x)
        if db[0] != dx[0]:
            raise ValueError("x and b should be on the same device.")
        if db[0] == "cpu":
            if not self._cpu:
                raise ValueError("Input device is CPU but the solver was initialized for CUDA.")
        elif db[0] == "cuda":
            if self._cpu:
                raise ValueError("Input device is CUDA but the solver was initialized for CPU.")
        else:
            raise ValueError("Unsupported input device! Only CPU and CUDA arrays are supported.")
        if not self._cpu and (tb.device.index != self._device or tx.device.index != self._device):
            raise ValueError("x and b should be on the device the solver was created on.")
        if tb.dtype != dtype or tx.dtype != dtype:
            raise TypeError(f"solve(): b and x must be {dtype} arrays (no implicit conversion).")
        if not tb.is_contiguous() or not tx.is_contiguous():
            raise TypeError("solve(): b and x must be C-contiguous.")
        if tb.shape[0] != self._n:
            raise ValueError("b and x must have n_rows rows.")
        nrhs = tb.shape[1] if tb.dim() == 2 else 1
        if self._cpu:
            return tb, tx, nrhs, None
        stream = torch.cuda.current_stream(self._device).cuda_stream
        return tb, tx, nrhs, stream

    def solve(self, b, x):
        """Solve A x = b for the right-hand sides in b (vector or (n, n_rhs)),
        writing x in place (asynchronous on the current CUDA stream)."""
        torch = _torch()
        dtype = torch.float32 if self._precision == 0 else torch.float64
        tb, tx, nrhs, stream = self._prepare(b, x, dtype)
        if self._cpu:
            self._solve_cpu(tb, tx, nrhs)
            return
        if self._refine:
            self._solve_refined(tb, tx, nrhs, stream, self._tol, self._max_iter, stats=False)
            return
        st = _ffi.lib().gbchol_solve(self._h, self._precision, nrhs, C.c_void_p(tb.data_ptr()),
                                     C.c_void_p(tx.data_ptr()), C.c_void_p(stream))
        _ffi.check(st)

    def _solve_cpu(self, tb, tx, nrhs):
        # host solve in FP64 (blocks until x is written, like cholmod_solve)
        if tx.numel() and not _writable(tx):
            raise ValueError("solve(): x must be writable.")
        st = _ffi.lib().gbchol_factor_solve(self._fh, self._precision, int(nrhs), C.c_void_p(tb.data_ptr()),
                                            C.c_void_p(tx.data_ptr()), 0)
        _ffi.check(st)

    def _solve_refined(self, tb, tx, nrhs, stream, tol, max_iter, stats):
        rs = _ffi.RefineStats()
        if tb.data_ptr() == tx.data_ptr():
            raise ValueError("Refined solves need distinct b and x arrays.")
        st = _ffi.lib().gbchol_solve_refined(
            self._h, nrhs, C.c_void_p(tb.data_ptr()), C.c_void_p(tx.data_ptr()), float(tol),
            int(max_iter), C.c_void_p(stream), C.byref(rs) if stats else None)
        _ffi.check(st)
        if stats:
            return _refine_result(int(rs.iterations), bool(rs.converged), float(rs.max_rel_residual), tol)
        return None

    def check(self):
        """Synchronise and raise if a device-side wait expired in a solve
        (nothing to check for a CPU solver: its solves are synchronous)."""
        if self._cpu:
            return
        _ffi.check(_ffi.lib().gbchol_check(self._h))

    def reserve(self, n_rhs):
        """Preallocate scratch for up to n_rhs RHS (before CUDA-graph capture)."""
        self._gpu_only("reserve")
        _ffi.check(_ffi.lib().gbchol_reserve(self._h, int(n_rhs)))

    def refactorize(self, ii, jj, x, type):
        """New values for the same sparsity pattern (arguments as the
        constructor's; NumPy or torch, host or device): the ordering, the
        symbolic factor and the level analysis are kept, the numeric factor is
        recomputed on the host and uploaded (gbchol_refactorize). ValueError if
        the pattern differs or the matrix is not positive definite; the solver
        then keeps its old factor. No counterpart in the reference."""
        type = MatrixType(int(type))
        nx = _check_shapes(self._n, ii, jj, x, type)
        hi = _host_vector(ii, np.int32, "ii")
        hj = _host_vector(jj, np.int32, "jj")
        hx = _host_vector(x, np.float64, "x")
        if self._cpu:
            _ffi.check(_ffi.lib().gbchol_factor_refactorize(self._fh, int(nx), _ptr(hi), _ptr(hj), _ptr(hx),
                                                            int(type), 0))
            return
        torch = _torch()
        with torch.cuda.device(self._device):
            st = _ffi.lib().gbchol_refactorize(self._h, int(nx), _ptr(hi), _ptr(hj), _ptr(hx), int(type))
        _ffi.check(st)

    def replan(self, min_top_width=8, part_keep=16, part_group=0):
        """Rebuild the solve plan with other tuning parameters (gbchol_replan):
        supernodes at least `min_top_width` columns wide and their ancestors
        are solved as dense blocks; long block lists keep `part_keep` blocks
        and hand the rest to partial sums of about `part_group` blocks.
        Results change only by rounding. Batches built from this solver must
        be built again. No counterpart in the reference."""
        self._gpu_only("replan")
        _ffi.check(_ffi.lib().gbchol_replan(self._h, int(min_top_width), int(part_keep), int(part_group)))

    def autotune(self, n_rhs, precision=None, candidates=(4, 8, 16, 32), reps=3):
        """Time `reps` solves of `n_rhs` RHS for each candidate top-region
        width and keep the fastest plan (gbchol_autotune); returns the chosen
        width. `precision`: "float" / "double" (default: the precision the
        solver's solves run in; FP32 for a refining CholeskySolverD). No
        counterpart in the reference."""
        self._gpu_only("autotune")
        if precision is None:
            prec = 0 if (self._precision == 0 or self._refine) else 1
        else:
            prec = 0 if precision == "float" else 1
        cand = (C.c_int32 * len(candidates))(*[int(c) for c in candidates])
        chosen = C.c_int32(0)
        _ffi.check(_ffi.lib().gbchol_autotune(self._h, prec, int(n_rhs), cand, len(candidates), int(reps),
                                              C.byref(chosen)))
        return int(chosen.value)

    def autotune_sweeps(self, n_rhs, precision=None, reps=3):
        """Time the sweep variants for `n_rhs` RHS on the current plan and keep
        the fastest for later solves of that RHS count (gbchol_autotune_sweeps):
        the top-region kernel ("sliced": 32-column RHS slices, "bulk": one work
        item per unit for every RHS column, "bulk_tc": the same on the tensor
        cores, "bulk_2slices" / "bulk_4slices": one work item per unit and
        column half / quarter), the row sweeps' lane mode (lanes over the RHS for <= 8 RHS) and
        the rows per row-sweep ticket. Returns the choice as a dict. No
        counterpart in the reference."""
        self._gpu_only("autotune_sweeps")
        if precision is None:
            prec = 0 if (self._precision == 0 or self._refine) else 1
        else:
            prec = 0 if precision == "float" else 1
        choice = C.c_int32(0)
        _ffi.check(_ffi.lib().gbchol_autotune_sweeps(self._h, prec, int(n_rhs), int(reps), C.byref(choice)))
        v = int(choice.value)
        return {"kernel": ("sliced", "bulk", "bulk_tc", "bulk_2slices", "bulk_4slices")[v & 15],
                "rhs_split": bool((v >> 4) & 15),
                "rows_per_ticket": v >> 8}

    def info(self) -> SolverInfo:
        self._gpu_only("info")
        inf = _ffi.Info()
        _ffi.check(_ffi.lib().gbchol_get_info(self._h, C.byref(inf)))
        return SolverInfo(inf.n, inf.device, inf.nnz_a, inf.nnz_l, inf.levels_lower,
                          inf.levels_upper, inf.n_supernodes, inf.max_supernode,
                          inf.factor_flops, inf.factor_seconds, inf.analysis_seconds,
                          inf.top_rows, inf.top_units, inf.top_blocks, inf.launches_per_solve)

    def levels(self, lower=True):
        """(row_levels, order, max_lvl) of the analysis of L (lower) or L^T."""
        self._gpu_only("levels")
        n = self._n
        lev = np.zeros(n, np.int32)
        order = np.zeros(n, np.int32)
        mx = C.c_int32(0)
        _ffi.check(_ffi.lib().gbchol_get_levels(self._h, 1 if lower else 0, _ptr(lev), _ptr(order),
                                                C.byref(mx)))
        return lev, order, int(mx.value)

    def factor(self):
        """Host copy (perm, colptr, rowidx, vals) of the factor L (CSC, diagonal first)."""
        n = self._n
        if self._cpu:
            nn, nz, nsn, fl = C.c_int32(), C.c_int64(), C.c_int32(), C.c_double()
            _ffi.check(_ffi.lib().gbchol_factor_info(self._fh, C.byref(nn), C.byref(nz), C.byref(nsn),
                                                     C.byref(fl)))
            perm = np.zeros(n, np.int32)
            colptr = np.zeros(n + 1, np.int32)
            rowidx = np.zeros(nz.value, np.int32)
            vals = np.zeros(nz.value, np.float64)
            _ffi.check(_ffi.lib().gbchol_factor_export(self._fh, _ptr(perm), _ptr(colptr), _ptr(rowidx),
                                                       _ptr(vals)))
            return perm, colptr, rowidx, vals
        nnz = self.info().nnz_l
        perm = np.zeros(n, np.int32)
        colptr = np.zeros(n + 1, np.int32)
        rowidx = np.zeros(nnz, np.int32)
        vals = np.zeros(nnz, np.float64)
        _ffi.check(_ffi.lib().gbchol_get_factor(self._h, _ptr(perm), _ptr(colptr), _ptr(rowidx),
                                                _ptr(vals)))
        return perm, colptr, rowidx, vals

    # -- serialised factor (no reference counterpart) ---------------------
    FORMAT = "gbchol-factor-1"

    def save(self, path):
        """Write the analysed factor (permutation and L in CSC, diagonal first,
        FP64 values) to an .npz file, so that another process rebuilds the
        solver with `load` without ordering or factorising again."""
        perm, colptr, rowidx, vals = self.factor()
        np.savez(path, format=np.array(self.FORMAT), n=np.int64(self._n), perm=perm, colptr=colptr,
                 rowidx=rowidx, vals=vals)

    @classmethod
    def load(cls, path, device=0):
        """Rebuild a solver from a file written by `save` on CUDA device
        `device` (gbchol_create_from_factor: the factor is validated, the
        level analysis and the solve plan are redone on the device). A loaded
        CholeskySolverD solves in FP64 (refinement needs A, which the file
        does not hold)."""
        with np.load(path) as z:
            if str(z["format"]) != cls.FORMAT:
                raise ValueError(f"Not a {cls.FORMAT} file.")
            n = int(z["n"])
            perm = np.ascontiguousarray(z["perm"], np.int32)
            colptr = np.ascontiguousarray(z["colptr"], np.int32)
            rowidx = np.ascontiguousarray(z["rowidx"], np.int32)
            vals = np.ascontiguousarray(z["vals"], np.float64)
        if perm.shape != (n,) or colptr.shape != (n + 1,) or rowidx.shape != vals.shape or \
                rowidx.shape[0] != int(colptr[-1]):
            raise ValueError("Inconsistent factor arrays in the file.")
        self = cls.__new__(cls)
        self._h = None
        self._fh = None
        self._cpu = False
        self._device = int(device)
        self._refine = False
        self._tol = 1e-10
        self._max_iter = 10
        store = _ffi.STORE_F32 if self._precision == 0 else _ffi.STORE_F64
        torch = _torch()
        h = C.c_void_p()
        with torch.cuda.device(self._device):
            st = _ffi.lib().gbchol_create_from_factor(n, _ptr(perm), _ptr(colptr), _ptr(rowidx), _ptr(vals),
                                                      store, C.byref(h))
        _ffi.check(st)
        self._h = h
        self._n = n
        return self

    @property
    def handle(self):
        return self._h


def _writable(t):
    try:
        return bool(t.numpy().flags.writeable)
    except (RuntimeError, TypeError, ValueError):
        return True


def _len(a):
    try:
        return int(a.shape[0])
    except (AttributeError, IndexError, TypeError):
        return len(a)


class CholeskySolverF(_CholeskySolver):
    """Single-precision solver implementation (src/docstr.h)."""

    _precision = 0


class CholeskySolverD(_CholeskySolver):
    """Double-precision solver implementation (src/docstr.h).

    ``refine=True`` keeps an FP32 copy of the factor and the FP64 matrix; then
    ``solve`` runs FP32 solves with FP64-residual iterative refinement to
    ``tol`` and ``solve_fp64`` the plain FP64 solve. (A solver built from CPU
    arrays solves in FP64 on the host and ignores ``refine``.)
    """

    _precision = 1

    def solve_refined(self, b, x, tol=None, max_iter=None) -> RefineResult:
        """FP32 solve + FP64 iterative refinement; synchronises and returns stats."""
        self._gpu_only("solve_refined")
        if not self._refine:
            raise RuntimeError("solve_refined needs CholeskySolverD(..., refine=True).")
        torch = _torch()
        tb, tx, nrhs, stream = self._prepare(b, x, torch.float64)
        return self._solve_refined(tb, tx, nrhs, stream, self._tol if tol is None else tol,
                                   self._max_iter if max_iter is None else max_iter, stats=True)

    def solve_fp64(self, b, x):
        """Plain FP64 solve regardless of ``refine``."""
        torch = _torch()
        tb, tx, nrhs, stream = self._prepare(b, x, torch.float64)
        if self._cpu:
            self._solve_cpu(tb, tx, nrhs)
            return
        st = _ffi.lib().gbchol_solve(self._h, 1, nrhs, C.c_void_p(tb.data_ptr()),
                                     C.c_void_p(tx.data_ptr()), C.c_void_p(stream))
        _ffi.check(st)
