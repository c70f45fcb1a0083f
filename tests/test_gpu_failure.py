"""Failure detection without a GPU fault: a bounded device-side wait on a flag
that nothing sets expires, records GBCHOL_ETIMEOUT, and the CUDA context stays
usable (a solve afterwards is correct). The reference's waits are unbounded
(kernels/kernels.cu:20-21, 108-109)."""
import ctypes as C
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_expires(cuda):
    from cholespy_gb300 import _ffi
    st = C.c_int32(-1)
    t0 = time.perf_counter()
    _ffi.check(_ffi.lib().gbchol_selftest_wait(20000, C.byref(st)))  # 20 ms
    dt = time.perf_counter() - t0
    assert st.value == _ffi.ETIMEOUT
    assert dt < 5.0
    # the context is still usable
    from cholespy_gb300 import CholeskySolverD, MatrixType, workloads
    torch = cuda
    n, vals, idx, b = workloads.config_grid64()
    s = CholeskySolverD(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                        torch.tensor(vals, device="cuda"), MatrixType.COO)
    bt = torch.tensor(b, device="cuda")
    xt = torch.zeros_like(bt)
    s.solve(bt, xt)
    s.check()
    import scipy.sparse as sp
    A = sp.csc_matrix((vals, (idx[0], idx[1])), shape=(n, n))
    assert np.linalg.norm(A @ xt.cpu().numpy() - b) / np.linalg.norm(b) < 1e-12


def test_invalid_factor_rejected_on_host(cuda):
    """A factor whose dependency structure could make a sweep wait forever
    (missing diagonal, unsorted rows) is refused before any kernel runs."""
    from cholespy_gb300 import _ffi
    h = C.c_void_p()
    perm = np.array([0, 1], np.int32)
    colptr = np.array([0, 1, 2], np.int32)
    rowidx = np.array([1, 1], np.int32)  # column 0 lacks its diagonal
    vals = np.ones(2)
    st = _ffi.lib().gbchol_create_from_factor(2, perm.ctypes.data, colptr.ctypes.data, rowidx.ctypes.data,
                                              vals.ctypes.data, _ffi.STORE_F64, C.byref(h))
    assert st == _ffi.EINVAL
    assert "diagonal" in _ffi.last_error()
