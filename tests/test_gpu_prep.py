"""GPU tests of the construction input prep on the device
(gbchol_create_device, csrc/prep.cu): the COO / CSR / CSC -> sorted,
duplicate-summed CSC conversion of CUDA inputs gives the same factor, bit for
bit, as the host conversion (gbchol_create; the reference's
src/cholesky_solver.cpp:8-149 after its device-to-host copies,
src/main.cpp:47-67), and rejects bad inputs with the host path's messages."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _factor_via(torch, n, ii, jj, x, fmt, device_prep):
    from cholespy_gb300 import _ffi
    lib = _ffi.lib()
    h = C.c_void_p()
    if device_prep:
        di = torch.tensor(ii, dtype=torch.int32, device="cuda")
        dj = torch.tensor(jj, dtype=torch.int32, device="cuda")
        dx = torch.tensor(x, dtype=torch.float64, device="cuda")
        st = lib.gbchol_create_device(n, len(x), C.c_void_p(di.data_ptr()), C.c_void_p(dj.data_ptr()),
                                      C.c_void_p(dx.data_ptr()), fmt, _ffi.STORE_F64 | _ffi.STORE_A64, C.byref(h))
    else:
        hi = np.ascontiguousarray(ii, np.int32)
        hj = np.ascontiguousarray(jj, np.int32)
        hx = np.ascontiguousarray(x, np.float64)
        st = lib.gbchol_create(n, len(x), hi.ctypes.data, hj.ctypes.data, hx.ctypes.data, fmt,
                               _ffi.STORE_F64 | _ffi.STORE_A64, C.byref(h))
    _ffi.check(st)
    return h


def _export(h):
    from cholespy_gb300 import _ffi
    lib = _ffi.lib()
    inf = _ffi.Info()
    _ffi.check(lib.gbchol_get_info(h, C.byref(inf)))
    n, nnz = inf.n, inf.nnz_l
    perm = np.zeros(n, np.int32)
    Lp = np.zeros(n + 1, np.int32)
    Li = np.zeros(nnz, np.int32)
    Lx = np.zeros(nnz, np.float64)
    _ffi.check(lib.gbchol_get_factor(h, perm.ctypes.data, Lp.ctypes.data, Li.ctypes.data, Lx.ctypes.data))
    return perm, Lp, Li, Lx


def _inputs(name):
    import scipy.sparse as sp
    from cholespy_gb300 import workloads
    if name == "ico4":
        n, faces, _ = workloads.icosphere(4)
        vals, idx = workloads.laplacian_coo(n, faces, 2.0)   # duplicate diagonal entries
    else:
        n = 16 ** 3
        vals, idx = workloads.grid3d_coo(16, 1e-3)
    rng = np.random.default_rng(3)
    p = rng.permutation(len(vals))                            # unsorted input order
    ii, jj, x = idx[0][p], idx[1][p], vals[p]
    csr = sp.csr_matrix((x, (ii, jj)), shape=(n, n))          # CSR / CSC with unsorted, duplicate entries
    return n, (ii, jj, x), csr


@pytest.mark.parametrize("name", ["ico4", "grid3d_16"])
@pytest.mark.parametrize("fmt", [2, 1, 0])
def test_device_prep_bit_identical(cuda, name, fmt):
    from cholespy_gb300 import _ffi
    torch = cuda
    n, (ii, jj, x), _ = _inputs(name)
    if fmt == 1:  # CSR built by hand, entries of a row in input order (not sorted, duplicates kept)
        order = np.argsort(ii, kind="stable")
        ptr = np.concatenate([[0], np.cumsum(np.bincount(ii, minlength=n))])
        a, b, v = ptr, jj[order], x[order]
    elif fmt == 0:  # CSC likewise
        order = np.argsort(jj, kind="stable")
        ptr = np.concatenate([[0], np.cumsum(np.bincount(jj, minlength=n))])
        a, b, v = ptr, ii[order], x[order]
    else:
        a, b, v = ii, jj, x
    hh = _factor_via(torch, n, a, b, v, fmt, False)
    hd = _factor_via(torch, n, a, b, v, fmt, True)
    try:
        for u, w in zip(_export(hh), _export(hd)):
            np.testing.assert_array_equal(u, w)
    finally:
        _ffi.lib().gbchol_destroy(hh)
        _ffi.lib().gbchol_destroy(hd)


def test_device_prep_errors(cuda):
    from cholespy_gb300 import CholeskySolverF, MatrixType
    torch = cuda
    n, (ii, jj, x), _ = _inputs("ico4")
    bad = ii.copy()
    bad[7] = n + 3
    with pytest.raises(ValueError, match="Sparse COO matrix: index out of range."):
        CholeskySolverF(n, torch.tensor(bad, device="cuda"), torch.tensor(jj, device="cuda"),
                        torch.tensor(x, device="cuda"), MatrixType.COO)
    ptr = np.concatenate([[0], np.cumsum(np.bincount(ii, minlength=n))])
    ptr[5] = ptr[6] + 1
    order = np.argsort(ii, kind="stable")
    with pytest.raises(ValueError, match="Sparse CSR matrix: Invalid pointer array."):
        CholeskySolverF(n, torch.tensor(ptr, device="cuda"), torch.tensor(jj[order], device="cuda"),
                        torch.tensor(x[order], device="cuda"), MatrixType.CSR)


def test_device_cast_matches_host_cast(cuda):
    """A solver keeping both factors casts its FP32 copy on the device; an
    FP32-only solver casts on the host. Same factor and plan, so their FP32
    solves agree bit for bit."""
    from cholespy_gb300 import CholeskySolverD, CholeskySolverF, MatrixType, _ffi
    torch = cuda
    n, (ii, jj, x), _ = _inputs("grid3d_16")
    args = (torch.tensor(ii, device="cuda"), torch.tensor(jj, device="cuda"), torch.tensor(x, device="cuda"),
            MatrixType.COO)
    sf = CholeskySolverF(n, *args)
    sd = CholeskySolverD(n, *args, refine=True)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for nrhs in (1, 8, 64, 128):
        b = torch.randn(n, nrhs, device="cuda", dtype=torch.float32)
        x1, x2 = torch.zeros_like(b), torch.zeros_like(b)
        _ffi.check(_ffi.lib().gbchol_solve(sf.handle, 0, nrhs, C.c_void_p(b.data_ptr()), C.c_void_p(x1.data_ptr()),
                                           stream))
        _ffi.check(_ffi.lib().gbchol_solve(sd.handle, 0, nrhs, C.c_void_p(b.data_ptr()), C.c_void_p(x2.data_ptr()),
                                           stream))
        torch.cuda.synchronize()
        assert torch.equal(x1, x2)
