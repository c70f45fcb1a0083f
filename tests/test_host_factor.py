"""CPU tests of the product's host factorisation (the CHOLMOD replacement)
through the C ABI, checked against the oracle's up-looking LL^T on the same
permutation, and of the input checks."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from cholespy_gb300 import _ffi, workloads

ROOT = Path(__file__).resolve().parent.parent


def factorize(gblib, n, ii, jj, x, fmt, threads=2):
    ii = np.ascontiguousarray(ii, np.int32)
    jj = np.ascontiguousarray(jj, np.int32)
    x = np.ascontiguousarray(x, np.float64)
    f = C.c_void_p()
    st = gblib.gbchol_factorize(n, len(x), ii.ctypes.data, jj.ctypes.data, x.ctypes.data, fmt,
                                threads, C.byref(f))
    _ffi.check(st)
    nn, nnz, nsn, fl = C.c_int32(), C.c_int64(), C.c_int32(), C.c_double()
    _ffi.check(gblib.gbchol_factor_info(f, C.byref(nn), C.byref(nnz), C.byref(nsn), C.byref(fl)))
    perm = np.zeros(n, np.int32)
    colptr = np.zeros(n + 1, np.int32)
    rowidx = np.zeros(nnz.value, np.int32)
    vals = np.zeros(nnz.value, np.float64)
    _ffi.check(gblib.gbchol_factor_export(f, perm.ctypes.data, colptr.ctypes.data,
                                          rowidx.ctypes.data, vals.ctypes.data))
    gblib.gbchol_factor_free(f)
    return perm, colptr, rowidx, vals, nsn.value


CASES = {
    "cube": lambda: (8, *workloads.laplacian_coo(*workloads.cube(), 2.0)),
    "ico3": lambda: (642, *workloads.laplacian_coo(*workloads.icosphere(3)[:2], 2.0)),
    "grid24": lambda: (576, *workloads.grid2d_coo(24, 10.0, 1.0)),
    "grid3d_10": lambda: (1000, *workloads.grid3d_coo(10, 1e-3)),
}


@pytest.mark.parametrize("case", list(CASES))
def test_factor_matches_oracle(gblib, case):
    n, vals, idx = CASES[case]()
    perm, colptr, rowidx, lv, nsn = factorize(gblib, n, idx[0], idx[1], vals, 2)
    assert sorted(perm) == list(range(n))
    cp, ri, av = oracle.build_csc(n, idx[0], idx[1], vals, 2)
    Lp, Li, Lx = oracle.cholesky(n, cp, ri, av, perm)
    np.testing.assert_array_equal(colptr, Lp)       # same symbolic pattern
    np.testing.assert_array_equal(rowidx, Li)
    np.testing.assert_allclose(lv, Lx, rtol=1e-11, atol=1e-13)
    # diagonal first in every column
    assert all(rowidx[colptr[j]] == j for j in range(n))
    assert 1 <= nsn <= n


@pytest.mark.parametrize("fmt", ["COO", "CSR", "CSC"])
def test_factor_input_formats_agree(gblib, fmt):
    n, vals, idx = CASES["ico3"]()
    if fmt == "COO":
        args = (idx[0], idx[1], vals, 2)
    elif fmt == "CSR":
        m = sp.csr_matrix((vals, (idx[0], idx[1])), shape=(n, n))
        args = (m.indptr, m.indices, m.data, 1)
    else:
        m = sp.csc_matrix((vals, (idx[0], idx[1])), shape=(n, n))
        args = (m.indptr, m.indices, m.data, 0)
    perm, colptr, rowidx, lv, _ = factorize(gblib, n, *args)
    p0, c0, r0, v0, _ = factorize(gblib, n, idx[0], idx[1], vals, 2)
    np.testing.assert_array_equal(perm, p0)
    np.testing.assert_array_equal(colptr, c0)
    np.testing.assert_allclose(lv, v0, rtol=1e-13, atol=1e-15)


def test_factor_uses_lower_triangle_only(gblib):
    """CHOLMOD is called with stype = -1: strictly upper entries are ignored."""
    n, vals, idx = CASES["grid24"]()
    upper = idx[0] < idx[1]
    junk = vals.copy()
    junk[upper] = 123.0
    a = factorize(gblib, n, idx[0], idx[1], vals, 2)
    b = factorize(gblib, n, idx[0], idx[1], junk, 2)
    np.testing.assert_array_equal(a[3], b[3])


def test_factor_not_posdef(gblib):
    vals = np.array([1.0, 3.0, 3.0, 1.0])
    ii = np.array([0, 1, 0, 1])
    jj = np.array([0, 0, 1, 1])
    with pytest.raises(ValueError, match="^Matrix is not positive definite!$"):
        factorize(gblib, 2, ii, jj, vals, 2)


def test_factor_bad_indices(gblib):
    with pytest.raises(ValueError):
        factorize(gblib, 3, [0, 3], [0, 1], [1.0, 1.0], 2)
    with pytest.raises(ValueError):
        factorize(gblib, 2, [0, 2, 1], [0, 1], [1.0, 1.0], 1)  # non-monotone pointers


@pytest.mark.parametrize("k", [10, 24])
def test_factor_threads_deterministic(gblib, k):
    """The factor is bit-identical for every thread count: subtrees are
    factorised as independent tasks, children are added in a fixed order and
    the dense kernels block independently of the threads. k=24 has fronts of
    several hundred rows, above the triangular solve's row blocks."""
    n, vals, idx = k ** 3, *workloads.grid3d_coo(k, 1e-3)
    a = factorize(gblib, n, idx[0], idx[1], vals, 2, threads=1)
    for t in (2, 3, 8):
        b = factorize(gblib, n, idx[0], idx[1], vals, 2, threads=t)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[3], b[3])


def test_nested_dissection_fill_reasonable(gblib):
    """Fill of the 3-D 7-point grid stays far below the dense bound."""
    n, vals, idx = 4096, *workloads.grid3d_coo(16, 1e-3)
    _, colptr, _, _, nsn = factorize(gblib, n, idx[0], idx[1], vals, 2)
    assert colptr[-1] < 400_000  # METIS-quality ND gives ~3.9e5 on 16^3


def _export(gblib, f, n):
    nn, nnz, nsn, fl = C.c_int32(), C.c_int64(), C.c_int32(), C.c_double()
    _ffi.check(gblib.gbchol_factor_info(f, C.byref(nn), C.byref(nnz), C.byref(nsn), C.byref(fl)))
    perm = np.zeros(n, np.int32)
    colptr = np.zeros(n + 1, np.int32)
    rowidx = np.zeros(nnz.value, np.int32)
    vals = np.zeros(nnz.value, np.float64)
    _ffi.check(gblib.gbchol_factor_export(f, perm.ctypes.data, colptr.ctypes.data, rowidx.ctypes.data,
                                          vals.ctypes.data))
    return perm, colptr, rowidx, vals


def test_factor_refactorize(gblib):
    """gbchol_factor_refactorize (no reference counterpart): new values on the
    same pattern give the factor a fresh factorisation gives (same ordering:
    nested dissection depends on the pattern only); a different pattern and a
    matrix that is not positive definite are refused and leave the factor as
    it was."""
    k = 20
    n = k * k
    v1, idx = workloads.grid2d_coo(k, 10.0, 1.0)
    v2, idx2 = workloads.grid2d_coo(k, 3.0, 2.5)
    assert np.array_equal(idx, idx2)
    ii = np.ascontiguousarray(idx[0], np.int32)
    jj = np.ascontiguousarray(idx[1], np.int32)
    x1 = np.ascontiguousarray(v1, np.float64)
    x2 = np.ascontiguousarray(v2, np.float64)
    f = C.c_void_p()
    _ffi.check(gblib.gbchol_factorize(n, len(x1), ii.ctypes.data, jj.ctypes.data, x1.ctypes.data, 2, 2,
                                      C.byref(f)))
    try:
        _ffi.check(gblib.gbchol_factor_refactorize(f, len(x2), ii.ctypes.data, jj.ctypes.data, x2.ctypes.data,
                                                   2, 2))
        perm, colptr, rowidx, vals = _export(gblib, f, n)
        p2, c2, r2, v2f, _ = factorize(gblib, n, ii, jj, x2, 2)
        assert np.array_equal(perm, p2) and np.array_equal(colptr, c2) and np.array_equal(rowidx, r2)
        np.testing.assert_allclose(vals, v2f, rtol=1e-12, atol=1e-14)
        # not positive definite: refused, values kept
        bad = -x2
        st = gblib.gbchol_factor_refactorize(f, len(bad), ii.ctypes.data, jj.ctypes.data, bad.ctypes.data,
                                             2, 2)
        assert st == _ffi.ENOTPOSDEF
        assert np.array_equal(_export(gblib, f, n)[3], vals)
        # another pattern (one off-diagonal pair dropped): refused
        keep = ~(((ii == 0) & (jj == 1)) | ((ii == 1) & (jj == 0)))
        i3 = np.ascontiguousarray(ii[keep]); j3 = np.ascontiguousarray(jj[keep]); x3 = np.ascontiguousarray(x2[keep])
        st = gblib.gbchol_factor_refactorize(f, len(x3), i3.ctypes.data, j3.ctypes.data, x3.ctypes.data,
                                             2, 2)
        assert st in (_ffi.EINVAL, _ffi.OK)
        if st == _ffi.EINVAL:
            assert "pattern" in _ffi.last_error()
            assert np.array_equal(_export(gblib, f, n)[3], vals)
    finally:
        gblib.gbchol_factor_free(f)


@pytest.mark.parametrize("fmt", ["COO", "CSR", "CSC"])
def test_refactorize_cached_symbolic_bit_identical(gblib, fmt):
    """New values with the very index arrays the factor was made from take the
    cached symbolic analysis (no input sort, ordering or symbolic step); the
    result is bit-identical to a fresh factorisation of the new values and to
    the full refactorisation path (reached here by giving the same matrix in
    another format). Duplicate COO entries are summed in input order."""
    import scipy.sparse as sp
    n, faces, _ = workloads.icosphere(3)
    v1, idx = workloads.laplacian_coo(n, faces, 2.0)   # duplicate diagonal entries
    v2, _ = workloads.laplacian_coo(n, faces, 7.5)
    if fmt == "COO":
        a1 = (idx[0], idx[1], v1)
        a2 = (idx[0], idx[1], v2)
        other = sp.csr_matrix((v2, (idx[0], idx[1])), shape=(n, n))
        other = (other.indptr, other.indices, other.data, 1)
        code = 2
    else:
        mk = sp.csr_matrix if fmt == "CSR" else sp.csc_matrix
        m1 = mk((v1, (idx[0], idx[1])), shape=(n, n))
        m2 = mk((v2, (idx[0], idx[1])), shape=(n, n))
        assert np.array_equal(m1.indices, m2.indices)
        a1 = (m1.indptr, m1.indices, m1.data)
        a2 = (m2.indptr, m2.indices, m2.data)
        other = (idx[0], idx[1], v2, 2)
        code = 1 if fmt == "CSR" else 0
    arr = [np.ascontiguousarray(a, t) for a, t in zip(a1, (np.int32, np.int32, np.float64))]
    new = [np.ascontiguousarray(a, t) for a, t in zip(a2, (np.int32, np.int32, np.float64))]
    f = C.c_void_p()
    _ffi.check(gblib.gbchol_factorize(n, len(arr[2]), arr[0].ctypes.data, arr[1].ctypes.data, arr[2].ctypes.data,
                                      code, 2, C.byref(f)))
    g = C.c_void_p()
    _ffi.check(gblib.gbchol_factorize(n, len(arr[2]), arr[0].ctypes.data, arr[1].ctypes.data, arr[2].ctypes.data,
                                      code, 2, C.byref(g)))
    try:
        _ffi.check(gblib.gbchol_factor_refactorize(f, len(new[2]), new[0].ctypes.data, new[1].ctypes.data,
                                                   new[2].ctypes.data, code, 2))
        cached = _export(gblib, f, n)
        fresh = factorize(gblib, n, new[0], new[1], new[2], code)
        assert np.array_equal(cached[0], fresh[0]) and np.array_equal(cached[2], fresh[2])
        assert np.array_equal(cached[3], fresh[3])
        oi, oj, ox, ocode = (np.ascontiguousarray(other[0], np.int32), np.ascontiguousarray(other[1], np.int32),
                             np.ascontiguousarray(other[2], np.float64), other[3])
        _ffi.check(gblib.gbchol_factor_refactorize(g, len(ox), oi.ctypes.data, oj.ctypes.data, ox.ctypes.data,
                                                   ocode, 2))
        full = _export(gblib, g, n)
        assert np.array_equal(cached[3], full[3])
    finally:
        gblib.gbchol_factor_free(f)
        gblib.gbchol_factor_free(g)


def test_factor_identical_for_one_openmp_thread(gblib, tmp_path):
    """Ordering (its piece tasks take the OpenMP team size), symbolic and
    numeric factorisation give the same factor, bit for bit, in a process
    limited to one OpenMP thread as in this one (34^3: large enough for
    every parallel path)."""
    import os
    import subprocess
    import sys
    k = 34
    vals, idx = workloads.grid3d_coo(k, 1e-3)
    n = k ** 3
    here = factorize(gblib, n, idx[0], idx[1], vals, 2, threads=0)
    script = (
        "import sys, numpy as np\n"
        f"sys.path.insert(0, {str(ROOT)!r}); sys.path.insert(0, {str(ROOT / 'tests')!r})\n"
        "from cholespy_gb300 import _ffi, workloads\n"
        "from test_host_factor import factorize\n"
        f"vals, idx = workloads.grid3d_coo({k}, 1e-3)\n"
        f"p, c, r, v, _ = factorize(_ffi.lib(), {n}, idx[0], idx[1], vals, 2, threads=0)\n"
        f"np.savez({str(tmp_path / 'f.npz')!r}, p=p, c=c, r=r, v=v)\n")
    env = dict(os.environ, OMP_NUM_THREADS="1")
    out = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    with np.load(tmp_path / "f.npz") as z:
        for a, b in zip(here[:4], (z["p"], z["c"], z["r"], z["v"])):
            assert np.array_equal(a, b)
