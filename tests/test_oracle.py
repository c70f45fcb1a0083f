"""CPU tests pinning the oracle (test infrastructure) before it is trusted:
against the reference tests' golden solutions (spsolve), against scipy's
format conversions, against dense numpy Cholesky, and the level analysis
against an independent longest-path computation."""
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from cholespy_gb300 import workloads

GOLDEN = Path(__file__).resolve().parent / "golden"


def _lower_csc(n, vals, idx):
    A = sp.csc_matrix((vals, (idx[0], idx[1])), shape=(n, n))
    A.sum_duplicates()
    A.sort_indices()
    return A


@pytest.mark.parametrize("fmt", [0, 1, 2])
def test_build_csc_matches_scipy(fmt):
    rng = np.random.default_rng(0)
    n = 50
    r = rng.integers(0, n, 400)
    c = rng.integers(0, n, 400)
    v = rng.standard_normal(400)
    ref = sp.csc_matrix((v, (r, c)), shape=(n, n))
    ref.sum_duplicates()
    ref.sort_indices()
    if fmt == 2:
        got = oracle.build_csc(n, r, c, v, 2)
    elif fmt == 1:
        m = sp.csr_matrix((v, (r, c)), shape=(n, n))  # scipy keeps duplicates
        got = oracle.build_csc(n, m.indptr, m.indices, m.data, 1)
    else:
        m = sp.csc_matrix((v, (r, c)), shape=(n, n))
        got = oracle.build_csc(n, m.indptr, m.indices, m.data, 0)
    np.testing.assert_array_equal(got[0], ref.indptr)
    np.testing.assert_array_equal(got[1], ref.indices)
    np.testing.assert_allclose(got[2], ref.data, rtol=1e-14, atol=1e-14)


def test_build_csc_rejects_bad_index():
    with pytest.raises(ValueError):
        oracle.build_csc(3, [0, 5], [0, 1], [1.0, 2.0], 2)


def _levels_longest_path(rowptr, cols, lower):
    n = len(rowptr) - 1
    lev = np.zeros(n, np.int64)
    rows = range(n) if lower else range(n - 1, -1, -1)
    for r in rows:
        s, e = rowptr[r], rowptr[r + 1]
        deps = cols[s:e - 1] if lower else cols[s + 1:e]
        lev[r] = 0 if len(deps) == 0 else lev[deps].max() + 1
    return lev


@pytest.mark.parametrize("name", ["cube", "ico3"])
def test_oracle_levels(name):
    d = np.load(GOLDEN / f"spsolve_{name}.npz")
    n = int(d["n"])
    A = _lower_csc(n, d["vals"], d["idx"])
    perm = np.arange(n, dtype=np.int32)[::-1].copy()
    Lp, Li, Lx = oracle.cholesky(n, A.indptr, A.indices, A.data, perm)
    lrp, lci, _ = oracle.csr_of_lower(Lp, Li, Lx)
    for lower, (rp, ci) in ((True, (lrp, lci)), (False, (Lp, Li))):
        lev, order, mx = oracle.levels(rp, ci, lower)
        ref = _levels_longest_path(rp, ci, lower)
        np.testing.assert_array_equal(lev, ref)
        assert mx == ref.max()
        # order = rows sorted by (level, row id)
        np.testing.assert_array_equal(order, np.lexsort((np.arange(n), ref)))


@pytest.mark.parametrize("n", [1, 7, 60])
def test_oracle_cholesky_dense(n):
    rng = np.random.default_rng(n)
    M = rng.standard_normal((n, n))
    A = M @ M.T + n * np.eye(n)
    A[np.abs(A) < 0.5] = 0.0
    A += n * np.eye(n)
    perm = rng.permutation(n).astype(np.int32)
    S = sp.csc_matrix(np.tril(A))
    Lp, Li, Lx = oracle.cholesky(n, S.indptr, S.indices, S.data, perm)
    L = sp.csc_matrix((Lx, Li, Lp), shape=(n, n)).toarray()
    P = A[np.ix_(perm, perm)]
    np.testing.assert_allclose(L, np.linalg.cholesky(P), rtol=1e-10, atol=1e-12)


def test_oracle_cholesky_not_posdef():
    A = sp.csc_matrix(np.array([[1.0, 0.0], [2.0, 1.0]]))
    with pytest.raises(ValueError, match="not positive definite"):
        oracle.cholesky(2, A.indptr, A.indices, A.data, np.arange(2, dtype=np.int32))


@pytest.mark.parametrize("name", ["cube", "ico3"])
def test_oracle_pinned_to_golden(name):
    """The oracle's CPU solve and its restatement of the reference's GPU
    sweeps reproduce the reference tests' spsolve answers."""
    d = np.load(GOLDEN / f"spsolve_{name}.npz")
    n, b, xref = int(d["n"]), d["b"], d["x"]
    colptr, rowidx, vals = oracle.build_csc(n, d["idx"][0], d["idx"][1], d["vals"], 2)
    perm = np.random.default_rng(1).permutation(n).astype(np.int32)
    Lp, Li, Lx = oracle.cholesky(n, colptr, rowidx, vals, perm)
    x = oracle.cpu_solve(perm, Lp, Li, Lx, b, threads=2)
    np.testing.assert_allclose(x, xref, rtol=1e-10, atol=1e-12)
    xd = oracle.reference_solve(perm, Lp, Li, Lx, b, np.float64)
    np.testing.assert_allclose(xd, xref, rtol=1e-10, atol=1e-12)
    xf = oracle.reference_solve(perm, Lp, Li, Lx, b, np.float32)
    assert np.allclose(xf, xref)  # the reference test's own criterion (float32)


def test_oracle_float_sweeps_use_fma_order():
    """r -= val * x is a fused multiply-add, accumulated in CSR order."""
    # 2x2 lower factor: row 1 = [l10, l11]
    colptr = np.array([0, 2, 3], np.int32)
    rowidx = np.array([0, 1, 1], np.int32)
    vals = np.array([1.0, 1.0 / 3.0, 1.0])
    perm = np.array([0, 1], np.int32)
    b = np.array([[3.0], [1.0]], np.float32)
    lrp, lci, lv = oracle.csr_of_lower(colptr, rowidx, vals)
    lev, order, _ = oracle.levels(lrp, lci, True)
    tmp = oracle.solve_lower(lrp, lci, lv.astype(np.float32), order, perm, b)
    expect = np.float32(np.float64(1.0) - np.float64(np.float32(1 / 3)) * 3.0)
    assert tmp[1, 0] == expect
