"""Solvers built from CPU arrays: the reference's CPU-device path
(src/main.cpp:68-70, 83-91; src/cholesky_solver.cpp:435-463), which solves
on the host cores in FP64 and rounds x to the arrays' type.

Ports the CPU halves of the reference's own tests (tests/test_cholesky.py:
test_solver and test_matrices with device="cpu", test_frameworks for numpy
and torch) and checks the product's host solve (gbchol_factor_solve) against
the oracle's restatement of cholmod_solve on the same factor. No GPU needed."""
import ctypes as C

import numpy as np
import pytest

import oracle
from cholespy_gb300 import _ffi, workloads
from helpers import RHS, STRUCTURES, reference_problem, spsolve_ref, structural_cases


def _solver_cls(variant):
    from cholespy_gb300 import CholeskySolverD, CholeskySolverF
    return CholeskySolverF if variant == "float" else CholeskySolverD


@pytest.mark.parametrize("name", ["cube", "ico3", "ico5"])
@pytest.mark.parametrize("variant", ["float", "double"])
def test_solver_cpu(gblib, name, variant):
    """tests/test_cholesky.py:10-44 with device="cpu": every RHS count of the
    reference test, 256 included (its CPU path has no 128 limit)."""
    import torch
    from cholespy_gb300 import MatrixType
    dtype = np.float32 if variant == "float" else np.float64
    n, vals, idx, b = reference_problem(name, dtype=dtype)
    x = spsolve_ref(n, vals, idx, b)
    solver = _solver_cls(variant)(n, torch.tensor(idx[0]), torch.tensor(idx[1]), torch.tensor(vals),
                                  MatrixType.COO)
    assert solver.is_cpu
    for n_rhs in RHS:
        b_t = torch.tensor(b[:, :n_rhs])
        x_t = torch.zeros_like(b_t)
        solver.solve(b_t, x_t)
        assert np.allclose(x_t.numpy(), x[:, :n_rhs])
    solver.check()


def test_matrices_cpu(gblib):
    """tests/test_cholesky.py:46-86 with device="cpu": COO, CSR and CSC agree."""
    import scipy.sparse as sp
    import torch
    from cholespy_gb300 import CholeskySolverF, MatrixType
    n, vals, idx, _ = reference_problem("cube")
    np.random.seed(45)
    A_csc = sp.csc_matrix((vals, (idx[0], idx[1])), shape=(n, n))
    A_csr = sp.csr_matrix((vals, (idx[0], idx[1])), shape=(n, n))
    b = np.random.random(size=(n, 32)).astype(np.float32)
    b_t = torch.tensor(b)
    x_ref = spsolve_ref(n, vals, idx, b)
    for ii, jj, xx, t in (
        (idx[0], idx[1], vals, MatrixType.COO),
        (A_csr.indptr, A_csr.indices, A_csr.data, MatrixType.CSR),
        (A_csc.indptr, A_csc.indices, A_csc.data, MatrixType.CSC),
    ):
        s = CholeskySolverF(n, torch.tensor(ii), torch.tensor(jj), torch.tensor(xx), t)
        x_t = torch.zeros_like(b_t)
        s.solve(b_t, x_t)
        assert np.allclose(x_t.numpy(), x_ref)


@pytest.mark.parametrize("framework", ["numpy", "torch"])
def test_frameworks_cpu(gblib, framework):
    """tests/test_cholesky.py:88-113 for the frameworks installed here."""
    from cholespy_gb300 import CholeskySolverF, MatrixType
    n, vals, idx, _ = reference_problem("cube")
    np.random.seed(45)
    b = np.random.random(size=(n, 32)).astype(np.float32)
    x_ref = spsolve_ref(n, vals, idx, b)
    if framework == "numpy":
        solver = CholeskySolverF(n, idx[0], idx[1], vals, MatrixType.COO)
        x = np.zeros_like(b)
        solver.solve(b, x)
        assert np.allclose(x, x_ref)
    else:
        import torch
        solver = CholeskySolverF(n, torch.tensor(idx[0]), torch.tensor(idx[1]), torch.tensor(vals),
                                 MatrixType.COO)
        x = torch.zeros_like(torch.tensor(b))
        solver.solve(torch.tensor(b), x)
        assert np.allclose(x.numpy(), x_ref)


# -- the C ABI against the oracle ------------------------------------------

def _factorize(gblib, n, vals, idx):
    ii = np.ascontiguousarray(idx[0], np.int32)
    jj = np.ascontiguousarray(idx[1], np.int32)
    x = np.ascontiguousarray(vals, np.float64)
    f = C.c_void_p()
    _ffi.check(gblib.gbchol_factorize(n, len(x), ii.ctypes.data, jj.ctypes.data, x.ctypes.data, 2, 0,
                                      C.byref(f)))
    nn, nnz, nsn, fl = C.c_int32(), C.c_int64(), C.c_int32(), C.c_double()
    _ffi.check(gblib.gbchol_factor_info(f, C.byref(nn), C.byref(nnz), C.byref(nsn), C.byref(fl)))
    perm = np.zeros(n, np.int32)
    colptr = np.zeros(n + 1, np.int32)
    rowidx = np.zeros(nnz.value, np.int32)
    lv = np.zeros(nnz.value, np.float64)
    _ffi.check(gblib.gbchol_factor_export(f, perm.ctypes.data, colptr.ctypes.data, rowidx.ctypes.data,
                                          lv.ctypes.data))
    return f, (perm, colptr, rowidx, lv)


def _host_solve(gblib, f, b, precision, threads, x=None):
    if x is None:
        x = np.zeros_like(b)
    nrhs = b.shape[1] if b.ndim == 2 else 1
    _ffi.check(gblib.gbchol_factor_solve(f, precision, nrhs, b.ctypes.data, x.ctypes.data, threads))
    return x


CASES = {
    "ico4": lambda: (2562, *workloads.laplacian_coo(*workloads.icosphere(4)[:2], 2.0)),
    "grid2d_40": lambda: (1600, *workloads.grid2d_coo(40, 10.0, 1.0)),
    # large enough for the parallel subtree and split-supernode phases
    "grid3d_18": lambda: (18 ** 3, *workloads.grid3d_coo(18, 1e-3)),
}


@pytest.fixture(scope="module", params=list(CASES))
def factored(request, gblib):
    n, vals, idx = CASES[request.param]()
    f, fac = _factorize(gblib, n, vals, idx)
    yield n, f, fac
    gblib.gbchol_factor_free(f)


@pytest.mark.parametrize("nrhs", [1, 3, 7, 8, 13, 32, 130])
def test_host_solve_matches_oracle(gblib, factored, nrhs):
    """FP64 host solve vs the oracle's cholmod_solve restatement on the same
    factor: <= 1e-12 relative (max-norm); every RHS chunk width (8, 4, 2, 1)."""
    n, f, (perm, colptr, rowidx, lv) = factored
    b = np.random.default_rng(nrhs).standard_normal((n, nrhs))
    x = _host_solve(gblib, f, b, 1, 0)
    xo = oracle.cpu_solve(perm, colptr, rowidx, lv, b, threads=4)
    assert np.abs(x - xo).max() <= 1e-12 * np.abs(xo).max()


def test_host_solve_float_rounds_fp64_result(gblib, factored):
    """CholeskySolverF on CPU arrays: b read as FP64, x the FP64 solution
    rounded to float (src/cholesky_solver.cpp:446-462)."""
    n, f, (perm, colptr, rowidx, lv) = factored
    b = np.random.default_rng(5).standard_normal((n, 5)).astype(np.float32)
    x = _host_solve(gblib, f, b, 0, 0)
    assert x.dtype == np.float32
    xo = oracle.cpu_solve(perm, colptr, rowidx, lv, b.astype(np.float64), threads=4)
    # one FP32 rounding of a result that agrees with the oracle to ~1e-15
    assert np.abs(x.astype(np.float64) - xo).max() <= 1.2e-7 * np.abs(xo).max()


@pytest.mark.parametrize("nrhs", [1, 4, 24])
def test_host_solve_thread_count_bit_identical(gblib, factored, nrhs):
    """The sum order is fixed by the factor and the RHS count: results are
    bit-identical for every thread count (1 thread, the split phases with
    fewer RHS chunks than threads, whole chunks per thread)."""
    n, f, _ = factored
    b = np.random.default_rng(11).standard_normal((n, nrhs))
    ref = _host_solve(gblib, f, b, 1, 1)
    for threads in (2, 3, 5, 8, 0):
        x = _host_solve(gblib, f, b, 1, threads)
        assert np.array_equal(x, ref), threads


def test_host_solve_aliased_and_vector(gblib, factored):
    """b and x may be the same array; a 1-D b is one RHS."""
    n, f, _ = factored
    b = np.random.default_rng(2).standard_normal(n)
    x = _host_solve(gblib, f, b, 1, 0)
    y = b.copy()
    _host_solve(gblib, f, y, 1, 0, x=y)
    assert np.array_equal(x, y)
    B = np.random.default_rng(3).standard_normal((n, 9))
    X = _host_solve(gblib, f, B, 1, 0)
    _host_solve(gblib, f, B, 1, 0, x=B)
    assert np.array_equal(X, B)


def test_host_solve_argument_checks(gblib, factored):
    n, f, _ = factored
    b = np.zeros((n, 2))
    assert gblib.gbchol_factor_solve(f, 2, 2, b.ctypes.data, b.ctypes.data, 0) == _ffi.EINVAL
    assert gblib.gbchol_factor_solve(f, 1, -1, b.ctypes.data, b.ctypes.data, 0) == _ffi.EINVAL
    assert gblib.gbchol_factor_solve(f, 1, 2, None, b.ctypes.data, 0) == _ffi.EINVAL
    assert gblib.gbchol_factor_solve(None, 1, 2, b.ctypes.data, b.ctypes.data, 0) == _ffi.EINVAL
    assert gblib.gbchol_factor_solve(f, 1, 0, None, None, 0) == _ffi.OK


# -- the Python edge -------------------------------------------------------

def test_cpu_solver_errors_and_extensions(gblib):
    """Device and dtype checks of src/main.cpp:83-100; GPU-only extensions
    refuse a CPU solver with a clear error."""
    from cholespy_gb300 import BatchSolver, CholeskySolverD, CholeskySolverF, MatrixType
    n, vals, idx, b = reference_problem("ico3", ncols=4)
    s = CholeskySolverD(n, idx[0], idx[1], vals, MatrixType.COO)
    x = np.zeros_like(b)
    s.solve(b, x)
    np.testing.assert_allclose(x, spsolve_ref(n, vals, idx, b), rtol=1e-10, atol=1e-12)
    with pytest.raises(TypeError):
        s.solve(b.astype(np.float32), x.astype(np.float32))
    with pytest.raises(ValueError, match="same dimensions"):
        s.solve(b, np.zeros((n, 3)))
    with pytest.raises(ValueError, match="1D or 2D"):
        s.solve(np.zeros((n, 2, 2)), np.zeros((n, 2, 2)))
    for call in (lambda: s.levels(), lambda: s.info(), lambda: s.replan(), lambda: s.reserve(4),
                 lambda: s.solve_refined(b, x)):
        with pytest.raises(RuntimeError, match="CUDA arrays"):
            call()
    with pytest.raises(ValueError, match="CUDA arrays"):
        BatchSolver([CholeskySolverF(n, idx[0], idx[1], vals, MatrixType.COO)], [1])
    # the plain FP64 solve of a CholeskySolverD is the same host solve
    x2 = np.zeros_like(b)
    s.solve_fp64(b, x2)
    assert np.array_equal(x, x2)


def test_cpu_solver_not_posdef(gblib):
    from cholespy_gb300 import CholeskySolverF, MatrixType
    n, vals, idx, _ = reference_problem("cube")
    with pytest.raises(ValueError, match="Matrix is not positive definite!"):
        CholeskySolverF(n, idx[0], idx[1], -vals, MatrixType.COO)


def test_cpu_solver_refactorize_and_factor(gblib):
    """New values on the same pattern; factor() exports the host factor."""
    from cholespy_gb300 import CholeskySolverD, MatrixType
    n, vals, idx, b = reference_problem("ico3", ncols=3)
    s = CholeskySolverD(n, idx[0], idx[1], vals, MatrixType.COO)
    perm, colptr, rowidx, lv = s.factor()
    assert sorted(perm) == list(range(n)) and colptr[-1] == len(rowidx) == len(lv)
    vals2 = vals * 1.5
    s.refactorize(idx[0], idx[1], vals2, MatrixType.COO)
    x = np.zeros_like(b)
    s.solve(b, x)
    np.testing.assert_allclose(x, spsolve_ref(n, vals2, idx, b), rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("case", list(STRUCTURES))
def test_host_solve_structures(gblib, case):
    """Elimination forests (several roots), a dense row, no off-diagonal
    entries, a 1 x 1 system and a dense block: solutions vs spsolve,
    bit-identical for 1 and all threads."""
    from scipy.sparse.linalg import spsolve
    A = structural_cases()[case]
    n = A.shape[0]
    f, _ = _factorize(gblib, n, A.data, (A.row, A.col))
    try:
        for r in (1, 5, 40):
            b = np.random.default_rng(r).standard_normal((n, r))
            x = _host_solve(gblib, f, b, 1, 0)
            xr = spsolve(A.tocsc(), b).reshape(b.shape)
            assert np.abs(x - xr).max() <= 1e-10 * np.abs(xr).max()
            assert np.array_equal(x, _host_solve(gblib, f, b, 1, 1))
    finally:
        gblib.gbchol_factor_free(f)


def test_cpu_solver_concurrent_solves(gblib):
    """Solves of one CPU solver from several threads at once (the first ones
    included, which build the host solve's structure) give the results of
    sequential solves: a solve only reads the factor."""
    import threading
    from cholespy_gb300 import CholeskySolverD, MatrixType
    n, vals, idx = 18 ** 3, *workloads.grid3d_coo(18, 1e-3)
    s = CholeskySolverD(n, idx[0], idx[1], vals, MatrixType.COO)
    bs = [np.random.default_rng(k).standard_normal((n, 1 + 3 * k)) for k in range(6)]
    xs = [np.zeros_like(b) for b in bs]
    errs = []

    def work(k):
        try:
            s.solve(bs[k], xs[k])
        except Exception as e:  # pragma: no cover - reported below
            errs.append(e)

    threads = [threading.Thread(target=work, args=(k,)) for k in range(len(bs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errs
    for b, x in zip(bs, xs):
        y = np.zeros_like(b)
        s.solve(b, y)
        assert np.array_equal(x, y)


class _DLPackOnly:
    """An array known only through the DLPack protocol (no NumPy or torch
    type), as TensorFlow, JAX or Dr.Jit arrays reach the solver."""

    def __init__(self, a):
        self._a = a

    def __dlpack__(self, *args, **kwargs):
        return self._a.__dlpack__(*args, **kwargs)

    def __dlpack_device__(self):
        return self._a.__dlpack_device__()

    @property
    def shape(self):
        return self._a.shape


def test_frameworks_dlpack_cpu(gblib):
    """tests/test_cholesky.py:88-199 for frameworks that are not installed
    here: the same case through arrays that expose only DLPack."""
    from cholespy_gb300 import CholeskySolverF, MatrixType
    n, vals, idx, _ = reference_problem("cube")
    np.random.seed(45)
    b = np.random.random(size=(n, 32)).astype(np.float32)
    x_ref = spsolve_ref(n, vals, idx, b)
    solver = CholeskySolverF(n, _DLPackOnly(np.ascontiguousarray(idx[0], np.int32)),
                             _DLPackOnly(np.ascontiguousarray(idx[1], np.int32)),
                             _DLPackOnly(np.ascontiguousarray(vals)), MatrixType.COO)
    assert solver.is_cpu
    x = np.zeros_like(b)
    solver.solve(_DLPackOnly(b), _DLPackOnly(x))
    assert np.allclose(x, x_ref)


def test_host_solve_plan_independent_of_threads(gblib):
    """The host solve's structure (built at a factor's first solve, in
    parallel for large factors) is the same whatever thread count builds it:
    two factors of one matrix, first solved with 1 and with all threads, give
    bit-identical solutions (32^3: above the parallel-build size)."""
    n, vals, idx = 32 ** 3, *workloads.grid3d_coo(32, 1e-3)
    f1, _ = _factorize(gblib, n, vals, idx)
    f2, _ = _factorize(gblib, n, vals, idx)
    try:
        b = np.random.default_rng(4).standard_normal((n, 3))
        x1 = _host_solve(gblib, f1, b, 1, 1)
        x2 = _host_solve(gblib, f2, b, 1, 0)
        assert np.array_equal(x1, x2)
        assert np.array_equal(_host_solve(gblib, f1, b, 1, 0), x1)
    finally:
        gblib.gbchol_factor_free(f1)
        gblib.gbchol_factor_free(f2)


@pytest.mark.parametrize("name", ["cube", "ico3"])
@pytest.mark.parametrize("variant", ["float", "double"])
def test_cpu_solver_golden(gblib, name, variant):
    """The CPU-array solver against the committed golden solutions of the
    reference's test recipe (tests/golden/, spsolve answers; the reference's
    own tests/test_cholesky.py:31-44 check np.allclose against spsolve)."""
    from pathlib import Path
    from cholespy_gb300 import MatrixType
    d = np.load(Path(__file__).resolve().parent / "golden" / f"spsolve_{name}.npz")
    n = int(d["n"])
    dt = np.float32 if variant == "float" else np.float64
    s = _solver_cls(variant)(n, d["idx"][0], d["idx"][1], d["vals"], MatrixType.COO)
    b = np.ascontiguousarray(d["b"], dt)
    x = np.zeros_like(b)
    s.solve(b, x)
    assert np.allclose(x, d["x"])
    if variant == "double":
        assert np.abs(x - d["x"]).max() <= 1e-12 * np.abs(d["x"]).max()


def test_reference_import_name(gblib):
    """`from cholespy import ...` (the reference's import name) gives this
    build's classes, so code written for the reference runs unchanged."""
    import cholespy
    import cholespy_gb300
    assert cholespy.CholeskySolverF is cholespy_gb300.CholeskySolverF
    assert cholespy.CholeskySolverD is cholespy_gb300.CholeskySolverD
    assert cholespy.MatrixType is cholespy_gb300.MatrixType
    n, vals, idx, b = reference_problem("cube", ncols=4)
    s = cholespy.CholeskySolverD(n, idx[0], idx[1], vals, cholespy.MatrixType.COO)
    x = np.zeros_like(b)
    s.solve(b, x)
    assert np.allclose(x, spsolve_ref(n, vals, idx, b))


def test_refine_result_never_reports_nonfinite_as_converged():
    """The Python edge reports a refined solve as converged only when its
    max relative residual is finite and within tol, whatever the device
    flag says (a NaN residual must not read as converged)."""
    from cholespy_gb300.solver import _refine_result
    assert _refine_result(1, True, 5e-14, 1e-10).converged
    assert not _refine_result(1, True, float("nan"), 1e-10).converged
    assert not _refine_result(1, True, float("inf"), 1e-10).converged
    assert not _refine_result(1, True, 2e-10, 1e-10).converged
    assert not _refine_result(3, False, 5e-14, 1e-10).converged
