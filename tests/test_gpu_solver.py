"""GPU parity tests of the drop-in solvers against the oracle.

Ports the reference's own tests (tests/test_cholesky.py: test_solver,
test_matrices) and adds bit-exact level-analysis checks, sweep parity with
the oracle's restatement of the reference's kernels on the same factor, and
iterative refinement to 1e-10."""
import numpy as np
import pytest

import oracle
from helpers import RHS, STRUCTURES, reference_problem, spsolve_ref, structural_cases, sym_matrix

pytestmark = pytest.mark.gpu


def _solver_cls(variant):
    from cholespy_gb300 import CholeskySolverD, CholeskySolverF
    return CholeskySolverF if variant == "float" else CholeskySolverD


@pytest.mark.parametrize("name", ["cube", "ico3", "ico5"])
@pytest.mark.parametrize("variant", ["float", "double"])
def test_solver(cuda, name, variant):
    """tests/test_cholesky.py:10-44 on CUDA."""
    from cholespy_gb300 import MatrixType
    torch = cuda
    dtype = np.float32 if variant == "float" else np.float64
    n, vals, idx, b = reference_problem(name, dtype=dtype)
    x = spsolve_ref(n, vals, idx, b)
    solver = _solver_cls(variant)(n, torch.tensor(idx[0], device="cuda"),
                                  torch.tensor(idx[1], device="cuda"),
                                  torch.tensor(vals, device="cuda"), MatrixType.COO)
    for n_rhs in RHS:
        b_t = torch.tensor(b[:, :n_rhs], device="cuda")
        x_t = torch.zeros_like(b_t)
        try:
            solver.solve(b_t, x_t)
            assert np.allclose(x_t.cpu().numpy(), x[:, :n_rhs])
        except ValueError as e:
            assert n_rhs > 128
            assert str(e) == "The number of RHS should be less than 128."
    solver.check()


def test_matrices(cuda):
    """tests/test_cholesky.py:46-86: COO, CSR and CSC inputs agree."""
    import scipy.sparse as sp
    from cholespy_gb300 import CholeskySolverF, MatrixType
    torch = cuda
    n, vals, idx, _ = reference_problem("cube")
    np.random.seed(45)
    A_csc = sp.csc_matrix((vals, (idx[0], idx[1])), shape=(n, n))
    A_csr = sp.csr_matrix((vals, (idx[0], idx[1])), shape=(n, n))
    b = np.random.random(size=(n, 32)).astype(np.float32)
    b_t = torch.tensor(b, device="cuda")
    x_ref = spsolve_ref(n, vals, idx, b)
    for ii, jj, xx, t in (
        (idx[0], idx[1], vals, MatrixType.COO),
        (A_csr.indptr, A_csr.indices, A_csr.data, MatrixType.CSR),
        (A_csc.indptr, A_csc.indices, A_csc.data, MatrixType.CSC),
    ):
        s = CholeskySolverF(n, torch.tensor(ii, device="cuda"), torch.tensor(jj, device="cuda"),
                            torch.tensor(xx, device="cuda"), t)
        x_t = torch.zeros_like(b_t)
        s.solve(b_t, x_t)
        assert np.allclose(x_t.cpu().numpy(), x_ref)


def _make(torch, n, vals, idx, cls):
    from cholespy_gb300 import MatrixType
    return cls(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
               torch.tensor(vals, device="cuda"), MatrixType.COO)


def _problems():
    from cholespy_gb300 import workloads
    yield "ico4", (lambda: (2562, *workloads.laplacian_coo(*workloads.icosphere(4)[:2], 2.0)))
    yield "grid64", (lambda: (4096, *workloads.grid2d_coo(64, 10.0, 1.0)))
    yield "grid3d_16", (lambda: (4096, *workloads.grid3d_coo(16, 1e-3)))


PROBLEMS = dict(_problems())


@pytest.mark.parametrize("name", list(PROBLEMS))
def test_levels_bit_exact(cuda, name):
    """GPU analysis == the reference's analysis (oracle restatement of
    kernels.cu:8-60 + cholesky_solver.cpp:349-367) on the same factor."""
    from cholespy_gb300 import CholeskySolverF
    n, vals, idx = PROBLEMS[name]()
    s = _make(cuda, n, vals, idx, CholeskySolverF)
    perm, colptr, rowidx, lv = s.factor()
    lrp, lci, _ = oracle.csr_of_lower(colptr, rowidx, lv)
    for lower, (rp, ci) in ((True, (lrp, lci)), (False, (colptr, rowidx))):
        lev_o, ord_o, mx_o = oracle.levels(rp, ci, lower)
        lev_g, ord_g, mx_g = s.levels(lower)
        np.testing.assert_array_equal(lev_g, lev_o)
        np.testing.assert_array_equal(ord_g, ord_o)
        assert mx_g == mx_o
    info = s.info()
    assert info.levels_lower == oracle.levels(lrp, lci, True)[2] + 1


@pytest.mark.parametrize("name", list(PROBLEMS))
@pytest.mark.parametrize("nrhs", [1, 3, 8, 13, 32, 100, 128])
def test_sweeps_match_oracle(cuda, name, nrhs):
    """FP64 solve == oracle FP64 sweeps (rel 1e-12); FP32 solve within 1e-5
    of the oracle's FP32 sweeps, on the same factor."""
    from cholespy_gb300 import CholeskySolverD, CholeskySolverF
    torch = cuda
    n, vals, idx = PROBLEMS[name]()
    rng = np.random.default_rng(nrhs)
    b = rng.standard_normal((n, nrhs))
    sd = _make(torch, n, vals, idx, CholeskySolverD)
    perm, colptr, rowidx, lv = sd.factor()
    xo = oracle.reference_solve(perm, colptr, rowidx, lv, b, np.float64)
    bt = torch.tensor(b, device="cuda")
    xt = torch.zeros_like(bt)
    sd.solve(bt, xt)
    sd.check()
    err = np.abs(xt.cpu().numpy() - xo).max() / np.abs(xo).max()
    assert err <= 1e-12, err
    sf = _make(torch, n, vals, idx, CholeskySolverF)
    xo32 = oracle.reference_solve(perm, colptr, rowidx, lv, b.astype(np.float32), np.float32)
    bt32 = torch.tensor(b.astype(np.float32), device="cuda")
    xt32 = torch.zeros_like(bt32)
    sf.solve(bt32, xt32)
    sf.check()
    err32 = np.abs(xt32.cpu().numpy().astype(np.float64) - xo32).max() / np.abs(xo32).max()
    assert err32 <= 1e-5, err32


def test_vector_rhs_and_alias(cuda):
    from cholespy_gb300 import CholeskySolverD
    torch = cuda
    n, vals, idx = PROBLEMS["grid64"]()
    s = _make(torch, n, vals, idx, CholeskySolverD)
    A = sym_matrix(n, vals, idx)
    b = np.random.default_rng(0).standard_normal(n)
    bt = torch.tensor(b, device="cuda")
    xt = torch.zeros_like(bt)
    s.solve(bt, xt)
    x = xt.cpu().numpy()
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-12
    # b and x may alias (the lower sweep consumes b before x is written)
    s.solve(bt, bt)
    np.testing.assert_allclose(bt.cpu().numpy(), x, rtol=1e-13, atol=1e-14)


def test_dense_oracle_grid64(cuda):
    """64x64 5-point Laplacian, A = I + 10 L, one N(0,1) RHS (seed 0):
    CholeskySolverD against an FP64 dense solve."""
    from cholespy_gb300 import CholeskySolverD, workloads
    torch = cuda
    n, vals, idx, b = workloads.config_grid64()
    s = _make(torch, n, vals, idx, CholeskySolverD)
    bt = torch.tensor(b, device="cuda")
    xt = torch.zeros_like(bt)
    s.solve(bt, xt)
    xd = np.linalg.solve(sym_matrix(n, vals, idx).toarray(), b)
    rel = np.abs(xt.cpu().numpy() - xd).max() / np.abs(xd).max()
    assert rel < 1e-12, rel


@pytest.mark.parametrize("nrhs", [1, 32, 128])
def test_refined_solve(cuda, nrhs):
    """FP32 factor + FP64 refinement reaches 1e-10 relative residual."""
    from cholespy_gb300 import CholeskySolverD, MatrixType, workloads
    torch = cuda
    n, vals, idx = 4096, *workloads.grid3d_coo(16, 1e-3)
    s = CholeskySolverD(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                        torch.tensor(vals, device="cuda"), MatrixType.COO, refine=True)
    b = np.random.default_rng(2).standard_normal((n, nrhs))
    bt = torch.tensor(b, device="cuda")
    xt = torch.zeros_like(bt)
    st = s.solve_refined(bt, xt, tol=1e-10, max_iter=10)
    assert st.converged and st.max_rel_residual <= 1e-10
    A = sym_matrix(n, vals, idx)
    x = xt.cpu().numpy()
    res = np.linalg.norm(b - A @ x, axis=0) / np.linalg.norm(b, axis=0)
    assert res.max() <= 1e-10
    # agrees with the plain FP64 solve
    x64 = torch.zeros_like(bt)
    s.solve_fp64(bt, x64)
    assert np.abs(x64.cpu().numpy() - x).max() / np.abs(x).max() < 1e-9
    # solve() on a refine=True solver also refines
    x2 = torch.zeros_like(bt)
    s.solve(bt, x2)
    np.testing.assert_allclose(x2.cpu().numpy(), x, rtol=0, atol=1e-12 * np.abs(x).max())


def test_errors(cuda):
    from cholespy_gb300 import CholeskySolverF, MatrixType
    torch = cuda
    n, vals, idx, _ = reference_problem("cube")
    s = _make(torch, n, vals, idx, CholeskySolverF)
    b = torch.zeros(n, 3, device="cuda")
    with pytest.raises(ValueError, match="same dimensions"):
        s.solve(b, torch.zeros(n, 4, device="cuda"))
    with pytest.raises(ValueError, match="Expected 1D or 2D"):
        s.solve(torch.zeros(n, 1, 1, device="cuda"), torch.zeros(n, 1, 1, device="cuda"))
    with pytest.raises(ValueError, match="same device"):
        s.solve(b, torch.zeros(n, 3))
    with pytest.raises(TypeError):
        s.solve(b.double(), torch.zeros(n, 3, device="cuda", dtype=torch.float64))
    with pytest.raises(ValueError, match="positive definite"):
        ii = torch.tensor([0, 1, 1, 0], device="cuda")
        CholeskySolverF(2, ii, torch.tensor([0, 1, 0, 1], device="cuda"),
                        torch.tensor([1.0, 1.0, 3.0, 3.0], dtype=torch.float64, device="cuda"),
                        MatrixType.COO)
    with pytest.raises(ValueError, match="same size"):
        CholeskySolverF(2, torch.tensor([0], device="cuda"), torch.tensor([0, 1], device="cuda"),
                        torch.tensor([1.0, 1.0], dtype=torch.float64, device="cuda"), MatrixType.COO)


def test_side_stream(cuda):
    from cholespy_gb300 import CholeskySolverF
    torch = cuda
    n, vals, idx = PROBLEMS["ico4"]()
    s = _make(torch, n, vals, idx, CholeskySolverF)
    b = torch.rand(n, 16, device="cuda")
    ref = torch.zeros_like(b)
    s.solve(b, ref)
    st = torch.cuda.Stream()
    st.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(st):
        x = torch.zeros_like(b)
        for _ in range(3):
            s.solve(b, x)
    torch.cuda.current_stream().wait_stream(st)
    torch.cuda.synchronize()
    assert torch.equal(x, ref)


def _from_factor(perm, colptr, rowidx, vals, store):
    import ctypes as C
    from cholespy_gb300 import _ffi
    h = C.c_void_p()
    a = [np.ascontiguousarray(v, dt) for v, dt in ((perm, np.int32), (colptr, np.int32),
                                                  (rowidx, np.int32), (vals, np.float64))]
    _ffi.check(_ffi.lib().gbchol_create_from_factor(len(perm), *[x.ctypes.data for x in a], store,
                                                    C.byref(h)))
    return h, a


def _levels_of(h, n, lower):
    import ctypes as C
    from cholespy_gb300 import _ffi
    lev = np.zeros(n, np.int32)
    order = np.zeros(n, np.int32)
    mx = C.c_int32()
    _ffi.check(_ffi.lib().gbchol_get_levels(h, 1 if lower else 0, lev.ctypes.data, order.ctypes.data,
                                            C.byref(mx)))
    return lev, order, mx.value


def test_levels_general_kernel(cuda, monkeypatch):
    """The sync-free level kernel (used when the etree candidates fail the
    check) also matches the oracle bit for bit."""
    from cholespy_gb300 import CholeskySolverF
    monkeypatch.setenv("GBCHOL_SYNCFREE_ANALYSIS", "1")
    n, vals, idx = PROBLEMS["grid3d_16"]()
    s = _make(cuda, n, vals, idx, CholeskySolverF)
    perm, colptr, rowidx, lv = s.factor()
    lrp, lci, _ = oracle.csr_of_lower(colptr, rowidx, lv)
    for lower, (rp, ci) in ((True, (lrp, lci)), (False, (colptr, rowidx))):
        lev_o, ord_o, mx_o = oracle.levels(rp, ci, lower)
        lev_g, ord_g, mx_g = s.levels(lower)
        np.testing.assert_array_equal(lev_g, lev_o)
        np.testing.assert_array_equal(ord_g, ord_o)


def test_levels_pattern_not_fill_closed(cuda):
    """A triangular matrix whose pattern is not closed under fill (entries of
    a true factor dropped): the etree candidates fail the GPU check and the
    general kernel produces the reference's levels; the solve still matches
    the oracle's sweeps on that matrix."""
    from cholespy_gb300 import _ffi
    torch = cuda
    n, vals, idx = PROBLEMS["ico4"]()
    import scipy.sparse as sp
    A = sp.csc_matrix((vals, (idx[0], idx[1])), shape=(n, n))
    A.sum_duplicates()
    perm = np.arange(n, dtype=np.int32)
    Lp, Li, Lx = oracle.cholesky(n, A.indptr, A.indices, A.data, perm)
    # drop every third off-diagonal entry that is not the column's first one
    keep = np.ones(len(Li), bool)
    for j in range(n):
        s, e = Lp[j], Lp[j + 1]
        for k in range(s + 2, e):
            if (k % 3) == 0:
                keep[k] = False
    cnt = np.array([keep[Lp[j]:Lp[j + 1]].sum() for j in range(n)])
    Lp2 = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)
    Li2, Lx2 = Li[keep], Lx[keep]
    h, _keep = _from_factor(perm, Lp2, Li2, Lx2, _ffi.STORE_F64)
    try:
        lrp, lci, _ = oracle.csr_of_lower(Lp2, Li2, Lx2)
        for lower, (rp, ci) in ((True, (lrp, lci)), (False, (Lp2, Li2))):
            lev_o, ord_o, mx_o = oracle.levels(rp, ci, lower)
            lev_g, ord_g, mx_g = _levels_of(h, n, lower)
            np.testing.assert_array_equal(lev_g, lev_o)
            np.testing.assert_array_equal(ord_g, ord_o)
            assert mx_g == mx_o
        b = np.random.default_rng(5).standard_normal((n, 4))
        xo = oracle.reference_solve(perm, Lp2, Li2, Lx2, b, np.float64)
        bt = torch.tensor(b, device="cuda")
        xt = torch.zeros_like(bt)
        import ctypes as C
        st = _ffi.lib().gbchol_solve(h, 1, 4, C.c_void_p(bt.data_ptr()), C.c_void_p(xt.data_ptr()),
                                     C.c_void_p(torch.cuda.current_stream().cuda_stream))
        _ffi.check(st)
        _ffi.check(_ffi.lib().gbchol_check(h))
        err = np.abs(xt.cpu().numpy() - xo).max() / np.abs(xo).max()
        assert err < 1e-12, err
    finally:
        _ffi.lib().gbchol_destroy(h)


@pytest.mark.parametrize("variant", ["float", "double"])
def test_repeated_solves_bit_identical(cuda, variant):
    """Every work item applies its blocks in a fixed order, so repeated solves
    are bit-identical whatever the scheduling; a stale read of a value
    published under a flag would show up as a difference. 3-D 7-point grid
    32^3 (supernodal top region with partial sums), 25 solves per RHS count,
    and the first checked by its residual."""
    from cholespy_gb300 import MatrixType, workloads
    torch = cuda
    k = 32
    vals, idx = workloads.grid3d_coo(k, 1e-3)
    n = k ** 3
    s = _solver_cls(variant)(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                             torch.tensor(vals, device="cuda"), MatrixType.COO)
    dt = torch.float32 if variant == "float" else torch.float64
    rng = np.random.default_rng(11)
    for nrhs in (1, 13, 40):
        b = rng.standard_normal((n, nrhs))
        b_t = torch.tensor(b, dtype=dt, device="cuda")
        x0 = torch.zeros_like(b_t)
        s.solve(b_t, x0)
        x = torch.empty_like(b_t)
        for _ in range(25):
            s.solve(b_t, x)
            assert torch.equal(x, x0)
        s.check()
        A = sym_matrix(n, vals, idx)
        res = np.abs(A @ x0.cpu().numpy().astype(np.float64) - b).max() / np.abs(b).max()
        assert res <= (2e-3 if variant == "float" else 1e-10), res


def test_replan_and_autotune(cuda):
    """gbchol_replan / gbchol_autotune (no reference counterpart): any top-region
    width and partial-sum setting gives the same solution up to rounding; the
    autotuner keeps one of its candidates; a batch built before a replan
    refuses to solve."""
    import cholespy_gb300 as cg
    from cholespy_gb300 import MatrixType, workloads
    torch = cuda
    k = 24
    vals, idx = workloads.grid3d_coo(k, 1e-3)
    n = k ** 3
    s = cg.CholeskySolverF(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                           torch.tensor(vals, device="cuda"), MatrixType.COO)
    rng = np.random.default_rng(5)
    b = rng.standard_normal((n, 20))
    b_t = torch.tensor(b, dtype=torch.float32, device="cuda")
    x_ref = spsolve_ref(n, vals, idx, b)
    scale = np.abs(x_ref).max()
    for width, keep, group in ((8, 16, 32), (1, 16, 32), (4, 2, 3), (16, 0, 0), (10 ** 6, 16, 32)):
        s.replan(width, keep, group)
        x_t = torch.zeros_like(b_t)
        s.solve(b_t, x_t)
        s.check()
        assert np.abs(x_t.cpu().numpy() - x_ref).max() <= 1e-3 * scale, (width, keep, group)
    batch = cg.BatchSolver([s], [20])
    batch.bind([b_t], [torch.zeros_like(b_t)])
    s.replan(8)
    with pytest.raises(RuntimeError):
        batch.solve()
    chosen = s.autotune(20, candidates=(4, 8, 32), reps=2)
    assert chosen in (4, 8, 32)
    x_t = torch.zeros_like(b_t)
    s.solve(b_t, x_t)
    s.check()
    assert np.abs(x_t.cpu().numpy() - x_ref).max() <= 1e-3 * scale


def test_refactorize(cuda):
    """solver.refactorize (no reference counterpart): new values on the same
    pattern solve the new system; a matrix that is not positive definite is
    refused and the old factor kept; a batch built before refuses to solve."""
    import cholespy_gb300 as cg
    from cholespy_gb300 import MatrixType, workloads
    torch = cuda
    k = 16
    v1, idx = workloads.grid3d_coo(k, 1e-3)
    v2, _ = workloads.grid3d_coo(k, 0.5)
    n = k ** 3
    for cls, tol in ((cg.CholeskySolverF, 1e-4), (cg.CholeskySolverD, 1e-10)):
        s = cls(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                torch.tensor(v1, device="cuda"), MatrixType.COO)
        dt = torch.float32 if cls is cg.CholeskySolverF else torch.float64
        b = np.random.default_rng(9).standard_normal((n, 5))
        b_t = torch.tensor(b, dtype=dt, device="cuda")
        batch = cg.BatchSolver([s], [5])
        batch.bind([b_t], [torch.zeros_like(b_t)])
        s.refactorize(idx[0], idx[1], v2, MatrixType.COO)
        x_t = torch.zeros_like(b_t)
        s.solve(b_t, x_t)
        s.check()
        x2 = spsolve_ref(n, v2, idx, b)
        assert np.abs(x_t.cpu().numpy() - x2).max() <= tol * np.abs(x2).max()
        with pytest.raises(ValueError):
            s.refactorize(idx[0], idx[1], -np.asarray(v2), MatrixType.COO)
        x_t.zero_()
        s.solve(b_t, x_t)
        assert np.abs(x_t.cpu().numpy() - x2).max() <= tol * np.abs(x2).max()
        with pytest.raises(RuntimeError):
            batch.solve()


def test_save_load(cuda, tmp_path):
    """solver.save / CholeskySolver*.load (no reference counterpart): the
    reloaded solver holds the same factor and plan, so its solves are
    bit-identical; a file of another format is refused."""
    import cholespy_gb300 as cg
    from cholespy_gb300 import MatrixType
    torch = cuda
    n, vals, idx, b = reference_problem("ico5", dtype=np.float32)
    for cls, dt in ((cg.CholeskySolverF, torch.float32), (cg.CholeskySolverD, torch.float64)):
        s = cls(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                torch.tensor(vals, device="cuda"), MatrixType.COO)
        path = tmp_path / f"{cls.__name__}.npz"
        s.save(path)
        t = cls.load(path)
        b_t = torch.tensor(b[:, :16], dtype=dt, device="cuda")
        x1, x2 = torch.zeros_like(b_t), torch.zeros_like(b_t)
        s.solve(b_t, x1)
        t.solve(b_t, x2)
        t.check()
        assert torch.equal(x1, x2)
    np.savez(tmp_path / "bad.npz", format=np.array("other"), n=np.int64(1))
    with pytest.raises(ValueError):
        cg.CholeskySolverF.load(tmp_path / "bad.npz")


@pytest.mark.parametrize("where", ["one_column", "all_columns", "inf"])
def test_refined_solve_nonfinite_rhs_never_converges(cuda, where):
    """A NaN or Inf in b must leave the refined solve unconverged with a
    non-finite max relative residual (a maximum that dropped NaN would
    report convergence at residual 0)."""
    from cholespy_gb300 import CholeskySolverD, MatrixType, workloads
    torch = cuda
    n, vals, idx = 4096, *workloads.grid3d_coo(16, 1e-3)
    s = CholeskySolverD(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                        torch.tensor(vals, device="cuda"), MatrixType.COO, refine=True)
    b = np.random.default_rng(5).standard_normal((n, 4))
    if where == "one_column":
        b[17, 2] = np.nan
    elif where == "all_columns":
        b[:] = np.nan
    else:
        b[5, 0] = np.inf
    bt = torch.tensor(b, device="cuda")
    xt = torch.zeros_like(bt)
    st = s.solve_refined(bt, xt, tol=1e-10, max_iter=3)
    s.check()
    assert not st.converged
    assert not np.isfinite(st.max_rel_residual)
    assert st.iterations == 3
    # a finite b on the same solver still converges afterwards
    b2 = np.random.default_rng(6).standard_normal((n, 4))
    st2 = s.solve_refined(torch.tensor(b2, device="cuda"), xt, tol=1e-10, max_iter=3)
    assert st2.converged and st2.max_rel_residual <= 1e-10


@pytest.mark.parametrize("name", ["grid3d_16", "ico4"])
@pytest.mark.parametrize("group", ["0", "3"])
@pytest.mark.parametrize("tensor_cores", ["0", "1"])
@pytest.mark.parametrize("fold", ["1", "2"])
def test_bulk_sweeps_match_oracle_and_narrow(cuda, name, group, tensor_cores, fold, monkeypatch):
    """The bulk-copy supernodal sweeps (FP32, 4..128 RHS in multiples of 4:
    one work item per unit holding every RHS column) against the oracle's
    FP32/FP64 sweeps and against the 32-column sweeps of a second solver on
    the same matrix (GBCHOL_BULK_MIN_RHS=129 keeps it on them), both
    shared-memory widths, with and without lower-sweep partial sums
    (GBCHOL_BULK_GROUP), one or two own-supernode blocks folded into the
    diagonal solve (GBCHOL_BULK_FOLD; both matrices have supernodes of more
    than three chunks), plain FP32 and the refined solve's mixed-precision
    sweeps."""
    from cholespy_gb300 import CholeskySolverD, CholeskySolverF, MatrixType
    torch = cuda
    n, vals, idx = PROBLEMS[name]()
    monkeypatch.setenv("GBCHOL_BULK_GROUP", group)
    monkeypatch.setenv("GBCHOL_BULK_KEEP", "2")
    monkeypatch.setenv("GBCHOL_BULK_TC", tensor_cores)
    monkeypatch.setenv("GBCHOL_BULK_MIN_RHS", "4")
    monkeypatch.setenv("GBCHOL_BULK_FOLD", fold)
    s_bulk = _make(torch, n, vals, idx, CholeskySolverF)
    sr = CholeskySolverD(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                         torch.tensor(vals, device="cuda"), MatrixType.COO, refine=True)
    monkeypatch.setenv("GBCHOL_BULK_MIN_RHS", "129")
    s_narrow = _make(torch, n, vals, idx, CholeskySolverF)
    perm, colptr, rowidx, lv = s_bulk.factor()
    for nrhs in (4, 12, 32, 36, 64, 68, 100, 128):
        b = np.random.default_rng(nrhs).standard_normal((n, nrhs))
        bt = torch.tensor(b.astype(np.float32), device="cuda")
        x1, x2 = torch.zeros_like(bt), torch.zeros_like(bt)
        s_bulk.solve(bt, x1)
        s_narrow.solve(bt, x2)
        s_bulk.check()
        s_narrow.check()
        x1h, x2h = x1.cpu().numpy().astype(np.float64), x2.cpu().numpy().astype(np.float64)
        xo64 = oracle.reference_solve(perm, colptr, rowidx, lv, b, np.float64)
        xo32 = oracle.reference_solve(perm, colptr, rowidx, lv, b.astype(np.float32), np.float32)
        scale = np.abs(xo64).max()
        err_b = np.abs(x1h - xo64).max() / scale
        err_o = np.abs(xo32 - xo64).max() / scale
        print(f"TCERR tc={tensor_cores} {name} nrhs={nrhs} err_bulk={err_b:.3e} err_oracle32={err_o:.3e}")
        assert err_b <= 4 * err_o + 1e-6, (nrhs, err_b, err_o)
        assert np.abs(x1h - x2h).max() / scale <= 1e-5
    # refined solve (FP32 sweeps reading FP64 b, adding into FP64 x)
    b = np.random.default_rng(7).standard_normal((n, 128))
    bt = torch.tensor(b, device="cuda")
    xt = torch.zeros_like(bt)
    st = sr.solve_refined(bt, xt, tol=1e-10, max_iter=5)
    assert st.converged
    A = sym_matrix(n, vals, idx)
    res = np.linalg.norm(b - A @ xt.cpu().numpy(), axis=0) / np.linalg.norm(b, axis=0)
    assert res.max() <= 1e-10


@pytest.mark.parametrize("slices", ["2", "4"])
def test_bulk_column_slices_match_oracle(cuda, slices, monkeypatch):
    """The bulk sweeps with the RHS columns cut into 2 or 4 independent
    slices per unit (GBCHOL_BULK_SLICES; RHS counts that do not split into
    multiples of 4 keep one slice) against the oracle's FP32 sweeps and the
    single-slice bulk sweeps of a second solver, plain FP32 and refined."""
    from cholespy_gb300 import CholeskySolverD, CholeskySolverF, MatrixType
    torch = cuda
    n, vals, idx = PROBLEMS["grid3d_16"]()
    monkeypatch.setenv("GBCHOL_BULK_MIN_RHS", "4")
    monkeypatch.setenv("GBCHOL_BULK_SLICES", slices)
    s_sl = _make(torch, n, vals, idx, CholeskySolverF)
    sr = CholeskySolverD(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                         torch.tensor(vals, device="cuda"), MatrixType.COO, refine=True)
    monkeypatch.setenv("GBCHOL_BULK_SLICES", "1")
    s_one = _make(torch, n, vals, idx, CholeskySolverF)
    perm, colptr, rowidx, lv = s_sl.factor()
    for nrhs in (8, 16, 24, 64, 100, 128):
        b = np.random.default_rng(nrhs).standard_normal((n, nrhs)).astype(np.float32)
        bt = torch.tensor(b, device="cuda")
        x1, x2 = torch.zeros_like(bt), torch.zeros_like(bt)
        s_sl.solve(bt, x1)
        s_one.solve(bt, x2)
        s_sl.check()
        s_one.check()
        xo = oracle.reference_solve(perm, colptr, rowidx, lv, b, np.float32)
        scale = np.abs(xo).max()
        assert np.abs(x1.cpu().numpy() - xo).max() / scale <= 1e-5, nrhs
        assert np.abs(x1.cpu().numpy() - x2.cpu().numpy()).max() / scale <= 1e-5, nrhs
    b = np.random.default_rng(9).standard_normal((n, 128))
    bt = torch.tensor(b, device="cuda")
    xt = torch.zeros_like(bt)
    st = sr.solve_refined(bt, xt, tol=1e-10, max_iter=5)
    assert st.converged
    A = sym_matrix(n, vals, idx)
    res = np.linalg.norm(b - A @ xt.cpu().numpy(), axis=0) / np.linalg.norm(b, axis=0)
    assert res.max() <= 1e-10


@pytest.mark.parametrize("case", STRUCTURES)
def test_structures_match_spsolve(cuda, case):
    """The GPU solves on unusual elimination structures (a forest of 40
    grids, a star, a diagonal matrix, a 1 x 1 system, one dense 96 x 96
    supernode) against spsolve: FP32 within 1e-4 and FP64 within 1e-10 of
    max |x| (condition numbers below 100), at RHS counts of the row sweeps
    (1, 3) and of the bulk sweeps (12, 128), and the refined solve to a
    1e-10 relative residual."""
    from scipy.sparse.linalg import spsolve
    from cholespy_gb300 import CholeskySolverD, CholeskySolverF, MatrixType
    torch = cuda
    A = structural_cases()[case]
    n = A.shape[0]
    args = (torch.tensor(A.row, device="cuda"), torch.tensor(A.col, device="cuda"),
            torch.tensor(A.data, device="cuda"), MatrixType.COO)
    sf = CholeskySolverF(n, *args)
    sd = CholeskySolverD(n, *args, refine=True)
    rng = np.random.default_rng(len(case))
    for nrhs in (1, 3, 12, 128):
        b = rng.standard_normal((n, nrhs))
        xr = spsolve(A.tocsc(), b).reshape(b.shape)
        scale = np.abs(xr).max()
        xf = torch.zeros((n, nrhs), device="cuda")
        sf.solve(torch.tensor(b.astype(np.float32), device="cuda"), xf)
        bd = torch.tensor(b, device="cuda")
        xd = torch.zeros_like(bd)
        sd.solve_fp64(bd, xd)
        sf.check()
        sd.check()
        assert np.abs(xf.cpu().numpy() - xr).max() <= 1e-4 * scale, nrhs
        assert np.abs(xd.cpu().numpy() - xr).max() <= 1e-10 * scale, nrhs
        xt = torch.zeros_like(bd)
        st = sd.solve_refined(bd, xt, tol=1e-10, max_iter=5)
        assert st.converged, nrhs
        res = np.linalg.norm(b - A.tocsr() @ xt.cpu().numpy(), axis=0) / np.linalg.norm(b, axis=0)
        assert res.max() <= 1e-10, nrhs


@pytest.mark.parametrize("nrhs", [4, 64])
def test_autotune_sweeps(cuda, nrhs):
    """gbchol_autotune_sweeps times every sweep variant for an RHS count
    (top-region kernel, row-sweep lane mode, rows per ticket), keeps the
    fastest, and solves with it afterwards: results still match the oracle
    (FP32 within 1e-5 relative to max |x|)."""
    from cholespy_gb300 import CholeskySolverF
    torch = cuda
    n, vals, idx = PROBLEMS["grid3d_16"]()
    s = _make(torch, n, vals, idx, CholeskySolverF)
    choice = s.autotune_sweeps(nrhs, reps=2)
    assert choice["kernel"] in ("sliced", "bulk", "bulk_tc", "bulk_2slices", "bulk_4slices")
    assert choice["rows_per_ticket"] in (1, 2, 4)
    assert choice["rhs_split"] in ((False, True) if nrhs <= 8 else (False,))
    perm, colptr, rowidx, lv = s.factor()
    b = np.random.default_rng(nrhs).standard_normal((n, nrhs)).astype(np.float32)
    bt = torch.tensor(b, device="cuda")
    xt = torch.zeros_like(bt)
    s.solve(bt, xt)
    s.check()
    xo = oracle.reference_solve(perm, colptr, rowidx, lv, b, np.float32)
    assert np.abs(xt.cpu().numpy() - xo).max() / np.abs(xo).max() <= 1e-5
