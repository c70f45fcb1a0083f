"""GPU parity on the benchmark configurations themselves, against the oracle.

Each configuration is built with the same generator and seed the benchmark
uses (cholespy_gb300/workloads.py):
  * icosphere 6 (n = 40 962), A = I + 19 L, CSC input, FP32, 3 RHS (seed 1):
    the GPU solve against the oracle's restatement of the reference's sweeps
    (kernels/kernels.cu:64-202) on the same factor, levels bit-exact;
  * 3-D 7-point Poisson on 64^3 (n = 262 144), shift 1e-3, N(0,1) RHS
    (seed 2), 1 / 32 / 128 RHS: the FP32 and FP64 solves against the
    oracle's FP32 / FP64 sweeps on the same factor, on columns taken from
    every 32-wide RHS slice, and the FP32 + FP64 refinement to 1e-10 relative
    residual on every column (host FP64 residual on the original A);
  * the first 24 systems of the 256-system batch (seed 3): the batched solve
    against per-system oracle sweeps;
  * icosphere 7 (n = 163 842) with edge weights U[0.5, 2] (seed 4), 3 RHS:
    the FP32 and FP64 gradients on A's stored entries against the gradient
    built from the oracle's FP64 solve, and against FP64 central differences
    (h = 1e-6) on 64 random edge weights.

Tolerances, stated per test: FP64 results within 1e-12 (max-norm, relative
to max |x|) of the oracle's FP64 sweeps; FP32 results within 1e-5 relative
residual (the parity bar for CholeskySolverF) and no less accurate than the
oracle's own FP32 sweeps (error against the FP64 oracle at most 4x the
oracle FP32 sweeps' error, plus 1e-6 of max |x|); refined FP32 within 1e-10
relative residual."""
import numpy as np
import pytest

import oracle
from helpers import sym_matrix

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / np.abs(b).max())


def _residual(A, x, b):
    return float((np.linalg.norm(b - A @ x, axis=0) / np.linalg.norm(b, axis=0)).max())


class _OracleSweeps:
    """The oracle's restatement of the reference's analysis + sweeps on one
    factor, with the CSR of L and both level orders computed once."""

    def __init__(self, perm, colptr, rowidx, lv):
        self.perm, self.colptr, self.rowidx, self.lv = perm, colptr, rowidx, lv
        self.lrp, self.lci, self.lval = oracle.csr_of_lower(colptr, rowidx, lv)
        self.ord_l = oracle.levels(self.lrp, self.lci, True)[1]
        self.ord_u = oracle.levels(colptr, rowidx, False)[1]

    def solve(self, b, dtype):
        b2 = np.ascontiguousarray(b, dtype=dtype)
        tmp = oracle.solve_lower(self.lrp, self.lci, self.lval.astype(dtype), self.ord_l, self.perm, b2)
        return oracle.solve_upper(self.colptr, self.rowidx, np.asarray(self.lv).astype(dtype), self.ord_u,
                                  self.perm, tmp)[1]


def _fp32_ok(x_gpu, xo32, xo64):
    """FP32 GPU result no less accurate than the oracle's FP32 sweeps."""
    err_g = _rel(x_gpu, xo64)
    err_o = _rel(xo32, xo64)
    assert err_g <= 4.0 * err_o + 1e-6, (err_g, err_o)
    return err_g, err_o


def test_config_icosphere6_f32(cuda):
    from cholespy_gb300 import CholeskySolverF, MatrixType, workloads
    torch = cuda
    n, vals, idx, b = workloads.config_icosphere6()
    colptr, rowidx, cvals = workloads.to_csc(n, vals, idx)
    s = CholeskySolverF(n, torch.tensor(colptr, device="cuda"), torch.tensor(rowidx, device="cuda"),
                        torch.tensor(cvals, device="cuda"), MatrixType.CSC)
    bt = torch.tensor(b.astype(np.float32), device="cuda")
    xt = torch.zeros_like(bt)
    s.solve(bt, xt)
    s.check()
    x = xt.cpu().numpy()
    perm, Lp, Li, Lx = s.factor()
    o = _OracleSweeps(perm, Lp, Li, Lx)
    xo64 = o.solve(b, np.float64)
    xo32 = o.solve(b, np.float32)
    _fp32_ok(x, xo32, xo64)
    assert _residual(sym_matrix(n, vals, idx), x.astype(np.float64), b) <= 1e-5
    for lower, (rp, ci) in ((True, (o.lrp, o.lci)), (False, (Lp, Li))):
        lev_o, ord_o, mx_o = oracle.levels(rp, ci, lower)
        lev_g, ord_g, mx_g = s.levels(lower)
        np.testing.assert_array_equal(lev_g, lev_o)
        np.testing.assert_array_equal(ord_g, ord_o)
        assert mx_g == mx_o


@pytest.fixture(scope="module")
def poisson64(cuda):
    """The 64^3 solver (FP32 and FP64 factors + FP64 A), its oracle, and the
    oracle's FP32/FP64 answers on one column of every 32-wide RHS slice."""
    from cholespy_gb300 import CholeskySolverD, MatrixType, workloads
    torch = cuda
    n, vals, idx, b = workloads.config_poisson64()
    s = CholeskySolverD(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                        torch.tensor(vals, device="cuda"), MatrixType.COO, refine=True)
    o = _OracleSweeps(*s.factor())
    cols = np.array([0, 31, 32, 63, 64, 95, 127])
    bs = np.ascontiguousarray(b[:, cols])
    return {"n": n, "b": b, "A": sym_matrix(n, vals, idx), "solver": s, "cols": cols,
            "xo64": o.solve(bs, np.float64), "xo32": o.solve(bs, np.float32)}


@pytest.mark.parametrize("nrhs", [1, 32, 128])
def test_config_poisson64(cuda, poisson64, nrhs):
    import ctypes as C

    from cholespy_gb300 import _ffi
    torch = cuda
    P = poisson64
    s, b, A = P["solver"], P["b"][:, :nrhs], P["A"]
    sel = np.nonzero(P["cols"] < nrhs)[0]
    cols = P["cols"][sel]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    # FP32 sweeps (the refined solve's inner solve), through the C ABI
    b32 = torch.tensor(b.astype(np.float32), device="cuda")
    x32 = torch.zeros_like(b32)
    _ffi.check(_ffi.lib().gbchol_solve(s.handle, 0, nrhs, C.c_void_p(b32.data_ptr()),
                                       C.c_void_p(x32.data_ptr()), stream))
    # plain FP64 solve
    bt = torch.tensor(b, device="cuda")
    x64 = torch.zeros_like(bt)
    s.solve_fp64(bt, x64)
    # FP32 + FP64 refinement
    xir = torch.zeros_like(bt)
    st = s.solve_refined(bt, xir, tol=1e-10, max_iter=5)
    s.check()
    x32h, x64h, xirh = x32.cpu().numpy(), x64.cpu().numpy(), xir.cpu().numpy()
    assert _rel(x64h[:, cols], P["xo64"][:, sel]) <= 1e-12
    _fp32_ok(x32h[:, cols], P["xo32"][:, sel], P["xo64"][:, sel])
    assert _residual(A, x32h.astype(np.float64), b) <= 1e-5
    assert st.converged and st.max_rel_residual <= 1e-10
    assert _residual(A, xirh, b) <= 1e-10
    assert _rel(xirh[:, cols], P["xo64"][:, sel]) <= 1e-9


def test_config_batch_slice(cuda):
    """The first 24 systems of the 256-system benchmark batch (same draws:
    each system's size, lambda, RHS count and RHS come in order from seed 3)."""
    from cholespy_gb300 import BatchSolver, CholeskySolverF, MatrixType, workloads
    torch = cuda
    systems = workloads.config_batch(count=24)
    solvers, bs, xs = [], [], []
    for n, vals, idx, b in systems:
        solvers.append(CholeskySolverF(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                                       torch.tensor(vals, device="cuda"), MatrixType.COO))
        bs.append(torch.tensor(b.astype(np.float32), device="cuda"))
        xs.append(torch.zeros_like(bs[-1]))
    batch = BatchSolver(solvers, [b.shape[1] for b in bs])
    batch.solve(bs, xs)
    batch.check()
    for (n, vals, idx, b), s, x in zip(systems, solvers, xs):
        o = _OracleSweeps(*s.factor())
        xh = x.cpu().numpy()
        _fp32_ok(xh, o.solve(b, np.float32), o.solve(b, np.float64))
        assert _residual(sym_matrix(n, vals, idx), xh.astype(np.float64), b) <= 1e-5


def test_config_autograd_icosphere7(cuda):
    """Loss = sum(w * x), x = A^{-1} b, A = I + 19 L_w: gradients on A's
    stored entries (FP32 and FP64 solvers) against the oracle-built FP64
    gradient, and the edge-weight gradient against FP64 central differences
    (h = 1e-6) on 64 random edges, each difference from two FP64 solves of
    the refactorised solver (same ordering and pattern)."""
    from cholespy_gb300 import CholeskySolverD, MatrixType, workloads
    from cholespy_gb300.autograd import DifferentiableSolver
    torch = cuda
    lam = 19.0
    n, faces, pos = workloads.icosphere(7)
    rng = np.random.default_rng(4)
    edges = workloads.mesh_edges(faces)
    w = rng.uniform(0.5, 2.0, size=len(edges))
    _, idx = workloads.laplacian_coo(n, faces, lam, weights=w)
    wl = rng.standard_normal((n, 3))
    ne = len(edges)

    def values(wv):
        # laplacian_coo's entry order: off-diagonals (i, j) then (j, i), the
        # diagonal terms lam * w of both ends of every edge, then the identity
        off = lam * np.asarray(wv)
        return np.concatenate([-off, -off, off, off, np.ones(n)])

    def edge_grad(g):
        # d loss / d w_e from the entry gradients (chain rule through values())
        return lam * (-g[:ne] - g[ne:2 * ne] + g[2 * ne:3 * ne] + g[3 * ne:4 * ne])

    v0 = values(w)
    np.testing.assert_array_equal(v0, workloads.laplacian_coo(n, faces, lam, weights=w)[0])
    ii, jj = torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda")
    grads = {}
    for prec, dt in (("float", torch.float32), ("double", torch.float64)):
        vt = torch.tensor(v0, device="cuda", requires_grad=True)
        ds = DifferentiableSolver(n, ii, jj, vt, MatrixType.COO, precision=prec)
        x = ds(torch.tensor(pos, device="cuda", dtype=dt))
        (torch.tensor(wl, device="cuda", dtype=dt) * x).sum().backward()
        grads[prec] = vt.grad.cpu().numpy()
        if prec == "double":
            perm, Lp, Li, Lx = ds.solver.factor()
    o = _OracleSweeps(perm, Lp, Li, Lx)
    xo = o.solve(pos, np.float64)
    gbo = o.solve(wl, np.float64)
    r, c = idx[0], idx[1]
    go = -(gbo[r] * xo[c]).sum(1) - np.where(r != c, (gbo[c] * xo[r]).sum(1), 0.0)
    go = np.where(r != c, 0.5 * go, go)
    scale = np.abs(go).max()
    np.testing.assert_allclose(grads["double"], go, rtol=1e-9, atol=1e-12 * scale)
    assert np.abs(grads["float"] - go).max() <= 1e-4 * scale

    # central differences of the edge-weight gradient
    sd = CholeskySolverD(n, ii, jj, torch.tensor(v0, device="cuda"), MatrixType.COO)
    bt = torch.tensor(pos, device="cuda")
    xt = torch.zeros_like(bt)

    def loss_at(wv):
        sd.refactorize(idx[0], idx[1], values(wv), MatrixType.COO)
        sd.solve(bt, xt)
        return float((xt.cpu().numpy() * wl).sum())

    ge64, ge32 = edge_grad(grads["double"]), edge_grad(grads["float"])
    h = 1e-6
    for e in np.random.default_rng(4).choice(ne, size=64, replace=False):
        wp, wm = w.copy(), w.copy()
        wp[e] += h
        wm[e] -= h
        fd = (loss_at(wp) - loss_at(wm)) / (2 * h)
        assert abs(ge64[e] - fd) <= 1e-5 * max(1.0, abs(fd)), (e, ge64[e], fd)
        assert abs(ge32[e] - fd) <= 1e-3 * max(1.0, abs(fd)), (e, ge32[e], fd)
