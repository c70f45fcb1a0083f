"""GPU tests of the differentiable solve: backward solve on the same factor
and the sparse gradient kernel on A's stored entries, checked in FP64
against central finite differences (h = 1e-6, 64 random edge weights) and
against the gradient built from the oracle's FP64 solve (restating the
reference's double-precision sweeps) on the same factor."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

LAM = 19.0


def _weighted_problem(level, seed):
    from cholespy_gb300 import workloads
    n, faces, pos = workloads.icosphere(level)
    rng = np.random.default_rng(seed)
    edges = workloads.mesh_edges(faces)
    w = rng.uniform(0.5, 2.0, size=len(edges))
    _, idx = workloads.laplacian_coo(n, faces, LAM, weights=w)
    wl = rng.standard_normal((n, 3))
    return n, edges, w, idx, pos, wl


def _values_from_weights(torch, w, n):
    """Differentiable COO values of A = I + LAM * L_w in the order of
    workloads.laplacian_coo: off-diagonals (i,j), (j,i); duplicate diagonals."""
    ww = torch.cat([w, w]) * LAM
    return torch.cat([-ww, ww, torch.ones(n, dtype=w.dtype, device=w.device)])


def _loss(torch, n, idx, w_t, b_t, wl_t, precision="double", symmetric=True):
    from cholespy_gb300 import MatrixType
    from cholespy_gb300.autograd import DifferentiableSolver
    vals = _values_from_weights(torch, w_t, n)
    ds = DifferentiableSolver(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                              vals, MatrixType.COO, precision=precision, symmetric=symmetric)
    x = ds(b_t)
    return (wl_t * x).sum(), ds, x


def test_gradient_vs_finite_differences(cuda):
    torch = cuda
    n, edges, w, idx, pos, wl = _weighted_problem(4, 4)
    w_t = torch.tensor(w, device="cuda", requires_grad=True)
    b_t = torch.tensor(pos, device="cuda", requires_grad=True)
    wl_t = torch.tensor(wl, device="cuda")
    loss, _, _ = _loss(torch, n, idx, w_t, b_t, wl_t)
    loss.backward()
    g = w_t.grad.cpu().numpy()
    rng = np.random.default_rng(4)
    picks = rng.choice(len(w), size=64, replace=False)
    h = 1e-6
    for e in picks:
        wp, wm = w.copy(), w.copy()
        wp[e] += h
        wm[e] -= h
        lp = _loss(torch, n, idx, torch.tensor(wp, device="cuda"), b_t.detach(), wl_t)[0].item()
        lm = _loss(torch, n, idx, torch.tensor(wm, device="cuda"), b_t.detach(), wl_t)[0].item()
        fd = (lp - lm) / (2 * h)
        assert abs(g[e] - fd) <= 1e-5 * max(1.0, abs(fd)), (e, g[e], fd)
    # grad_b = A^{-1} wl
    gb = b_t.grad.cpu().numpy()
    import scipy.sparse as sp
    vals = _values_from_weights(torch, torch.tensor(w), n).numpy()
    A = sp.csc_matrix((vals, (idx[0], idx[1])), shape=(n, n))
    np.testing.assert_allclose(A @ gb, wl, rtol=1e-9, atol=1e-9)


def test_gradient_vs_oracle_double_solve(cuda):
    """Entry gradients equal the formula evaluated with the oracle's FP64
    restatement of the reference's sweeps on the same factor."""
    from cholespy_gb300 import CholeskySolverD
    torch = cuda
    n, edges, w, idx, pos, wl = _weighted_problem(5, 7)
    vals = _values_from_weights(torch, torch.tensor(w, device="cuda"), n).detach().requires_grad_(True)
    from cholespy_gb300 import MatrixType
    from cholespy_gb300.autograd import DifferentiableSolver
    ds = DifferentiableSolver(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                              vals, MatrixType.COO, precision="double")
    b_t = torch.tensor(pos, device="cuda")
    x = ds(b_t)
    (torch.tensor(wl, device="cuda") * x).sum().backward()
    g = vals.grad.cpu().numpy()
    perm, colptr, rowidx, lv = ds.solver.factor()
    xo = oracle.reference_solve(perm, colptr, rowidx, lv, pos, np.float64)
    gbo = oracle.reference_solve(perm, colptr, rowidx, lv, wl, np.float64)
    r, c = idx[0], idx[1]
    go = -(gbo[r] * xo[c]).sum(1) - np.where(r != c, (gbo[c] * xo[r]).sum(1), 0.0)
    go = np.where(r != c, 0.5 * go, go)
    np.testing.assert_allclose(g, go, rtol=1e-9, atol=1e-12 * np.abs(go).max())


def test_gradient_lower_mode_single_entries(cuda):
    """symmetric=False is the exact derivative of the lower-triangle forward:
    perturbing one stored entry below the diagonal matches central
    differences; entries above the diagonal get exactly 0."""
    from cholespy_gb300 import MatrixType
    from cholespy_gb300.autograd import DifferentiableSolver
    torch = cuda
    n, edges, w, idx, pos, wl = _weighted_problem(3, 11)
    base = _values_from_weights(torch, torch.tensor(w), n).numpy()
    vals = torch.tensor(base, device="cuda", requires_grad=True)
    ii, jj = torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda")
    b_t = torch.tensor(pos, device="cuda")
    wl_t = torch.tensor(wl, device="cuda")
    ds = DifferentiableSolver(n, ii, jj, vals, MatrixType.COO, precision="double", symmetric=False)
    (wl_t * ds(b_t)).sum().backward()
    g = vals.grad.cpu().numpy()
    assert np.all(g[idx[0] < idx[1]] == 0.0)

    def loss_at(v):
        d = DifferentiableSolver(n, ii, jj, torch.tensor(v, device="cuda"), MatrixType.COO,
                                 precision="double", symmetric=False)
        return (wl_t * d(b_t)).sum().item()

    rng = np.random.default_rng(0)
    lower = np.nonzero(idx[0] > idx[1])[0]
    for e in rng.choice(lower, size=16, replace=False):
        vp, vm = base.copy(), base.copy()
        vp[e] += 1e-6
        vm[e] -= 1e-6
        fd = (loss_at(vp) - loss_at(vm)) / 2e-6
        assert abs(g[e] - fd) <= 1e-5 * max(1.0, abs(fd)), (e, g[e], fd)


def test_gradient_float_solver(cuda):
    """The FP32 solver's gradients stay within 1e-4 of the FP64 ones."""
    torch = cuda
    n, edges, w, idx, pos, wl = _weighted_problem(4, 9)
    grads = []
    for prec, dt in (("float", torch.float32), ("double", torch.float64)):
        w_t = torch.tensor(w, device="cuda", requires_grad=True)
        loss, _, _ = _loss(torch, n, idx, w_t, torch.tensor(pos, device="cuda", dtype=dt),
                           torch.tensor(wl, device="cuda", dtype=dt), precision=prec)
        loss.backward()
        grads.append(w_t.grad.cpu().numpy())
    err = np.abs(grads[0] - grads[1]).max() / np.abs(grads[1]).max()
    assert err < 1e-4, err
