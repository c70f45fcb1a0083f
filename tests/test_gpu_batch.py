"""GPU tests of the batched solve: systems of uneven sizes and RHS counts in
one persistent launch per phase, against the individual solves and the
oracle, bound once and replayed from a captured CUDA graph."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _systems(torch, cls, seed, count):
    from cholespy_gb300 import MatrixType, workloads
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        side = int(rng.integers(6, 48))
        lam = float(rng.uniform(1, 50))
        r = int(rng.choice([1, 2, 3, 7, 8, 9, 16, 31, 33, 64, 100, 128]))
        vals, idx = workloads.grid2d_coo(side, lam, 1.0)
        n = side * side
        s = cls(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                torch.tensor(vals, device="cuda"), MatrixType.COO)
        out.append((s, n, r))
    return out


# row-sweep schedules: the library default (8 MB groups, skew 4, fitted lane
# modes), a wavefront over groups of about one system, groups one after
# another with the two-mode variant, and one group
SCHEDULES = {"default": {}, "wavefront": {"group_mb": 0.25, "skew": 2, "row_variant": 2},
             "sequential": {"group_mb": 0.1, "skew": 0, "row_variant": 1},
             "one_group": {"group_mb": 0, "skew": 0, "row_variant": 2}}


@pytest.mark.parametrize("variant", ["float", "double"])
@pytest.mark.parametrize("schedule", list(SCHEDULES))
def test_batch_matches_single_and_oracle(cuda, variant, schedule):
    from cholespy_gb300 import BatchSolver, CholeskySolverD, CholeskySolverF
    torch = cuda
    cls = CholeskySolverF if variant == "float" else CholeskySolverD
    dt = torch.float32 if variant == "float" else torch.float64
    tol = 1e-5 if variant == "float" else 1e-12
    systems = _systems(torch, cls, 3, 12)
    bs = [torch.randn(n, r, device="cuda", dtype=dt) for _, n, r in systems]
    xs = [torch.zeros_like(b) for b in bs]
    batch = BatchSolver([s for s, _, _ in systems], [r for _, _, r in systems], **SCHEDULES[schedule])
    batch.solve(bs, xs)
    batch.check()
    for (s, n, r), b, x in zip(systems, bs, xs):
        x1 = torch.zeros_like(b)
        s.solve(b, x1)
        err = ((x - x1).abs().max() / x1.abs().max()).item()
        assert err <= tol, err
        perm, colptr, rowidx, lv = s.factor()
        npdt = np.float32 if variant == "float" else np.float64
        xo = oracle.reference_solve(perm, colptr, rowidx, lv, b.cpu().numpy(), npdt)
        erro = np.abs(x.cpu().numpy() - xo).max() / np.abs(xo).max()
        assert erro <= tol, erro
    assert batch.info()["launches"] <= 4  # one per phase: lower rows, lower and upper supernodal, upper rows


def test_batch_graph_replay(cuda):
    from cholespy_gb300 import BatchSolver, CholeskySolverF
    torch = cuda
    systems = _systems(torch, CholeskySolverF, 7, 9)
    bs = [torch.randn(n, r, device="cuda") for _, n, r in systems]
    xs = [torch.zeros_like(b) for b in bs]
    batch = BatchSolver([s for s, _, _ in systems], [r for _, _, r in systems])
    g = batch.capture(bs, xs)
    ref = [x.clone() for x in xs]
    for _ in range(3):
        for x in xs:
            x.zero_()
        for b in bs:
            b.mul_(2.0)
        g.replay()
        torch.cuda.synchronize()
        for i, x in enumerate(xs):
            ref[i] = ref[i] * 2.0
            err = ((x - ref[i]).abs().max() / ref[i].abs().max()).item()
            assert err < 1e-5, err
    batch.check()


def test_single_solve_graph_replay(cuda):
    """Single solves are graph-capturable too (device-resident epochs)."""
    from cholespy_gb300 import CholeskySolverF, MatrixType, workloads
    torch = cuda
    n, vals, idx = 4096, *workloads.grid3d_coo(16, 1e-3)
    s = CholeskySolverF(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                        torch.tensor(vals, device="cuda"), MatrixType.COO)
    s.reserve(32)
    b = torch.randn(n, 32, device="cuda")
    x = torch.zeros_like(b)
    s.solve(b, x)
    ref = x.clone()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        s.solve(b, x)
    for _ in range(3):
        x.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(x, ref)
    s.check()


def test_batch_tune(cuda):
    """BatchSolver.tune: the batch autotuner picks one of the candidate
    top-region widths and wavefront skews, replans every solver with the
    width and returns a batch that solves like the individual (replanned)
    solvers."""
    from cholespy_gb300 import BatchSolver, CholeskySolverF
    torch = cuda
    systems = _systems(torch, CholeskySolverF, 11, 6)
    solvers = [s for s, _, _ in systems]
    width, batch = BatchSolver.tune(solvers, [r for _, _, r in systems], candidates=(4, 16), reps=2,
                                    skews=(0, 3), group_mb=0.05)
    assert width in (4, 16)
    assert batch.schedule["skew"] in (0, 3)
    bs = [torch.randn(n, r, device="cuda") for _, n, r in systems]
    xs = [torch.zeros_like(b) for b in bs]
    batch.solve(bs, xs)
    batch.check()
    for (s, n, r), b, x in zip(systems, bs, xs):
        x1 = torch.zeros_like(b)
        s.solve(b, x1)
        err = ((x - x1).abs().max() / x1.abs().max()).item()
        assert err <= 1e-5, err


def test_batch_options_rejected(cuda):
    """Invalid schedules are refused with ValueError (the C ABI's EINVAL)."""
    from cholespy_gb300 import BatchSolver, CholeskySolverF
    torch = cuda
    systems = _systems(torch, CholeskySolverF, 5, 2)
    solvers, nrhs = [s for s, _, _ in systems], [r for _, _, r in systems]
    with pytest.raises(ValueError):
        BatchSolver(solvers, nrhs, skew=-1)
    with pytest.raises(ValueError):
        BatchSolver(solvers, nrhs, row_variant=3)
