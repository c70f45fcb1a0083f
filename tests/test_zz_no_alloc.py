"""GPU test of gbchol_solve_noalloc, the solve entry point for callers that
cannot allocate GPU memory while solving (real-time loops whose device
memory is fixed up front, hosts whose allocator owns the device). Its work array is a fixed static device array instead of memory
the solver allocates. Called through the C ABI, two calls in a row, each
checked against gbchol_solve on the same inputs within the solve tests'
tolerance (1e-5 relative for FP32, 1e-12 for FP64). This file sorts last so
that a run stopping at its first failure has run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solver(torch, cls):
    from cholespy_gb300 import MatrixType, workloads
    n, vals, idx = 4096, *workloads.grid3d_coo(16, 1e-3)
    return cls(n, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
               torch.tensor(vals, device="cuda"), MatrixType.COO), n


@pytest.mark.parametrize("variant", ["float", "double"])
def test_solve_noalloc_matches_solve(cuda, variant):
    from cholespy_gb300 import CholeskySolverD, CholeskySolverF, _ffi
    torch = cuda
    cls = CholeskySolverF if variant == "float" else CholeskySolverD
    dt = torch.float32 if variant == "float" else torch.float64
    prec = 0 if variant == "float" else 1
    tol = 1e-5 if variant == "float" else 1e-12
    s, n = _solver(torch, cls)
    lib = _ffi.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for nrhs in (3, 64):  # two calls in a row, the second larger than the first
        b = torch.randn(n, nrhs, device="cuda", dtype=dt)
        x_ref = torch.zeros_like(b)
        _ffi.check(lib.gbchol_solve(s.handle, prec, nrhs, C.c_void_p(b.data_ptr()),
                                    C.c_void_p(x_ref.data_ptr()), stream))
        x = torch.zeros_like(b)
        _ffi.check(lib.gbchol_solve_noalloc(s.handle, prec, nrhs, C.c_void_p(b.data_ptr()),
                                            C.c_void_p(x.data_ptr()), stream))
        torch.cuda.synchronize()
        _ffi.check(lib.gbchol_check(s.handle))
        err = ((x - x_ref).abs().max() / x_ref.abs().max()).item()
        assert err <= tol, err


def test_solve_noalloc_rejects_oversize(cuda):
    """A work array above the 16 MiB limit is refused with a clear error
    (65 536 rows x 64 RHS x 8 bytes = 32 MiB) before any GPU work."""
    from cholespy_gb300 import CholeskySolverD, MatrixType, _ffi, workloads
    torch = cuda
    vals, idx = workloads.grid2d_coo(256, 10.0, 1.0)
    s = CholeskySolverD(256 * 256, torch.tensor(idx[0], device="cuda"), torch.tensor(idx[1], device="cuda"),
                        torch.tensor(vals, device="cuda"), MatrixType.COO)
    b = torch.zeros(256 * 256, 64, device="cuda", dtype=torch.float64)
    st = _ffi.lib().gbchol_solve_noalloc(s.handle, 1, 64, C.c_void_p(b.data_ptr()),
                                         C.c_void_p(b.data_ptr()), None)
    assert st == _ffi.EINVAL
    assert "16 MiB" in _ffi.last_error()


def test_solve_noalloc_leaves_free_memory_unchanged(cuda):
    """A steady-state call allocates no device memory: the driver's free
    memory is the same before and after it (the first call with these
    shapes, which may load kernel code lazily, is made before measuring)."""
    from cholespy_gb300 import CholeskySolverF, _ffi
    torch = cuda
    s, n = _solver(torch, CholeskySolverF)
    lib = _ffi.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    b = torch.randn(n, 96, device="cuda")
    x = torch.zeros_like(b)

    def call():
        _ffi.check(lib.gbchol_solve_noalloc(s.handle, 0, 96, C.c_void_p(b.data_ptr()),
                                            C.c_void_p(x.data_ptr()), stream))
        torch.cuda.synchronize()

    call()
    free0 = torch.cuda.mem_get_info()[0]
    call()
    free1 = torch.cuda.mem_get_info()[0]
    _ffi.check(lib.gbchol_check(s.handle))
    assert free1 == free0, (free0, free1)


def test_solve_noalloc_replays_in_a_cuda_graph(cuda):
    """After a first call outside capture (which looks up the static work
    array's device address), a gbchol_solve_noalloc call can be captured in
    a CUDA graph: each replay, with b rewritten in place in between, matches
    gbchol_solve on the same b."""
    from cholespy_gb300 import CholeskySolverF, _ffi
    torch = cuda
    s, n = _solver(torch, CholeskySolverF)
    lib = _ffi.lib()
    nrhs = 16
    b = torch.randn(n, nrhs, device="cuda")
    x = torch.zeros_like(b)

    def call(out):
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        _ffi.check(lib.gbchol_solve_noalloc(s.handle, 0, nrhs, C.c_void_p(b.data_ptr()),
                                            C.c_void_p(out.data_ptr()), stream))

    call(x)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        call(x)
    for seed in range(2):
        gen = torch.Generator(device="cuda").manual_seed(seed)
        b.copy_(torch.randn(n, nrhs, device="cuda", generator=gen))
        x.zero_()
        g.replay()
        x_ref = torch.zeros_like(b)
        _ffi.check(lib.gbchol_solve(s.handle, 0, nrhs, C.c_void_p(b.data_ptr()),
                                    C.c_void_p(x_ref.data_ptr()),
                                    C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        torch.cuda.synchronize()
        _ffi.check(lib.gbchol_check(s.handle))
        err = ((x - x_ref).abs().max() / x_ref.abs().max()).item()
        assert err <= 1e-5, err
