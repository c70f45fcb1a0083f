"""Batched solves: many factors of uneven sizes and RHS counts in one
persistent launch per sweep phase (gbchol_batch_* in include/gbchol.h).

    batch = BatchSolver([s0, s1, ...], nrhs=[r0, r1, ...])
    batch.solve(bs, xs)          # bs[k], xs[k]: CUDA tensors (n_k, r_k)
    g = batch.capture(bs, xs)    # CUDA graph of the bound solve
    g.replay()
    width, batch = BatchSolver.tune([s0, s1, ...], nrhs=[r0, r1, ...])

The row sweeps' schedule (group budget, wavefront skew, lane-mode variant;
gbchol_batch_options) takes the library's defaults unless given.

No counterpart in the reference (each of its solvers is solved separately).
"""
from __future__ import annotations

import ctypes as C

from . import _ffi
from .solver import CholeskySolverD, CholeskySolverF


class BatchSolver:
    def __init__(self, solvers, nrhs, group_mb=None, skew=None, row_variant=None):
        if not solvers:
            raise ValueError("A batch needs at least one solver.")
        kinds = {type(s) for s in solvers}
        if kinds == {CholeskySolverF}:
            self._precision = 0
        elif kinds <= {CholeskySolverD}:
            self._precision = 1
        else:
            raise ValueError("A batch holds solvers of one precision.")
        if any(getattr(s, "is_cpu", False) for s in solvers):
            raise ValueError("A batch solves on the GPU: build its solvers from CUDA arrays.")
        if len(nrhs) != len(solvers):
            raise ValueError("One RHS count per solver.")
        self._solvers = list(solvers)          # keep the factors alive
        self._nrhs = [int(r) for r in nrhs]
        self._device = solvers[0]._device
        arr = (C.c_void_p * len(solvers))(*[s.handle.value for s in solvers])
        rr = (C.c_int32 * len(solvers))(*self._nrhs)
        h = C.c_void_p()
        if group_mb is None and skew is None and row_variant is None:
            _ffi.check(_ffi.lib().gbchol_batch_create(len(solvers), arr, rr, self._precision, C.byref(h)))
            self.schedule = None
        else:
            o = _ffi.BatchOptions(int((8 if group_mb is None else group_mb) * (1 << 20)),
                                  4 if skew is None else int(skew), 2 if row_variant is None else int(row_variant))
            _ffi.check(_ffi.lib().gbchol_batch_create_ex(len(solvers), arr, rr, self._precision, C.byref(o),
                                                         C.byref(h)))
            self.schedule = {"group_mb": o.group_bytes / (1 << 20), "skew": o.skew, "row_variant": o.row_variant}
        self._h = h
        self._bound = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _ffi.lib().gbchol_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    def _check_io(self, bs, xs):
        import torch
        dt = torch.float32 if self._precision == 0 else torch.float64
        if len(bs) != len(self._solvers) or len(xs) != len(self._solvers):
            raise ValueError("One b and one x per solver.")
        for s, r, b, x in zip(self._solvers, self._nrhs, bs, xs):
            for t in (b, x):
                if not t.is_cuda or t.device.index != self._device:
                    raise ValueError("Batch arrays must be CUDA tensors on the solvers' device.")
                if t.dtype != dt or not t.is_contiguous():
                    raise TypeError(f"Batch arrays must be C-contiguous {dt}.")
                shape = tuple(t.shape)
                if shape != (s._n, r) and not (r == 1 and shape == (s._n,)):
                    raise ValueError("b and x of system k must have shape (n_k, nrhs_k).")

    def bind(self, bs, xs):
        """Bind the per-system device arrays (uploads the descriptor tables)."""
        self._check_io(bs, xs)
        key = tuple((b.data_ptr(), x.data_ptr()) for b, x in zip(bs, xs))
        if key == self._bound:
            return
        n = len(bs)
        bp = (C.c_void_p * n)(*[b.data_ptr() for b in bs])
        xp = (C.c_void_p * n)(*[x.data_ptr() for x in xs])
        _ffi.check(_ffi.lib().gbchol_batch_set_io(self._h, bp, xp))
        self._keep = (list(bs), list(xs))
        self._bound = key

    def solve(self, bs=None, xs=None):
        """Solve every system (asynchronously on the current CUDA stream)."""
        import torch
        if bs is not None:
            self.bind(bs, xs)
        stream = torch.cuda.current_stream(self._device).cuda_stream
        _ffi.check(_ffi.lib().gbchol_batch_solve(self._h, C.c_void_p(stream)))

    def check(self):
        import torch
        stream = torch.cuda.current_stream(self._device).cuda_stream
        _ffi.check(_ffi.lib().gbchol_batch_check(self._h, C.c_void_p(stream)))

    def info(self):
        la, z, r = C.c_int32(), C.c_int64(), C.c_int64()
        _ffi.check(_ffi.lib().gbchol_batch_info(self._h, C.byref(la), C.byref(z), C.byref(r)))
        return {"launches": la.value, "nnz_l": z.value, "rows": r.value}

    @classmethod
    def tune(cls, solvers, nrhs, candidates=(8, 16, 32), reps=3, skews=(0, 4), group_mb=8):
        """Autotuner of the batch: for each candidate top-region width,
        rebuild every solver's plan with it (`replan`); for each wavefront
        skew of the row sweeps' schedule (groups of `group_mb` MB), build the
        batch and time `reps` batched solves (CUDA events, after one warm-up
        solve) on zero right-hand sides of the batch's shapes; keep the
        fastest pair for all solvers. Returns (width, BatchSolver built on
        that width and skew; its `schedule` names the skew). Batches built
        earlier from these solvers must be built again. No counterpart in
        the reference."""
        import torch
        if not candidates or reps < 1 or not skews:
            raise ValueError("At least one candidate width, one skew and one repetition are needed.")
        solvers = list(solvers)
        if len(nrhs) != len(solvers):
            raise ValueError("One RHS count per solver.")
        if not solvers:
            raise ValueError("A batch needs at least one solver.")
        dev = torch.device("cuda", solvers[0]._device)
        dt = torch.float64 if isinstance(solvers[0], CholeskySolverD) else torch.float32
        bs = [torch.zeros(s._n, int(r), device=dev, dtype=dt) for s, r in zip(solvers, nrhs)]
        xs = [torch.zeros_like(b) for b in bs]
        best, best_t = None, None
        with torch.cuda.device(dev):
            for w in candidates:
                for s in solvers:
                    s.replan(int(w))
                for k in skews:
                    batch = cls(solvers, nrhs, group_mb=group_mb, skew=int(k))
                    batch.solve(bs, xs)
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record()
                    for _ in range(reps):
                        batch.solve()
                    e1.record()
                    e1.synchronize()
                    batch.check()
                    t = e0.elapsed_time(e1)
                    if best_t is None or t < best_t:
                        best, best_t = (int(w), int(k)), t
                    del batch
            for s in solvers:
                s.replan(best[0])
        return best[0], cls(solvers, nrhs, group_mb=group_mb, skew=best[1])

    def capture(self, bs, xs):
        """CUDA graph of one batched solve on the given arrays (replay() to run)."""
        import torch
        self.bind(bs, xs)
        self.solve()  # warm up outside capture
        torch.cuda.synchronize(self._device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.solve()
        return g
