#!/usr/bin/env python
"""Benchmark: 3-D 7-point Poisson on a 64^3 grid (n = 262 144, diagonal
shift 1e-3), N(0,1) right-hand sides (seed 2), n_rhs = 128.

Headline `value`: RHS-solves/s of the FP32-factor solve with FP64-residual
iterative refinement to a max relative residual of 1e-10 (inputs resident in
HBM). Also reported: the plain FP64 GPU solve on the same factor (and the
ratio), an end-to-end figure through the public API with host buffers, the
roofline of the dominant kernel (the triangular sweep), clocks, and the
oracle's FP64 CPU solve on the host cores as `cpu_baseline`.

`--impl reference` times the CPU solve of the reference's path instead
(cholmod_solve semantics, restated by the oracle; CHOLMOD itself is absent)
on all host cores, on the same workload.

Multi-GPU: the solve does not shard, so N ranks run N independent replicas
(one per GPU, no collective on the data path) and `value` sums them.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--k", type=int, default=64, help="grid side (n = k^3)")
    p.add_argument("--nrhs", type=int, default=128)
    p.add_argument("--tol", type=float, default=1e-10)
    p.add_argument("--max-iter", type=int, default=5)
    p.add_argument("--cpu-sample-rhs", type=int, default=32,
                   help="RHS columns of the bounded CPU sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


# ------------------------------------------------------------- helpers ----

def hbm_peak():
    try:
        d = json.loads(PEAKS_FILE.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload(args):
    from cholespy_gb300 import workloads
    vals, idx = workloads.grid3d_coo(args.k, 1e-3)
    n = args.k ** 3
    rng = np.random.default_rng(2)
    b = rng.standard_normal((n, args.nrhs))
    return n, vals, idx, b


def config_dict(args, n, nnz_a, nnz_l, extra=None):
    d = {
        "workload": f"poisson3d_7pt_{args.k}^3_shift1e-3_nrhs{args.nrhs}",
        "n": n, "nnz_a": int(nnz_a), "nnz_l": int(nnz_l), "n_rhs": args.nrhs,
        "tol": args.tol, "rhs": "N(0,1) seed 2", "ordering": "nested dissection (host)",
        "l2": "inputs larger than L2 (factor alone exceeds 129 MB)",
    }
    if extra:
        d.update(extra)
    return d


def algorithmic_bytes(n, nnz_l, r, s):
    """Both sweeps of one solve (reference layout: CSR of L and of L^T):
    2*[nnz(L)*(s+4) + 4(n+1)] + 4n (perm) + 2*n*r*s (read b, write x)."""
    return 2 * (nnz_l * (s + 4) + 4 * (n + 1)) + 4 * n + 2 * n * r * s


# ------------------------------------------------------ reference arm ----

def run_reference(args, world, rank):
    """CPU solve of the reference's path (oracle port of cholmod_solve) on all
    host cores; rank 0 only."""
    if rank != 0:
        return
    import ctypes as C

    import oracle
    from cholespy_gb300 import _build, _ffi
    _build.build()
    n, vals, idx, b = workload(args)
    lib = _ffi.lib()
    ii = np.ascontiguousarray(idx[0], np.int32)
    jj = np.ascontiguousarray(idx[1], np.int32)
    xx = np.ascontiguousarray(vals, np.float64)
    f = C.c_void_p()
    _ffi.check(lib.gbchol_factorize(n, len(xx), ii.ctypes.data, jj.ctypes.data, xx.ctypes.data, 2, 0,
                                    C.byref(f)))
    nn, nnz, nsn, fl = C.c_int32(), C.c_int64(), C.c_int32(), C.c_double()
    lib.gbchol_factor_info(f, C.byref(nn), C.byref(nnz), C.byref(nsn), C.byref(fl))
    perm = np.zeros(n, np.int32)
    Lp = np.zeros(n + 1, np.int32)
    Li = np.zeros(nnz.value, np.int32)
    Lx = np.zeros(nnz.value, np.float64)
    lib.gbchol_factor_export(f, perm.ctypes.data, Lp.ctypes.data, Li.ctypes.data, Lx.ctypes.data)
    lib.gbchol_factor_free(f)
    cores = os.cpu_count() or 1
    sample = max(1, min(args.cpu_sample_rhs, args.nrhs))
    bs = np.ascontiguousarray(b[:, :sample])
    for _ in range(args.warmup):
        oracle.cpu_solve(perm, Lp, Li, Lx, bs, threads=cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.cpu_solve(perm, Lp, Li, Lx, bs, threads=cores)
    dt = time.perf_counter() - t0
    value = sample * args.steps / dt
    line = {
        "impl": "reference", "metric": "RHS-solves/s", "value": value, "unit": "RHS-solves/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(args, n, len(vals), nnz.value),
        "cpu_baseline": {"value": value, "unit": "RHS-solves/s", "cores": cores, "kind": "port",
                         "sample": f"{sample} of {args.nrhs} RHS columns per step, FP64 "
                                   "forward/back substitution (cholmod_solve semantics), "
                                   "RHS split over threads"},
        "e2e": {"value": value, "unit": "RHS-solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------ our arm ----

def run_ours(args, world, rank, local):
    import torch

    from cholespy_gb300 import CholeskySolverD, MatrixType, _build
    _build.build()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    n, vals, idx, b = workload(args)
    t0 = time.perf_counter()
    solver = CholeskySolverD(n, torch.tensor(idx[0]).to(dev), torch.tensor(idx[1]).to(dev),
                             torch.tensor(vals).to(dev), MatrixType.COO, refine=True,
                             tol=args.tol, max_iter=args.max_iter)
    t_ctor = time.perf_counter() - t0
    info = solver.info()
    solver.reserve(args.nrhs)
    bd = torch.tensor(b, device=dev)
    xd = torch.zeros_like(bd)
    stream = torch.cuda.current_stream(dev)

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize(dev)
        barrier(world)
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        barrier(world)
        return e0.elapsed_time(e1) / 1e3

    # headline: FP32 + refinement, device-resident inputs
    sampler = ClockSampler(dev.index)
    for _ in range(args.warmup):
        solver.solve(bd, xd)
    sampler.start()
    t_ir = timed(lambda: solver.solve(bd, xd), args.steps, 0)
    clocks = sampler.stop()
    solver.check()
    t_ir = max_over_ranks(t_ir, world)
    value = world * args.nrhs * args.steps / t_ir

    # accuracy of the refined solve (outside the timed region)
    stats = solver.solve_refined(bd, xd)
    x_ir = xd.cpu().numpy()

    # plain FP64 solve on the same factor
    x64 = torch.zeros_like(bd)
    t_64 = max_over_ranks(timed(lambda: solver.solve_fp64(bd, x64), args.steps, args.warmup), world)
    value_64 = world * args.nrhs * args.steps / t_64
    solver.check()

    # plain FP32 solve: the dominant kernel pair, for the roofline
    b32 = bd.float()
    x32 = torch.zeros_like(b32)
    from cholespy_gb300 import _ffi
    import ctypes as C

    def f32_solve():
        _ffi.check(_ffi.lib().gbchol_solve(solver.handle, 0, args.nrhs, C.c_void_p(b32.data_ptr()),
                                           C.c_void_p(x32.data_ptr()), C.c_void_p(stream.cuda_stream)))

    t_32 = timed(f32_solve, args.steps, args.warmup) / args.steps
    bytes32 = algorithmic_bytes(n, info.nnz_l, args.nrhs, 4)
    peak, peak_kind = hbm_peak()
    achieved = bytes32 / t_32 / 1e9

    # end to end through the public API with pinned host buffers
    bh = torch.tensor(b).pin_memory()
    xh = torch.empty_like(bh).pin_memory()

    def e2e_step():
        bd.copy_(bh, non_blocking=True)
        solver.solve(bd, xd)
        xh.copy_(xd, non_blocking=True)

    t_e2e = max_over_ranks(timed(e2e_step, args.steps, args.warmup), world)
    e2e_value = world * args.nrhs * args.steps / t_e2e

    # residuals / errors against the FP64 matrix
    import scipy.sparse as sp
    A = sp.csc_matrix((vals, (idx[0], idx[1])), shape=(n, n))
    A.sum_duplicates()
    low = sp.tril(A)
    A = (low + sp.tril(low, -1).T).tocsr()
    bn = np.linalg.norm(b, axis=0)
    res_ir = float((np.linalg.norm(b - A @ x_ir, axis=0) / bn).max())
    x64h = x64.cpu().numpy()
    res_64 = float((np.linalg.norm(b - A @ x64h, axis=0) / bn).max())
    err_ir_vs_64 = float(np.abs(x_ir - x64h).max() / np.abs(x64h).max())

    # CPU baseline: oracle FP64 solve on the same factor, bounded sample
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        perm, Lp, Li, Lx = solver.factor()
        cores = os.cpu_count() or 1
        sample = max(1, min(args.cpu_sample_rhs, args.nrhs))
        bs = np.ascontiguousarray(b[:, :sample])
        c0 = time.perf_counter()
        oracle.cpu_solve(perm, Lp, Li, Lx, bs, threads=cores)
        cdt = time.perf_counter() - c0
        cpu = {"value": sample / cdt, "unit": "RHS-solves/s", "cores": cores, "kind": "port",
               "sample": f"{sample} of {args.nrhs} RHS columns, one FP64 solve "
                         "(cholmod_solve semantics) on the same factor, RHS split over threads"}

    lps = info.launches_per_solve
    launches = lps + (args.max_iter + 1) + args.max_iter * lps
    line = {
        "metric": "RHS-solves/s (FP32 factor + FP64 iterative refinement to 1e-10)",
        "value": value, "unit": "RHS-solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_ir / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": config_dict(args, n, len(vals), info.nnz_l,
                              {"levels_lower": info.levels_lower, "levels_upper": info.levels_upper,
                               "supernodes": info.n_supernodes, "max_supernode": info.max_supernode,
                               "top_rows": info.top_rows, "top_units": info.top_units,
                               "top_blocks": info.top_blocks,
                               "factor_s": info.factor_seconds, "analysis_s": info.analysis_seconds,
                               "ctor_s": t_ctor, "parallelism": f"replicas x{world}"}),
        "refine": {"iterations": stats.iterations, "converged": stats.converged,
                   "max_rel_residual_device": stats.max_rel_residual,
                   "max_rel_residual_host": res_ir, "max_rel_err_vs_fp64_solve": err_ir_vs_64},
        "fp64_plain": {"value": value_64, "unit": "RHS-solves/s", "ms_per_step": 1e3 * t_64 / args.steps,
                       "max_rel_residual": res_64, "ir_over_fp64": value / value_64},
        "roofline": {"kernel": "triangular sweeps (FP32 solve, lower+upper)", "bound": "hbm",
                     "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "algorithmic_bytes": bytes32, "ms_per_solve": 1e3 * t_32},
        "e2e": {"value": e2e_value, "unit": "RHS-solves/s",
                "h2d_bytes_per_step": int(b.nbytes), "d2h_bytes_per_step": int(b.nbytes)},
        "clocks": clocks,
        "gpu_launches": launches * args.steps,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    world, rank, local = dist_setup(args)
    try:
        if args.impl == "reference":
            run_reference(args, world, rank)
        else:
            run_ours(args, world, rank, local)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
