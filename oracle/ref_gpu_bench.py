"""Times the reference's own GPU solve (kernels/kernels.cu compiled from
source, launched by oracle/ref_gpu.cpp with the reference's protocol) next to
this library's solve on the same factor and the same device-resident RHS.

Test infrastructure, not the product: run on a GPU machine after build():
    python -m oracle.ref_gpu_bench [--cases ico6_r3,ico6_r128,...]
Prints one JSON line per case (median of CUDA-event timings after warm-up).
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402


def build_case(name):
    from cholespy_gb300 import workloads
    if name.startswith("ico"):
        level = int(name[3])
        n, faces, pos = workloads.icosphere(level)
        lam = 19.0
        vals, idx = workloads.laplacian_coo(n, faces, lam)
        return n, vals, idx
    if name.startswith("p3d"):
        k = int(name[3:])
        vals, idx = workloads.grid3d_coo(k, 1e-3)
        return k ** 3, vals, idx
    if name.startswith("grid"):
        k = int(name[4:])
        vals, idx = workloads.grid2d_coo(k, 10.0, 1.0)
        return k * k, vals, idx
    raise ValueError(name)


def timed(torch, fn, reps, warm=3):
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts))


def main():
    import torch

    from cholespy_gb300 import CholeskySolverD, CholeskySolverF, MatrixType
    from oracle import ref_gpu
    ap = argparse.ArgumentParser()
    ap.add_argument("--cases", default="ico6:3:f,ico6:128:f,grid64:1:d,p3d32:1:f,p3d32:128:f")
    ap.add_argument("--reps", type=int, default=10)
    args = ap.parse_args()
    for case in args.cases.split(","):
        name, nrhs, prec = case.split(":")
        nrhs = int(nrhs)
        n, vals, idx = build_case(name)
        cls = CholeskySolverF if prec == "f" else CholeskySolverD
        dt = torch.float32 if prec == "f" else torch.float64
        t0 = time.perf_counter()
        s = cls(n, torch.tensor(idx[0]).cuda(), torch.tensor(idx[1]).cuda(), torch.tensor(vals).cuda(),
                MatrixType.COO)
        t_ours_ctor = time.perf_counter() - t0
        perm, colptr, rowidx, lv = s.factor()
        t0 = time.perf_counter()
        r = ref_gpu.RefGpuSolver(perm, colptr, rowidx, lv, double=prec == "d")
        t_ref_analysis = time.perf_counter() - t0
        b = torch.randn(n, nrhs, device="cuda", dtype=dt)
        x = torch.zeros_like(b)
        xr = torch.zeros_like(b)
        t_ours = timed(torch, lambda: s.solve(b, x), args.reps)
        t_ref = timed(torch, lambda: r.solve(b, xr), args.reps)
        err = ((x - xr).abs().max() / xr.abs().max()).item()
        info = s.info()
        print(json.dumps({"case": name, "nrhs": nrhs, "precision": prec, "n": n, "nnz_l": info.nnz_l,
                          "levels": info.levels_lower, "ours_ms": t_ours, "reference_gpu_ms": t_ref,
                          "speedup": t_ref / t_ours, "ours_rhs_solves_per_s": nrhs * 1e3 / t_ours,
                          "reference_rhs_solves_per_s": nrhs * 1e3 / t_ref, "max_rel_diff": err,
                          "ours_ctor_s": t_ours_ctor, "reference_gpu_analysis_s": t_ref_analysis}),
              flush=True)
        r.close()


if __name__ == "__main__":
    main()
