"""The bench's multi-process path on CPU (gloo, world size 2): rank set-up,
barrier and max over ranks, and the reference arm under torchrun (rank 0
measures and prints, the other rank exits without work). The solve itself
does not shard (replicas only), so no collective touches the data path."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, str(ROOT))
    import bench
    w, r, _ = bench.dist_setup(None)
    bench.barrier(w)
    v = bench.max_over_ranks(r + 1.5, w)
    Path(out_dir, f"rank{r}.txt").write_text(repr((w, r, v)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_rank_helpers_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    got = sorted(eval(Path(tmp_path, f"rank{r}.txt").read_text()) for r in range(2))
    assert got == [(2, 0, 2.5), (2, 1, 2.5)]


def test_reference_arm_two_ranks():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "1", "--k", "10", "--nrhs", "4"]
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert p.returncode == 0, p.stderr[-3000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout  # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["metric"].startswith("RHS-solves/s")


def test_bench_cpu_workload_line():
    """`bench.py --workload cpu` (the CPU-array path, no GPU) prints one JSON
    line with the contract keys and a converged FP32-rounded solution."""
    out = subprocess.run([sys.executable, "bench.py", "--workload", "cpu", "--steps", "2", "--warmup", "1",
                          "--nrhs", "16"], cwd=str(ROOT), capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "steps", "warmup", "ms_per_step", "config", "cpu_baseline"):
        assert key in line
    assert line["value"] > 0 and line["gpu_launches"] == 0
    assert line["config"]["max_rel_residual"] < 1e-5
