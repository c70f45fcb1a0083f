"""Host-side check of the supernodal solve plan (no GPU): tests/plan_check.cpp
runs every sweep item in ticket order on the CPU and checks each wait, the
partial sums of the lower sweep and the solution; it also checks the
multi-threaded CSC transpose against a serial one for several thread counts,
and the bulk sweeps' schedule (tickets, partial-sum coverage, upper blocks)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HOST = ROOT / "cholespy_gb300" / "csrc" / "host"


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_plan_schedule_and_solution(tmp_path):
    exe = tmp_path / "plan_check"
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-I", str(HOST), "-I", str(ROOT / "include"),
           str(Path(__file__).with_name("plan_check.cpp")), *map(str, sorted(HOST.glob("*.cpp"))), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    p = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stdout[-4000:] + p.stderr[-2000:]
    # 17 plans x 2 RHS counts, the transpose check, 7 plans x 4 bulk schedules
    assert "FAIL" not in p.stdout and p.stdout.count(" ok") == 63, p.stdout
