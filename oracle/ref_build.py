"""ORACLE build recipe for the reference's own GPU kernels (test infrastructure).

Compiles the reference's kernels/kernels.cu FROM SOURCE, where it lies in the
reference checkout, to an sm_103a cubin in oracle/_ref/ (git-ignored; it
travels with the working tree). The reference's shipped PTX / bin2c header /
object files are not used. The cubin is loaded by oracle/ref_gpu.cpp, a
launcher restating the reference's host flow (src/cholesky_solver.cpp:299-432).

When the reference checkout is absent (on the GPU machine) an existing cubin is
used as is; only the launcher is (re)built from oracle/ref_gpu.cpp.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
CUBIN = REF_DIR / "ref_kernels.cubin"
LAUNCHER_SRC = HERE / "ref_gpu.cpp"
LAUNCHER = REF_DIR / "libref_gpu.so"
# The reference checkout: $CHOLESPY_REFERENCE_DIR, or the --reference argument
# of this script, else the build container's read-only checkout.
REFERENCE_DIR = Path(os.environ.get("CHOLESPY_REFERENCE_DIR", "/root/reference"))


def reference_kernels() -> Path:
    return REFERENCE_DIR / "kernels" / "kernels.cu"


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    return None


def build_cubin() -> bool:
    src = reference_kernels()
    if not src.exists():
        return CUBIN.exists()
    nvcc = _nvcc()
    if nvcc is None:
        return CUBIN.exists()
    REF_DIR.mkdir(exist_ok=True)
    src_stamp = f"{src.stat().st_mtime_ns}"
    stamp = REF_DIR / "ref_kernels.stamp"
    if CUBIN.exists() and stamp.exists() and stamp.read_text() == src_stamp:
        return True
    subprocess.run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                    "-o", str(CUBIN), str(src)], check=True)
    stamp.write_text(src_stamp)
    return True


def build_launcher() -> bool:
    """Compile the driver-API launcher (needs cuda.h and libcuda)."""
    REF_DIR.mkdir(exist_ok=True)
    inc = Path("/usr/local/cuda/include")
    if not (inc / "cuda.h").exists():
        return False
    stamp = REF_DIR / "libref_gpu.stamp"
    key = f"{LAUNCHER_SRC.stat().st_mtime_ns}:{os.uname().machine}"
    if LAUNCHER.exists() and stamp.exists() and stamp.read_text() == key:
        return True
    libdirs = ["/usr/local/cuda/lib64/stubs", "/usr/local/cuda/lib64"]
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", str(inc), str(LAUNCHER_SRC),
           "-o", str(LAUNCHER)] + [f"-L{d}" for d in libdirs] + ["-lcuda"]
    subprocess.run(cmd, check=True)
    stamp.write_text(key)
    return True


def build_if_present() -> bool:
    ok = build_cubin()
    if ok:
        try:
            build_launcher()
        except subprocess.CalledProcessError:
            return False
    return ok and LAUNCHER.exists()


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--reference", help="path of the reference checkout")
    args = ap.parse_args()
    if args.reference:
        REFERENCE_DIR = Path(args.reference)
    print("cubin:", build_cubin(), "launcher:", build_launcher())
