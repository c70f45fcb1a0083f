"""In-tree build of libgbchol.so (CUDA kernels for sm_103a + host C++).

Compiles every translation unit in parallel (nvcc for ``csrc/*.cu``, g++ for
``csrc/host/*.cpp``) and links one shared library into
``cholespy_gb300/_lib/``. A stamp file holding a hash of the sources and
flags skips the build when nothing changed. No cmake, no torch extension
machinery: the library exposes a plain C ABI (``include/gbchol.h``).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OUT_DIR = PKG / "_lib"
BUILD_DIR = PKG / "_build"
LIB_NAME = "libgbchol.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-fopenmp", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbchol")


def _sources():
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted((CSRC / "host").glob("*.cpp"))
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + \
        sorted((CSRC / "host").glob("*.h")) + sorted(INCLUDE.glob("*.h"))
    return cu, cpp, headers


def _digest(files, extra):
    h = hashlib.sha256()
    for f in files:
        h.update(str(f.relative_to(ROOT)).encode())
        h.update(f.read_bytes())
    h.update(repr(extra).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def lib_path() -> Path:
    return OUT_DIR / LIB_NAME


def build(verbose: bool = False, force: bool = False) -> Path:
    cu, cpp, headers = _sources()
    nvcc = _nvcc()
    digest = _digest(cu + cpp + headers, (NVCC_FLAGS, CXX_FLAGS))
    stamp = OUT_DIR / (LIB_NAME + ".stamp")
    lib = lib_path()
    if not force and lib.exists() and stamp.exists() and stamp.read_text() == digest:
        return lib
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    inc = ["-I", str(INCLUDE), "-I", str(CSRC)]
    jobs = []
    for src in cu:
        obj = BUILD_DIR / (src.stem + ".cu.o")
        jobs.append(([nvcc, *NVCC_FLAGS, *inc, "-c", str(src), "-o", str(obj)], obj))
    for src in cpp:
        obj = BUILD_DIR / (src.stem + ".cpp.o")
        jobs.append((["g++", *CXX_FLAGS, *inc, "-c", str(src), "-o", str(obj)], obj))

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
        return p.stderr

    workers = max(1, min(len(jobs), os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(workers) as ex:
        for err in ex.map(run, [j[0] for j in jobs]):
            if verbose and err:
                print(err, file=sys.stderr)
    tmp = lib.with_suffix(".so.tmp")
    run([nvcc, *ARCH, "-shared", "-o", str(tmp), *[str(j[1]) for j in jobs],
         "-Xcompiler", "-fopenmp", "-lgomp"])
    os.replace(tmp, lib)
    stamp.write_text(digest)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
