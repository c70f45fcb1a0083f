"""Regenerates the committed golden fixtures of tests/golden/.

The reference's own tests pin solutions to scipy.sparse.linalg.spsolve on
mesh Laplacians (reference tests/test_cholesky.py:10-44, tests/utils.py:3-20):
A = I + 2 L_graph with duplicate diagonal COO entries, b ~ U[0, 1) from
np.random.seed(45). This script writes those systems and spsolve's answers
for the cube and the level-3 icosphere (first 16 RHS columns) so the CPU
tests can pin the oracle without recomputing them.

Run from the repository root:  python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from helpers import reference_problem, spsolve_ref  # noqa: E402


def main():
    out = Path(__file__).resolve().parent
    for name, cols in (("cube", 256), ("ico3", 16)):
        n, vals, idx, b = reference_problem(name)
        b = b[:, :cols]
        x = spsolve_ref(n, vals, idx, b)
        np.savez_compressed(out / f"spsolve_{name}.npz", n=n, vals=vals, idx=idx.astype(np.int32),
                            b=b, x=x)
        print(name, n, vals.shape, b.shape)


if __name__ == "__main__":
    main()
