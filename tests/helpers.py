"""Test matrices with the semantics of the reference's tests (tests/utils.py):
A = I + lambda * L_graph on meshes, lambda = 2, duplicate diagonal COO
entries, b ~ U[0, 1) from np.random.seed(45) with 256 columns."""
import numpy as np

from cholespy_gb300 import workloads

RHS = [1, 4, 16, 64, 128, 256]


def mesh(name):
    if name == "cube":
        return workloads.cube()
    level = int(name[len("ico"):])
    n, faces, _ = workloads.icosphere(level)
    return n, faces


def reference_problem(name, lam=2.0, ncols=256, dtype=np.float64):
    n, faces = mesh(name)
    vals, idx = workloads.laplacian_coo(n, faces, lam)
    np.random.seed(45)
    b = np.random.random(size=(n, ncols)).astype(dtype)
    return n, vals, idx, b


def spsolve_ref(n, vals, idx, b):
    import scipy.sparse as sp
    from scipy.sparse.linalg import spsolve
    A = sp.csc_matrix((vals, (idx[0], idx[1])), shape=(n, n))
    x = spsolve(A, b.astype(np.float64))
    return x.reshape(b.shape)


def sym_matrix(n, vals, idx):
    """Symmetric scipy matrix from A's lower triangle (CHOLMOD stype = -1)."""
    import scipy.sparse as sp
    A = sp.csc_matrix((vals, (idx[0], idx[1])), shape=(n, n))
    A.sum_duplicates()
    low = sp.tril(A)
    return (low + sp.tril(low, -1).T).tocsr()
