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


STRUCTURES = ["forest", "star", "diagonal", "one", "dense96"]


def structural_cases():
    """Matrices whose elimination structure is unusual, as scipy COO (both
    triangles): a forest of 40 disconnected grids of different sizes (many
    elimination-tree roots), a star (one row coupled to every other), a
    diagonal matrix (no dependencies), a 1 x 1 system, and a dense 96 x 96
    SPD block (one supernode of three 32-column chunks). All are
    well conditioned (condition numbers below 100)."""
    import scipy.sparse as sp
    blocks = []
    for k in range(40):
        m = 5 + (k * 7) % 23
        vals, idx = workloads.grid2d_coo(m, 10.0, 1.0)
        blocks.append(sp.coo_matrix((vals, idx), shape=(m * m, m * m)).tocsr())
    forest = sp.block_diag(blocks).tocoo()
    n = 3000
    rows = np.r_[np.arange(n), np.arange(1, n)]
    cols = np.r_[np.arange(n), np.zeros(n - 1, int)]
    vals = np.r_[np.full(n, 4.0), np.full(n - 1, -1.0 / np.sqrt(n))]
    star = sp.coo_matrix((vals, (rows, cols)), shape=(n, n))
    star = (star + sp.tril(star, -1).T).tocoo()
    g = np.random.default_rng(96).standard_normal((96, 96))
    dense = sp.coo_matrix(g @ g.T / 96 + 2.0 * np.eye(96))
    return {"forest": forest, "star": star, "diagonal": (sp.identity(500) * 3.0).tocoo(),
            "one": sp.coo_matrix(np.array([[2.5]])), "dense96": dense}
