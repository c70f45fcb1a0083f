"""Seeded synthetic SPD systems for the benchmark configurations and tests.

* mesh Laplacians A = I + lambda * L_graph built the way the reference's test
  helper does (tests/utils.py:3-20): off-diagonal -lambda per unique edge, the
  diagonal +lambda repeated once per neighbour as DUPLICATE COO entries plus
  an identity entry, so the solver must sum duplicates;
* icospheres by midpoint subdivision of an icosahedron (topology like the
  reference's get_icosphere, tests/utils.py:23-82, plus vertex positions,
  which the reference does not generate) and a closed cube surface;
* 2-D 5-point and 3-D 7-point grid Laplacians (Dirichlet stencils).
"""
from __future__ import annotations

import itertools
import math

import numpy as np


# ---------------------------------------------------------------- meshes ----

def icosahedron():
    """12 vertices on the unit sphere and the 20 faces (outward oriented)."""
    phi = (1.0 + math.sqrt(5.0)) / 2.0
    v = []
    for a, b in itertools.product((-1.0, 1.0), repeat=2):
        v += [(0.0, a, b * phi), (a, b * phi, 0.0), (b * phi, 0.0, a)]
    v = np.array(v)
    faces = []
    for i, j, k in itertools.combinations(range(12), 3):
        if all(abs(np.linalg.norm(v[p] - v[q]) - 2.0) < 1e-9 for p, q in ((i, j), (j, k), (i, k))):
            n = np.cross(v[j] - v[i], v[k] - v[i])
            faces.append((i, j, k) if np.dot(n, v[i]) > 0 else (i, k, j))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v, np.array(faces, dtype=np.int64)


def icosphere(level: int):
    """(n_verts, faces, positions) of the icosahedron subdivided `level` times.

    10 * 4**level + 2 vertices (level 6: 40 962, level 7: 163 842)."""
    pos, faces = icosahedron()
    pos = [tuple(p) for p in pos]
    for _ in range(level):
        mid = {}

        def midpoint(a, b):
            key = (a, b) if a < b else (b, a)
            m = mid.get(key)
            if m is None:
                pa, pb = np.array(pos[a]), np.array(pos[b])
                pm = (pa + pb) / 2.0
                pm /= np.linalg.norm(pm)
                m = len(pos)
                pos.append(tuple(pm))
                mid[key] = m
            return m

        new = []
        for a, b, c in faces:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            new += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = np.array(new, dtype=np.int64)
    return len(pos), faces, np.array(pos)


def cube():
    """(8, faces): the closed surface of a unit cube, two triangles per side."""
    corners = [(x, y, z) for x in (0, 1) for y in (0, 1) for z in (0, 1)]
    idx = {c: i for i, c in enumerate(corners)}
    faces = []
    for axis in range(3):
        for side in (0, 1):
            quad = [c for c in corners if c[axis] == side]
            # order the 4 corners around the square
            o = [a for a in range(3) if a != axis]
            quad.sort(key=lambda c: math.atan2(c[o[1]] - 0.5, c[o[0]] - 0.5))
            q = [idx[c] for c in quad]
            faces += [(q[0], q[1], q[2]), (q[0], q[2], q[3])]
    return 8, np.array(faces, dtype=np.int64)


def mesh_edges(faces):
    """Unique undirected edges (i < j) of a triangle mesh."""
    f = np.asarray(faces)
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    e = np.sort(e, axis=1)
    return np.unique(e, axis=0)


def laplacian_coo(n_verts, faces, lam, weights=None):
    """COO (values, idx[2, nnz]) of A = I + lam * L with duplicate diagonal
    entries, following the reference's get_coo_arrays (tests/utils.py:3-20).
    `weights` (one per unique edge, as in mesh_edges) gives a weighted L."""
    e = mesh_edges(faces)
    w = np.ones(len(e)) if weights is None else np.asarray(weights, dtype=np.float64)
    ii = np.concatenate([e[:, 0], e[:, 1]])
    jj = np.concatenate([e[:, 1], e[:, 0]])
    ww = np.concatenate([w, w]) * lam
    diag = np.arange(n_verts)
    rows = np.concatenate([ii, ii, diag])
    cols = np.concatenate([jj, ii, diag])
    vals = np.concatenate([-ww, ww, np.ones(n_verts)])
    return vals, np.stack([rows, cols]).astype(np.int64)


# ----------------------------------------------------------------- grids ----

def grid2d_coo(k, lam=1.0, shift=1.0):
    """COO of shift*I + lam * L5 on a k x k grid (L5: 4 on the diagonal, -1 per
    grid neighbour). n = k*k, nnz = k*k + 4*k*(k-1)."""
    n = k * k
    ids = np.arange(n).reshape(k, k)
    r, c = [ids.ravel()], [ids.ravel()]
    v = [np.full(n, shift + 4.0 * lam)]
    for a, b in ((ids[1:, :], ids[:-1, :]), (ids[:, 1:], ids[:, :-1])):
        a, b = a.ravel(), b.ravel()
        r += [a, b]
        c += [b, a]
        v += [np.full(a.size, -lam), np.full(a.size, -lam)]
    return np.concatenate(v), np.stack([np.concatenate(r), np.concatenate(c)]).astype(np.int64)


def grid3d_coo(k, shift=1e-3):
    """COO of L7 + shift*I on a k^3 grid (L7: 6 on the diagonal, -1 per grid
    neighbour). k = 64 gives n = 262 144 and nnz = 1 810 432."""
    n = k ** 3
    ids = np.arange(n).reshape(k, k, k)
    r, c = [ids.ravel()], [ids.ravel()]
    v = [np.full(n, 6.0 + shift)]
    for a, b in ((ids[1:], ids[:-1]), (ids[:, 1:], ids[:, :-1]), (ids[:, :, 1:], ids[:, :, :-1])):
        a, b = a.ravel(), b.ravel()
        r += [a, b]
        c += [b, a]
        v += [np.full(a.size, -1.0), np.full(a.size, -1.0)]
    return np.concatenate(v), np.stack([np.concatenate(r), np.concatenate(c)]).astype(np.int64)


def to_csc(n, vals, idx):
    """(indptr, indices, data) CSC arrays of a COO matrix with duplicates summed."""
    import scipy.sparse as sp
    m = sp.csc_matrix((vals, (idx[0], idx[1])), shape=(n, n))
    m.sum_duplicates()
    m.sort_indices()
    return m.indptr.astype(np.int32), m.indices.astype(np.int32), m.data.astype(np.float64)


def to_csr(n, vals, idx):
    import scipy.sparse as sp
    m = sp.csr_matrix((vals, (idx[0], idx[1])), shape=(n, n))
    m.sum_duplicates()
    m.sort_indices()
    return m.indptr.astype(np.int32), m.indices.astype(np.int32), m.data.astype(np.float64)


# ------------------------------------------------------- named workloads ----

def config_grid64(seed=0):
    """2-D 5-point Laplacian on 64 x 64, A = I + 10 L, COO, one N(0,1) RHS."""
    vals, idx = grid2d_coo(64, lam=10.0, shift=1.0)
    rng = np.random.default_rng(seed)
    return 64 * 64, vals, idx, rng.standard_normal((64 * 64, 1))


def config_icosphere6(seed=1, level=6):
    """Icosphere subdivision 6, A = I + 19 L, CSC, RHS = xyz + N(0, 0.01)."""
    n, faces, pos = icosphere(level)
    vals, idx = laplacian_coo(n, faces, 19.0)
    rng = np.random.default_rng(seed)
    b = pos + rng.normal(0.0, 0.01, size=pos.shape)
    return n, vals, idx, b


def config_poisson64(seed=2, k=64, nrhs=128):
    """3-D 7-point Poisson on k^3 with diagonal shift 1e-3, N(0,1) RHS."""
    vals, idx = grid3d_coo(k, 1e-3)
    rng = np.random.default_rng(seed)
    return k ** 3, vals, idx, rng.standard_normal((k ** 3, nrhs))


def config_batch(seed=3, count=256, n_min=1e3, n_max=1e5, max_rhs=128):
    """256 grid systems A_k = I + lam_k L5, n_k log-uniform in [1e3, 1e5]
    (side = round(sqrt(n_k))), lam_k ~ U[1, 50], n_rhs_k ~ U{1..128}."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        nk = math.exp(rng.uniform(math.log(n_min), math.log(n_max)))
        side = max(2, int(round(math.sqrt(nk))))
        lam = rng.uniform(1.0, 50.0)
        r = int(rng.integers(1, max_rhs + 1))
        vals, idx = grid2d_coo(side, lam=lam, shift=1.0)
        b = rng.standard_normal((side * side, r))
        out.append((side * side, vals, idx, b))
    return out


def config_icosphere7_weighted(seed=4, level=7, lam=19.0):
    """Icosphere subdivision 7, A = I + 19 L_w, edge weights U[0.5, 2], n_rhs = 3,
    loss weights w ~ N(0, 1)."""
    n, faces, pos = icosphere(level)
    rng = np.random.default_rng(seed)
    e = mesh_edges(faces)
    w_edges = rng.uniform(0.5, 2.0, size=len(e))
    vals, idx = laplacian_coo(n, faces, lam, weights=w_edges)
    b = pos.copy()
    wloss = rng.standard_normal((n, 3))
    return n, vals, idx, b, wloss
