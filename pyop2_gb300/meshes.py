"""Seeded synthetic meshes with the shapes of the benchmark configurations.

All generators are vectorised numpy and deterministic for a given seed.
Vertex jitter is uniform in (-0.2h, 0.2h) on interior vertices only, so the
domain stays the unit square / cube and cell measures sum to 1.
"""
import numpy as np


def unit_square_tris(n, jitter=0.2, seed=0):
    """n x n quads, each split into two triangles along a fixed diagonal.

    Returns (coords float64[(n+1)^2, 2], cells int32[2 n^2, 3]); vertices are
    numbered lexicographically (x fastest).
    """
    h = 1.0 / n
    i, j = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="xy")
    coords = np.stack([i.ravel() * h, j.ravel() * h], axis=1).astype(np.float64)
    if jitter:
        rng = np.random.default_rng(seed)
        inner = ((i.ravel() > 0) & (i.ravel() < n) & (j.ravel() > 0) & (j.ravel() < n))
        d = rng.uniform(-jitter * h, jitter * h, size=(coords.shape[0], 2))
        coords[inner] += d[inner]
    qi, qj = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    v00 = (qj * (n + 1) + qi).ravel()
    v10 = v00 + 1
    v01 = v00 + (n + 1)
    v11 = v01 + 1
    lower = np.stack([v00, v10, v11], axis=1)
    upper = np.stack([v00, v11, v01], axis=1)
    cells = np.empty((2 * n * n, 3), dtype=np.int32)
    cells[0::2] = lower
    cells[1::2] = upper
    return coords, cells


def unit_cube_tets(n, permute=False, seed=0, jitter=0.0):
    """n^3 hexes, each split into 6 Kuhn tetrahedra sharing the (1,1,1)
    diagonal.  Returns (coords float64[(n+1)^3, 3], cells int32[6 n^3, 4]).

    With permute=True the vertex ids are relabelled by a seeded random
    permutation (map values and coordinate rows permuted consistently).
    """
    m = n + 1
    h = 1.0 / n
    k, j, i = np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij")
    coords = np.stack([i.ravel() * h, j.ravel() * h, k.ravel() * h], axis=1).astype(np.float64)
    rng = np.random.default_rng(seed)
    if jitter:
        inner = ((i > 0) & (i < n) & (j > 0) & (j < n) & (k > 0) & (k < n)).ravel()
        d = rng.uniform(-jitter * h, jitter * h, size=coords.shape)
        coords[inner] += d[inner]
    hk, hj, hi = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    base = (hk * m * m + hj * m + hi).ravel().astype(np.int64)
    step = {0: 1, 1: m, 2: m * m}
    v7 = base + 1 + m + m * m
    tets = []
    for a, b, c in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        p1 = base + step[a]
        p2 = p1 + step[b]
        tets.append(np.stack([base, p1, p2, v7], axis=1))
    cells = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)
    if permute:
        perm = rng.permutation(coords.shape[0])        # new id of old vertex v is perm[v]
        inv = np.empty_like(perm)
        inv[perm] = np.arange(len(perm))
        coords = coords[inv]
        cells = perm[cells].astype(np.int32)
    return coords, cells


def p2_square(n, jitter=0.2, seed=0):
    """P2 Lagrange numbering of the n x n split-square mesh of unit_square_tris.

    Returns (coords float64[V, 2], cell2vert int32[C, 3], cell2dof int32[C, 6],
    ndofs).  Dofs 0..V-1 are the vertices, then one per edge: horizontal
    edges, vertical edges, quad diagonals, numbered analytically.  Local dof
    order is (v0, v1, v2, e12, e02, e01), e_ab the edge joining local
    vertices a and b.
    """
    coords, cells = unit_square_tris(n, jitter=jitter, seed=seed)
    V = (n + 1) * (n + 1)
    qi, qj = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    qi, qj = qi.ravel(), qj.ravel()
    H = lambda i, j: V + j * n + i                                   # (i,j)-(i+1,j)
    Vt = lambda i, j: V + n * (n + 1) + j * (n + 1) + i              # (i,j)-(i,j+1)
    D = lambda i, j: V + 2 * n * (n + 1) + j * n + i                 # (i,j)-(i+1,j+1)
    c2d = np.empty((2 * n * n, 6), dtype=np.int64)
    c2d[:, :3] = cells
    # lower [v00, v10, v11]: e12 = v10-v11, e02 = v00-v11, e01 = v00-v10
    c2d[0::2, 3] = Vt(qi + 1, qj)
    c2d[0::2, 4] = D(qi, qj)
    c2d[0::2, 5] = H(qi, qj)
    # upper [v00, v11, v01]: e12 = v11-v01, e02 = v00-v01, e01 = v00-v11
    c2d[1::2, 3] = H(qi, qj + 1)
    c2d[1::2, 4] = Vt(qi, qj)
    c2d[1::2, 5] = D(qi, qj)
    return coords, cells, c2d.astype(np.int32), V + 2 * n * (n + 1) + n * n


def batch_sizes(nmeshes=256, lo=1e3, hi=1e6, seed=0):
    """Cell counts drawn log-uniformly in [lo, hi] and the grid size n of each
    mesh (2 n^2 cells, n = round(sqrt(C / 2)))."""
    rng = np.random.default_rng(seed)
    cells = np.exp(rng.uniform(np.log(lo), np.log(hi), nmeshes))
    return [max(1, int(round(np.sqrt(c / 2)))) for c in cells]


def extruded_prisms(n, layers, seed=0, jitter=0.2):
    """Base: n x n split squares (2 n^2 triangles); extruded to `layers`
    layers (layers - 1 prism cells per column, height 1/(layers-1)).

    Nodes are numbered column-wise: node = base_vertex * layers + level.
    Returns (base_coords float64[Vb, 2], base_cells int32[Cb, 3],
    cell2node_base int32[Cb, 6] (bottom 3, top 3), offset int32[6] (all 1),
    nnodes, node_coords float64[Vb * layers, 3]).
    """
    bc, tri = unit_square_tris(n, jitter=jitter, seed=seed)
    Vb = bc.shape[0]
    base = np.concatenate([tri * layers, tri * layers + 1], axis=1).astype(np.int32)
    offset = np.ones(6, dtype=np.int32)
    z = np.arange(layers, dtype=np.float64) / (layers - 1)
    nc = np.empty((Vb, layers, 3))
    nc[:, :, 0:2] = bc[:, None, :]
    nc[:, :, 2] = z[None, :]
    return bc, tri, base, offset, Vb * layers, nc.reshape(-1, 3)


def lognormal(n, sigma, seed):
    return np.random.default_rng(seed).lognormal(0.0, sigma, size=n)
