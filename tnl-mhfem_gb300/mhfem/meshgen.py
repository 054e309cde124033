"""Seeded synthetic simplex meshes and random fields (numpy).

The reference runs on meshes read from VTK files (its example meshes are
Git-LFS stubs); these generators build the jittered structured meshes the
benchmark workloads are defined on:

* ``square_triangles(N)``: the unit square as N x N squares, each split into
  two triangles along the (0,0)-(1,1) diagonal;
* ``cube_tetrahedra(N)``: the unit cube as N^3 cubes, each split into six
  tetrahedra along its main diagonal (Kuhn split, conforming between cubes).

Interior vertices are jittered uniformly by +-jitter*h per coordinate; boundary
vertices stay on the grid so the domain is exact.  Local vertex e of a cell is
opposite its local face e.
"""
from __future__ import annotations

import itertools

import numpy as np


def square_triangles(N: int, jitter: float = 0.2, seed: int = 1234):
    h = 1.0 / N
    idx = np.arange(N + 1)
    iy, ix = np.meshgrid(idx, idx, indexing="ij")
    coords = np.stack([ix.ravel() * h, iy.ravel() * h], axis=1)
    rng = np.random.default_rng(seed)
    J = rng.uniform(-jitter * h, jitter * h, size=coords.shape)
    interior = ((ix > 0) & (ix < N) & (iy > 0) & (iy < N)).ravel()
    coords[interior] += J[interior]
    sy, sx = np.meshgrid(np.arange(N), np.arange(N), indexing="ij")
    v00 = (sy * (N + 1) + sx).ravel()
    v10 = v00 + 1
    v01 = v00 + (N + 1)
    v11 = v01 + 1
    cells = np.empty((2 * N * N, 3), np.int32)
    cells[0::2] = np.stack([v00, v10, v11], axis=1)
    cells[1::2] = np.stack([v00, v11, v01], axis=1)
    return coords, cells


_KUHN_PERMS = list(itertools.permutations(range(3)))


def cube_tetrahedra(N: int, jitter: float = 0.15, seed: int = 1234):
    h = 1.0 / N
    idx = np.arange(N + 1)
    iz, iy, ix = np.meshgrid(idx, idx, idx, indexing="ij")
    coords = np.stack([ix.ravel() * h, iy.ravel() * h, iz.ravel() * h], axis=1)
    rng = np.random.default_rng(seed)
    J = rng.uniform(-jitter * h, jitter * h, size=coords.shape)
    interior = ((ix > 0) & (ix < N) & (iy > 0) & (iy < N) & (iz > 0) & (iz < N)).ravel()
    coords[interior] += J[interior]
    cz, cy, cx = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    base = ((cz * (N + 1) + cy) * (N + 1) + cx).ravel().astype(np.int64)
    step = np.array([1, N + 1, (N + 1) * (N + 1)], dtype=np.int64)
    cells = np.empty((6 * N ** 3, 4), np.int32)
    for t, perm in enumerate(_KUHN_PERMS):
        v0 = base
        v1 = v0 + step[perm[0]]
        v2 = v1 + step[perm[1]]
        v3 = v2 + step[perm[2]]
        cells[t::6] = np.stack([v0, v1, v2, v3], axis=1)
    return coords, cells


def _graded_axis(N: int, amplitude: float = 0.25) -> np.ndarray:
    """N + 1 monotone nodes on [0, 1] with non-uniform spacing (sine grading)."""
    i = np.arange(N + 1, dtype=np.float64)
    return i / N + amplitude / N * np.sin(2 * np.pi * i / N) / (2 * np.pi) * 2


def square_rectangles(N: int, graded: bool = True):
    """N x N axis-aligned rectangles on the unit square (tensor-product grid,
    graded so the cells are not squares).  Vertex order of each cell as the
    reference's Quadrangle: v0 lower-left, v1 lower-right, v2 upper-right,
    v3 upper-left."""
    x = _graded_axis(N) if graded else np.linspace(0, 1, N + 1)
    y = _graded_axis(N, 0.15) if graded else np.linspace(0, 1, N + 1)
    X, Y = np.meshgrid(x, y, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel()], axis=1)
    vid = lambda i, j: i * (N + 1) + j
    i, j = np.meshgrid(np.arange(N), np.arange(N), indexing="ij")
    i, j = i.ravel(), j.ravel()
    cells = np.stack([vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1)], axis=1).astype(np.int32)
    return coords, cells


def cube_cuboids(N: int, graded: bool = True):
    """N^3 axis-aligned cuboids on the unit cube (graded tensor-product grid).
    Vertex order as the reference's Hexahedron: the bottom rectangle
    v0..v3 counterclockwise from the lowest corner, then the top v4..v7."""
    ax = [(_graded_axis(N, a) if graded else np.linspace(0, 1, N + 1)) for a in (0.25, 0.15, 0.2)]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    M = N + 1
    vid = lambda i, j, k: (i * M + j) * M + k
    i, j, k = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    cells = np.stack([vid(i, j, k), vid(i + 1, j, k), vid(i + 1, j + 1, k), vid(i, j + 1, k),
                      vid(i, j, k + 1), vid(i + 1, j, k + 1), vid(i + 1, j + 1, k + 1), vid(i, j + 1, k + 1)],
                     axis=1).astype(np.int32)
    return coords, cells


# local vertices of the faces of a rectangle / cuboid (TNL Quadrangle and
# Hexahedron subentity order)
BOX_FACES = {2: [[0, 1], [1, 2], [2, 3], [3, 0]],
             3: [[0, 1, 2, 3], [0, 1, 5, 4], [1, 2, 6, 5], [2, 3, 7, 6], [3, 0, 4, 7], [4, 5, 6, 7]]}


def is_box_mesh(coords: np.ndarray, cells: np.ndarray) -> bool:
    """2^dim vertices per cell: rectangles / cuboids (else simplices)."""
    return cells.shape[1] == 2 ** coords.shape[1]


def count_faces(cells: np.ndarray, box: bool = False) -> int:
    """Number of distinct faces (sorted vertex tuples) of a conforming mesh."""
    nv = cells.shape[1]
    if box:
        dim = 2 if nv == 4 else 3
        f = np.stack([cells[:, q] for q in BOX_FACES[dim]], axis=1)
    else:
        f = np.stack([np.delete(cells, e, axis=1) for e in range(nv)], axis=1)
    f = np.sort(f.reshape(-1, f.shape[-1]), axis=1)
    return int(np.unique(f, axis=0).shape[0])


def gaussian_field(shape, corr_length: float = 0.1, seed: int = 5678) -> np.ndarray:
    """Zero-mean, unit-variance Gaussian random field on a periodic grid of
    the unit square/cube, with Gaussian covariance of the given correlation
    length: white noise filtered in Fourier space by exp(-|k|^2 l^2 / 4)."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(shape)
    ks = [np.fft.fftfreq(s, d=1.0 / s) * 2 * np.pi for s in shape]
    grids = np.meshgrid(*ks, indexing="ij")
    k2 = sum(g * g for g in grids)
    g = np.real(np.fft.ifftn(np.fft.fftn(w) * np.exp(-k2 * corr_length ** 2 / 4.0)))
    g -= g.mean()
    sd = g.std()
    return g / sd if sd > 0 else g


def cell_centroids(coords: np.ndarray, cells: np.ndarray) -> np.ndarray:
    return coords[cells].mean(axis=1)


def cell_grid_index(centroids: np.ndarray, N: int) -> tuple:
    """Index of the grid square/cube that contains each centroid."""
    ij = np.clip(np.floor(centroids * N).astype(np.int64), 0, N - 1)
    return tuple(ij[:, d] for d in range(ij.shape[1]))


def face_centroids(coords: np.ndarray, face_verts: np.ndarray) -> np.ndarray:
    return coords[face_verts].mean(axis=1)


def outward_face_normals(coords: np.ndarray, cells: np.ndarray) -> np.ndarray:
    """Outward normals scaled by the face measure, [C][nf][dim].  Simplices:
    face e is opposite local vertex e.  Axis-aligned boxes (2^dim vertices
    per cell): the faces of the Quadrangle (bottom, right, top, left) and
    Hexahedron (bottom, front, right, back, left, top) orders."""
    C, nv = cells.shape
    dim = coords.shape[1]
    if nv == 2 ** dim:
        h = coords[cells[:, 2 if dim == 2 else 6]] - coords[cells[:, 0]]
        if dim == 2:
            out = np.zeros((C, 4, 2))
            out[:, 0, 1] = -h[:, 0]; out[:, 1, 0] = h[:, 1]; out[:, 2, 1] = h[:, 0]; out[:, 3, 0] = -h[:, 1]
            return out
        out = np.zeros((C, 6, 3))
        axy, axz, ayz = h[:, 0] * h[:, 1], h[:, 0] * h[:, 2], h[:, 1] * h[:, 2]
        out[:, 0, 2] = -axy; out[:, 1, 1] = -axz; out[:, 2, 0] = ayz
        out[:, 3, 1] = axz; out[:, 4, 0] = -ayz; out[:, 5, 2] = axy
        return out
    nf = nv
    X = coords[cells]  # [C][nf][dim]
    out = np.empty((C, nf, dim))
    for e in range(nf):
        others = [v for v in range(nf) if v != e]
        if dim == 2:
            t = X[:, others[1]] - X[:, others[0]]
            n = np.stack([t[:, 1], -t[:, 0]], axis=1)
        else:
            n = 0.5 * np.cross(X[:, others[1]] - X[:, others[0]], X[:, others[2]] - X[:, others[0]])
        d = X[:, others[0]] - X[:, e]
        sgn = np.sign(np.einsum("ij,ij->i", n, d))
        out[:, e] = n * sgn[:, None]
    return out
