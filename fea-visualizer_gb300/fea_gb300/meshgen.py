"""Synthetic triangle meshes and initial fields for the FEM hot path.

The reference loads meshes from `.obj` files (`src/Utils/Surface.cpp:57-133`) or
triangulates a hand-drawn PSLG (`src/Utils/Surface.cpp:25-49`).  Neither the mesh
library nor the triangulator ships with it, so the workloads here are generated:

* ``icosphere(level)``: midpoint subdivision of the icosahedron projected onto the
  unit sphere.  V = 10*4^L + 2, T = 20*4^L (level 5 gives the 10,242 / 20,480 mesh
  of `assets/fem_meshes/icosphere.obj`, level 8 the 655,362-vertex sphere).
* ``jittered_grid(n, seed)``: the unit square from an n x n vertex grid, every cell
  split along a seeded random diagonal, interior vertices jittered by U(-0.3,0.3)*h.
* ``read_obj(path)``: a triangle reader with the semantics of
  `Surface::init_from_obj` (all `v` records, faces fan-triangulated).

Every generator is deterministic for a given seed and returns float32 xyz [V,3]
and uint32 triangles [T,3] with counter-clockwise (outward) winding.
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "icosphere", "jittered_grid", "cylinder", "read_obj", "boundary_vertices",
    "gray_scott_patches", "gaussian_bumps", "sphere_point", "fourier_field",
]


def _icosahedron():
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([
        [-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
        [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
        [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1],
    ], dtype=np.float64)
    f = np.array([
        [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
        [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
        [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
        [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1],
    ], dtype=np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v, f


def icosphere(level: int):
    """Unit icosphere after `level` midpoint subdivisions.

    Midpoints are numbered after the existing vertices in the order of their
    sorted (min, max) edge key, so the numbering is fully determined by `level`.
    """
    v, f = _icosahedron()
    for _ in range(int(level)):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        lo = np.minimum(e[:, 0], e[:, 1])
        hi = np.maximum(e[:, 0], e[:, 1])
        key = lo * nv + hi
        uk, inv = np.unique(key, return_inverse=True)
        ulo = uk // nv
        uhi = uk % nv
        mid = 0.5 * (v[ulo] + v[uhi])
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        nf = f.shape[0]
        m01 = nv + inv[:nf]
        m12 = nv + inv[nf:2 * nf]
        m20 = nv + inv[2 * nf:]
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        f = np.concatenate([
            np.stack([a, m01, m20], 1),
            np.stack([b, m12, m01], 1),
            np.stack([c, m20, m12], 1),
            np.stack([m01, m12, m20], 1),
        ], axis=0)
        v = np.concatenate([v, mid], axis=0)
    return v.astype(np.float32), f.astype(np.uint32)


def jittered_grid(n: int, seed: int = 0, jitter: float = 0.3):
    """Unit square from an n x n vertex grid (vertex (i, j) has index j*n + i).

    Each cell gets a seeded random diagonal; interior vertices move by
    U(-jitter, jitter)*h in x and y (h = 1/(n-1)); the mesh lies in z = 0.
    """
    n = int(n)
    rng = np.random.default_rng(seed)
    h = 1.0 / (n - 1)
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    x = ii.astype(np.float64) * h
    y = jj.astype(np.float64) * h
    jit = rng.uniform(-jitter, jitter, size=(2, n, n)) * h
    interior = (ii > 0) & (ii < n - 1) & (jj > 0) & (jj < n - 1)
    x = np.where(interior, x + jit[0], x)
    y = np.where(interior, y + jit[1], y)
    xyz = np.stack([x.ravel(), y.ravel(), np.zeros(n * n)], 1).astype(np.float32)
    ci, cj = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing="xy")
    ci = ci.ravel()
    cj = cj.ravel()
    v00 = cj * n + ci
    v10 = v00 + 1
    v01 = v00 + n
    v11 = v01 + 1
    diag = rng.integers(0, 2, size=v00.shape[0])
    t1 = np.where(diag[:, None] == 0, np.stack([v00, v10, v11], 1), np.stack([v00, v10, v01], 1))
    t2 = np.where(diag[:, None] == 0, np.stack([v00, v11, v01], 1), np.stack([v10, v11, v01], 1))
    tri = np.stack([t1, t2], 1).reshape(-1, 3)
    return xyz, tri.astype(np.uint32)


def cylinder(n_around: int, n_along: int, radius: float = 1.0, height: float = 2.0):
    """Open tube (two boundary loops), quads split along the (0,2) diagonal.

    A stand-in for `assets/fem_meshes/tube.obj` that exercises Dirichlet
    boundaries without depending on a quad-splitting rule.
    """
    th = np.arange(n_around) * (2 * np.pi / n_around)
    z = np.linspace(-height / 2, height / 2, n_along)
    tt, zz = np.meshgrid(th, z, indexing="xy")
    xyz = np.stack([radius * np.cos(tt).ravel(), radius * np.sin(tt).ravel(), zz.ravel()], 1)
    tris = []
    for j in range(n_along - 1):
        for i in range(n_around):
            a = j * n_around + i
            b = j * n_around + (i + 1) % n_around
            c = b + n_around
            d = a + n_around
            tris.append((a, b, c))
            tris.append((a, c, d))
    return xyz.astype(np.float32), np.array(tris, dtype=np.uint32)


def read_obj(path: str):
    """Read `v` and `f` records of an OBJ file.

    Follows `Surface::init_from_obj` (`src/Utils/Surface.cpp:57-92`): every `v`
    record becomes a vertex, every face becomes triangles.  Faces with more than
    three corners are split as a fan (0, k, k+1); the reference delegates this to
    tinyobjloader, whose split rule is not vendored with it.
    """
    verts = []
    tris = []
    with open(path, "r") as fh:
        for line in fh:
            if line.startswith("v "):
                p = line.split()
                verts.append((float(p[1]), float(p[2]), float(p[3])))
            elif line.startswith("f "):
                idx = []
                for tok in line.split()[1:]:
                    k = int(tok.split("/")[0])
                    idx.append(k - 1 if k > 0 else len(verts) + k)
                for k in range(1, len(idx) - 1):
                    tris.append((idx[0], idx[k], idx[k + 1]))
    if not verts:
        raise ValueError(f"{path} holds no vertices")
    return np.array(verts, dtype=np.float32), np.array(tris, dtype=np.uint32)


def boundary_vertices(tri: np.ndarray, nverts: int) -> np.ndarray:
    """Vertices on an edge used by exactly one triangle (`Surface.cpp:104-122`)."""
    t = tri.astype(np.int64)
    a = np.concatenate([t[:, 0], t[:, 1], t[:, 2]])
    b = np.concatenate([t[:, 1], t[:, 2], t[:, 0]])
    keep = a != b
    a, b = a[keep], b[keep]
    lo = np.minimum(a, b)
    hi = np.maximum(a, b)
    key = lo * nverts + hi
    uk, cnt = np.unique(key, return_counts=True)
    once = uk[cnt == 1]
    out = np.zeros(nverts, dtype=np.uint8)
    out[once // nverts] = 1
    out[once % nverts] = 1
    return out


def gray_scott_patches(xyz: np.ndarray, seed: int = 0, n_patches: int = 20,
                       side: float = 0.05, noise: float = 0.01):
    """u = 1, v = 0, except seeded squares (u = 0.5, v = 0.25), plus noise.

    Squares of side `side` are placed uniformly in the bounding box of the
    first two coordinates (planar meshes).  The noise is additive
    U(-noise, noise) on both fields, clipped to [0, 1].
    """
    rng = np.random.default_rng(seed)
    x = xyz[:, 0].astype(np.float64)
    y = xyz[:, 1].astype(np.float64)
    lo = np.array([x.min(), y.min()])
    hi = np.array([x.max(), y.max()])
    u = np.ones(xyz.shape[0])
    v = np.zeros(xyz.shape[0])
    for _ in range(n_patches):
        c = lo + rng.uniform(0.0, 1.0, 2) * (hi - lo - side)
        m = (x >= c[0]) & (x <= c[0] + side) & (y >= c[1]) & (y <= c[1] + side)
        u[m] = 0.5
        v[m] = 0.25
    u += rng.uniform(-noise, noise, u.shape)
    v += rng.uniform(-noise, noise, v.shape)
    return np.clip(u, 0, 1).astype(np.float32), np.clip(v, 0, 1).astype(np.float32)


def sphere_patches(xyz: np.ndarray, seed: int = 0, n_patches: int = 20,
                   radius: float = 0.15, noise: float = 0.01):
    """Gray-Scott patches on a sphere: geodesic caps instead of squares."""
    rng = np.random.default_rng(seed)
    p = xyz.astype(np.float64)
    u = np.ones(p.shape[0])
    v = np.zeros(p.shape[0])
    for _ in range(n_patches):
        c = sphere_point(rng)
        m = np.linalg.norm(p - c, axis=1) < radius
        u[m] = 0.5
        v[m] = 0.25
    u += rng.uniform(-noise, noise, u.shape)
    v += rng.uniform(-noise, noise, v.shape)
    return np.clip(u, 0, 1).astype(np.float32), np.clip(v, 0, 1).astype(np.float32)


def sphere_point(rng) -> np.ndarray:
    """Uniform point on the unit sphere."""
    g = rng.normal(size=3)
    return g / np.linalg.norm(g)


def gaussian_bumps(xyz: np.ndarray, seed: int = 0, n_bumps: int = 1,
                   width2: float = 0.02, amplitude=None):
    """Sum of exp(-|x - p|^2 / width2) at seeded points p on the unit sphere.

    With `amplitude=None` every bump has amplitude 1; otherwise amplitudes are
    drawn from U(amplitude[0], amplitude[1]).
    """
    rng = np.random.default_rng(seed)
    p = xyz.astype(np.float64)
    out = np.zeros(p.shape[0])
    for _ in range(n_bumps):
        c = sphere_point(rng)
        a = 1.0 if amplitude is None else rng.uniform(amplitude[0], amplitude[1])
        out += a * np.exp(-np.sum((p - c) ** 2, axis=1) / width2)
    return out


def fourier_field(points: np.ndarray, seed: int = 0, n_modes: int = 16, max_freq: int = 4):
    """Smooth seeded random field: a sum of `n_modes` planar Fourier modes.

    g(x, y) = sum_m a_m cos(2*pi*(kx_m x + ky_m y) + phi_m) / sqrt(n_modes),
    integer wave numbers in [-max_freq, max_freq], a_m ~ N(0, 1).
    """
    rng = np.random.default_rng(seed)
    x = points[:, 0].astype(np.float64)
    y = points[:, 1].astype(np.float64)
    g = np.zeros(points.shape[0])
    for _ in range(n_modes):
        kx, ky = rng.integers(-max_freq, max_freq + 1, 2)
        a = rng.normal()
        ph = rng.uniform(0, 2 * np.pi)
        g += a * np.cos(2 * np.pi * (kx * x + ky * y) + ph)
    return g / np.sqrt(n_modes)
