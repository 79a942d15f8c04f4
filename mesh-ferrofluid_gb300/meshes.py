"""Deterministic synthetic surface meshes for the MoM / Laplace-BEM workloads.

The reference loads meshes from `assets/` (``demo/demo_Helmholtz_MOM_3d.py:158``,
``demo/demo_Laplace_3d.py:106``); those assets are not shipped, so every workload here
is generated from a seed:

* ``icosphere(level)`` -- the icosahedron refined ``level`` times, vertices on the unit
  sphere.  F = 20*4**level triangles, V = 10*4**level + 2, E = 30*4**level RWG edges.
  Children of a face are stored next to each other, so consecutive faces are
  spatially close (useful for tile locality on the GPU).
* ``ellipsoid(level, axes, jitter, seed)`` -- a scaled icosphere with vertices jittered
  along their normals by N(0, jitter * mean edge length).
* ``star_shape(level, seed)`` -- r(theta, phi) = 1 + sum of 6 random real spherical
  harmonics with l <= 4 and amplitudes U(0, 0.15).
* ``fibonacci_lattice(n)`` -- the same lattice as ``FibonacciLattice``
  (``src/utils/functions.py:1024-1054``), in float64.

All faces are counter-clockwise seen from outside, so (v1-v0) x (v2-v1) points outward,
matching ``compute_tensor_face_normals`` (``src/utils/mesh_utils.py:158-197``).
"""
from __future__ import annotations

import math

import numpy as np

__all__ = [
    "icosphere",
    "ellipsoid",
    "star_shape",
    "fibonacci_lattice",
    "mean_edge_length",
]


def _icosahedron():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array(
        [
            [-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
            [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
            [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1],
        ],
        dtype=np.float64,
    )
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array(
        [
            [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
            [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
            [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
            [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1],
        ],
        dtype=np.int64,
    )
    return v, f


def icosphere(level: int, radius: float = 1.0):
    """Return ``(verts [V,3] float64, faces [F,3] int32)`` of the refined icosahedron."""
    if level < 0:
        raise ValueError("level must be >= 0")
    verts, faces = _icosahedron()
    verts = list(map(tuple, verts))
    for _ in range(level):
        cache: dict[tuple[int, int], int] = {}

        def midpoint(a: int, b: int) -> int:
            key = (a, b) if a < b else (b, a)
            idx = cache.get(key)
            if idx is None:
                p = np.add(verts[a], verts[b]) * 0.5
                p /= np.linalg.norm(p)
                verts.append(tuple(p))
                idx = len(verts) - 1
                cache[key] = idx
            return idx

        new_faces = np.empty((faces.shape[0] * 4, 3), dtype=np.int64)
        for i, (a, b, c) in enumerate(faces):
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            new_faces[4 * i + 0] = (a, ab, ca)
            new_faces[4 * i + 1] = (b, bc, ab)
            new_faces[4 * i + 2] = (c, ca, bc)
            new_faces[4 * i + 3] = (ab, bc, ca)
        faces = new_faces
    v = np.asarray(verts, dtype=np.float64) * radius
    return v, faces.astype(np.int32)


def vertex_normals(verts: np.ndarray, faces: np.ndarray) -> np.ndarray:
    """Area-weighted vertex normals (``compute_tensor_vert_normals``, mesh_utils.py:242-274)."""
    p0, p1, p2 = verts[faces[:, 0]], verts[faces[:, 1]], verts[faces[:, 2]]
    fn = np.cross(p1 - p0, p2 - p1)  # = 2 * area * unit normal
    vn = np.zeros_like(verts)
    for a in range(3):
        np.add.at(vn, faces[:, a], fn)
    return vn / np.linalg.norm(vn, axis=1, keepdims=True)


def mean_edge_length(verts: np.ndarray, faces: np.ndarray) -> float:
    e = np.concatenate(
        [verts[faces[:, 1]] - verts[faces[:, 0]],
         verts[faces[:, 2]] - verts[faces[:, 1]],
         verts[faces[:, 0]] - verts[faces[:, 2]]]
    )
    return float(np.linalg.norm(e, axis=1).mean())


def ellipsoid(level: int, axes=(1.0, 0.7, 0.5), jitter: float = 0.01, seed: int = 0):
    """Scaled icosphere with normal jitter N(0, jitter * mean edge length), seeded."""
    v, f = icosphere(level)
    v = v * np.asarray(axes, dtype=np.float64)[None, :]
    if jitter > 0:
        rng = np.random.default_rng(seed)
        n = vertex_normals(v, f)
        h = mean_edge_length(v, f)
        v = v + n * rng.normal(0.0, jitter * h, size=(v.shape[0], 1))
    return v, f


def _real_sph_harm(l: int, m: int, theta: np.ndarray, phi: np.ndarray) -> np.ndarray:
    """Real spherical harmonic Y_lm (orthonormal), theta polar, phi azimuth."""
    from scipy.special import lpmv

    am = abs(m)
    norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
    p = lpmv(am, l, np.cos(theta))
    if m > 0:
        return math.sqrt(2.0) * norm * p * np.cos(am * phi)
    if m < 0:
        return math.sqrt(2.0) * norm * p * np.sin(am * phi)
    return norm * p


def star_shape(level: int, seed: int = 0, n_terms: int = 6, lmax: int = 4, amp: float = 0.15):
    """Star-shaped closed surface r = 1 + sum_{i<6} a_i Y_{l_i m_i}, a_i ~ U(0, amp)."""
    v, f = icosphere(level)
    rng = np.random.default_rng(seed)
    theta = np.arccos(np.clip(v[:, 2], -1.0, 1.0))
    phi = np.arctan2(v[:, 1], v[:, 0])
    r = np.ones(v.shape[0])
    for _ in range(n_terms):
        l = int(rng.integers(0, lmax + 1))
        m = int(rng.integers(-l, l + 1))
        a = float(rng.uniform(0.0, amp))
        r += a * _real_sph_harm(l, m, theta, phi)
    return v * r[:, None], f


def fibonacci_lattice(n_rays: int) -> np.ndarray:
    """Unit directions on a Fibonacci lattice (``FibonacciLattice``, functions.py:1024-1054)."""
    golden = (1.0 + math.sqrt(5.0)) / 2.0
    if n_rays % 2 == 1:
        n_max, n_min = n_rays // 2, -(n_rays // 2)
    else:
        n_max, n_min = n_rays // 2 - 1, -(n_rays // 2)
    ns = np.linspace(n_min, n_max, n_rays)
    phis = 2.0 * math.pi * ns / golden
    thetas = np.arccos(2.0 * ns / n_rays)
    return np.stack(
        [np.sin(thetas) * np.cos(phis), np.sin(thetas) * np.sin(phis), np.cos(thetas)], axis=-1
    )
