"""Test scenes and checks for the closest-hit ray query (test infrastructure).

Scenes are triangle meshes in numpy (float32 vertices as the plugin takes them, int32
faces).  ``compare_hits`` accepts a GPU result against the double-precision brute-force
oracle: equal faces with distances within ``rtol``, or, where the faces differ, a ray that
passes within ``edge_tol`` (barycentric) of an edge of the face either side reports, or two
hits at the same distance (adjacent faces along a shared edge).
"""
from __future__ import annotations

import importlib
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def _meshes():
    return importlib.import_module("mesh-ferrofluid_gb300").meshes


def grid(nx, ny, x0=0.0, y0=0.0, size=1.0, height=None):
    """Regular grid of 2 nx ny triangles on [x0, x0+size] x [y0, y0+size]; z = height(x, y)."""
    xs = x0 + size * np.arange(nx + 1) / nx
    ys = y0 + size * np.arange(ny + 1) / ny
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    Z = np.zeros_like(X) if height is None else height(X, Y)
    verts = np.stack([X, Y, Z], -1).reshape(-1, 3)
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    v00 = (i * (ny + 1) + j).ravel()
    v10 = ((i + 1) * (ny + 1) + j).ravel()
    v01 = (i * (ny + 1) + j + 1).ravel()
    v11 = ((i + 1) * (ny + 1) + j + 1).ravel()
    # cell (i, j) -> faces 2 (i ny + j) (lower-left, x' + y' < 1) and 2 (i ny + j) + 1
    faces = np.stack([np.stack([v00, v10, v01], -1), np.stack([v10, v11, v01], -1)], 1).reshape(-1, 3)
    return verts.astype(np.float32), faces.astype(np.int32)


def grid_face_at(x, y, nx, ny, x0=0.0, y0=0.0, size=1.0):
    """Face of ``grid`` under the point (x, y) (points strictly inside a triangle)."""
    u = (x - x0) / size * nx
    v = (y - y0) / size * ny
    i = np.floor(u).astype(np.int64)
    j = np.floor(v).astype(np.int64)
    upper = (u - i) + (v - j) > 1.0
    return 2 * (i * ny + j) + upper


def merge(*parts):
    verts, faces, off = [], [], 0
    for v, f in parts:
        verts.append(np.asarray(v, np.float32))
        faces.append(np.asarray(f, np.int64) + off)
        off += len(v)
    return np.concatenate(verts), np.concatenate(faces).astype(np.int32)


def scene_spheres_and_ground(level=3):
    """Unit icosphere at the origin, an ellipsoid beside it and a ground grid below."""
    M = _meshes()
    v1, f1 = M.icosphere(level, 1.0)
    v2, f2 = M.ellipsoid(level - 1)
    v2 = v2 * 0.8 + np.array([2.5, 0.3, 0.2])
    v3, f3 = grid(40, 40, -6.0, -6.0, 12.0)
    v3 = v3 + np.array([0.0, 0.0, -1.5], np.float32)
    return merge((v1, f1), (v2, f2), (v3, f3))


def triangle_soup(n, seed=0, box=10.0, size=0.3):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-box / 2, box / 2, (n, 1, 3))
    v = (c + rng.normal(scale=size, size=(n, 3, 3))).reshape(-1, 3)
    return v.astype(np.float32), np.arange(3 * n, dtype=np.int32).reshape(n, 3)


def random_dirs(n, seed=0):
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    return (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)


def hit_margin(verts, faces, o, d, f):
    """Smallest barycentric coordinate of the ray / plane-of-face point (double)."""
    v = np.asarray(verts, np.float64)
    tri = v[np.asarray(faces)[f]]
    o = np.asarray(o, np.float64)
    d = np.asarray(d, np.float64)
    d = d / np.linalg.norm(d, axis=-1, keepdims=True)
    e1 = tri[:, 1] - tri[:, 0]
    e2 = tri[:, 2] - tri[:, 0]
    p = np.cross(d, e2)
    det = np.einsum("ij,ij->i", e1, p)
    det = np.where(np.abs(det) < 1e-300, 1e-300, det)
    s = o - tri[:, 0]
    u = np.einsum("ij,ij->i", s, p) / det
    q = np.cross(s, e1)
    w = np.einsum("ij,ij->i", d, q) / det
    return np.minimum(np.minimum(u, w), 1.0 - u - w)


def compare_hits(verts, faces, origins, dirs, got, ref, rtol=2e-5, edge_tol=1e-4, max_bad_frac=0.0):
    """Returns (n_rays, n_face_mismatch, n_unexplained); asserts distance agreement."""
    got = np.asarray(got, np.float64).reshape(-1, 4)
    ref = np.asarray(ref, np.float64).reshape(-1, 4)
    h = np.asarray(origins).reshape(-1, 3).shape[0]
    w = got.shape[0] // h
    o = np.repeat(np.asarray(origins, np.float64).reshape(h, 1, 3), w, 1).reshape(-1, 3)
    d = np.asarray(dirs, np.float64).reshape(-1, 3)
    fg, fr = got[:, 0].astype(np.int64), ref[:, 0].astype(np.int64)
    assert np.all((got[:, 1] == 0) & (got[:, 2] == 0))
    assert np.all((fg >= 0) == (got[:, 3] > 0)) and np.all(got[fg < 0, 3] == -1)
    same = fg == fr
    hit = same & (fg >= 0)
    scale = np.maximum(1.0, ref[hit, 3])
    assert np.all(np.abs(got[hit, 3] - ref[hit, 3]) <= rtol * scale), "distance mismatch on equal faces"
    bad = np.nonzero(~same)[0]
    unexplained = 0
    for r in bad:
        both = fg[r] >= 0 and fr[r] >= 0
        if both and abs(got[r, 3] - ref[r, 3]) <= rtol * max(1.0, ref[r, 3]):
            continue  # same distance: a shared edge / vertex or coincident faces
        edge = False
        for f in (fg[r], fr[r]):
            if f >= 0 and hit_margin(verts, faces, o[r:r + 1], d[r:r + 1], np.array([f]))[0] < edge_tol:
                edge = True
        if not edge:
            unexplained += 1
    assert unexplained <= max_bad_frac * len(fg), f"{unexplained} of {len(fg)} rays disagree off edges"
    return len(fg), len(bad), unexplained
