"""The ray-query oracle (brute-force Moller-Trumbore in double) pinned by known answers.

The reference's own ray query runs through Vulkan ray-tracing shaders, which cannot run on
these machines, so the oracle is pinned analytically: flat and height-field grids hit from
above (face and distance known in closed form), rays from the centre of a closed icosphere
(every ray hits, at the plane distance of its face), tMin / tMax, ties between coincident
faces, and misses.
"""
import numpy as np
import pytest

import ray_scenes as S


def test_grid_from_above_known_faces_and_depths(oracle):
    nx, ny = 16, 12
    v, f = S.grid(nx, ny, -1.0, -1.0, 2.0)
    rng = np.random.default_rng(1)
    xy = rng.uniform(-0.999, 0.999, (300, 2))
    # keep points away from cell diagonals and cell borders
    u, w = (xy[:, 0] + 1) / 2 * nx, (xy[:, 1] + 1) / 2 * ny
    ok = (np.abs((u % 1) + (w % 1) - 1) > 1e-3) & ((u % 1) > 1e-3) & ((w % 1) > 1e-3)
    xy = xy[ok]
    h = rng.uniform(0.5, 3.0, len(xy))
    origins = np.concatenate([xy, h[:, None]], 1)
    dirs = np.tile(np.array([0.0, 0.0, -1.0]), (len(xy), 1, 1))
    out = oracle.ray_query(v, f, origins, dirs)
    assert out.shape == (len(xy), 1, 4)
    np.testing.assert_array_equal(out[:, 0, 0], S.grid_face_at(xy[:, 0], xy[:, 1], nx, ny, -1.0, -1.0, 2.0))
    np.testing.assert_allclose(out[:, 0, 3], h, rtol=1e-12)
    assert np.all(out[:, 0, 1:3] == 0)


def test_height_field_depths(oracle):
    nx = ny = 20
    v, f = S.grid(nx, ny, 0.0, 0.0, 1.0, height=lambda X, Y: 0.3 * X + 0.2 * Y)  # planar: exact
    xy = np.array([[0.111, 0.523], [0.77, 0.31], [0.5013, 0.9871]])
    origins = np.concatenate([xy, np.full((3, 1), 2.0)], 1)
    out = oracle.ray_query(v, f, origins, np.tile([0.0, 0.0, -7.0], (3, 1, 1)))  # unnormalised dir
    np.testing.assert_allclose(out[:, 0, 3], 2.0 - (0.3 * xy[:, 0] + 0.2 * xy[:, 1]), rtol=1e-6)


def test_icosphere_from_centre_every_ray_hits_its_face(oracle, pkg):
    v, f = pkg.meshes.icosphere(2, 1.0)
    d = S.random_dirs(400, seed=2)
    out = oracle.ray_query(v, f, np.zeros((1, 3)), d[None])
    fi = out[0, :, 0].astype(np.int64)
    assert np.all(fi >= 0)
    tri = v[f[fi]].astype(np.float64)
    d = d.astype(np.float64)
    d /= np.linalg.norm(d, axis=1, keepdims=True)  # the query normalises its directions
    n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    t = np.einsum("ij,ij->i", n, tri[:, 0]) / np.einsum("ij,ij->i", n, d)
    np.testing.assert_allclose(out[0, :, 3], t, rtol=1e-12)
    assert np.all(S.hit_margin(v, f, np.zeros((400, 3)), d, fi) >= -1e-12)


def test_tmin_tmax_and_misses(oracle):
    v, f = S.grid(4, 4, -1.0, -1.0, 2.0)
    o = np.array([[0.13, 0.21, 0.0], [0.13, 0.21, 0.5], [0.13, 0.21, 0.5], [5.0, 5.0, 1.0]])
    d = np.array([[[0, 0, -1.0]], [[0, 0, 1.0]], [[0, 0, -1.0]], [[0, 0, -1.0]]])
    out = oracle.ray_query(v, f, o, d)
    assert out[0, 0, 0] == -1 and out[0, 0, 3] == -1   # origin on the surface: t = 0 < tMin
    assert out[1, 0, 0] == -1                           # pointing away
    assert out[2, 0, 0] >= 0 and out[2, 0, 3] == pytest.approx(0.5)
    assert out[3, 0, 0] == -1                           # beside the grid
    near = oracle.ray_query(v, f, o[2:3], d[2:3], tmax=0.4)
    assert near[0, 0, 0] == -1


def test_coincident_faces_tie_to_lower_index(oracle):
    v, f = S.grid(2, 2)
    f2 = np.concatenate([f[::-1], f])  # every face twice; duplicates come later in the list
    out = oracle.ray_query(v, f2, np.array([[0.2, 0.1, 1.0]]), np.array([[[0, 0, -1.0]]]))
    assert int(out[0, 0, 0]) == len(f) - 1 - int(S.grid_face_at(0.2, 0.1, 2, 2))
