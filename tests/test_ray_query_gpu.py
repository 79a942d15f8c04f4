"""GPU ray query (LBVH + closest-hit kernel) against the brute-force double oracle.

Acceptance per ray: the same face and distance within 2e-5 relative, or, where the float32
kernel and the double oracle pick different faces, a ray within 1e-4 (barycentric) of an
edge of either face or two hits at the same distance (see ray_scenes.compare_hits).  At full
size (a 524 288-face height field, 131 072 rays) the check is exact and size independent:
vertical rays over a grid hit the triangle under them at the height-field depth.
"""
import numpy as np
import pytest
import torch

import ray_scenes as S

pytestmark = pytest.mark.gpu


def _app(pkg, v, f):
    return pkg.ray_query.RayQueryApp(v.reshape(-1), f.reshape(-1).astype(np.uint32))


def test_scene_random_rays_match_oracle(pkg, cuda, oracle):
    v, f = S.scene_spheres_and_ground(3)
    app = _app(pkg, v, f)
    origins = np.array([[0, 0, 0], [0, -5, 2], [3, 3, 3], [2.5, 0.3, 0.2], [-4, 1, -1.0], [0, 0, 30]], np.float32)
    dirs = np.stack([S.random_dirs(2048, seed=s) for s in range(len(origins))])
    got = app.QueryForNLOS(origins.reshape(-1), dirs.reshape(-1))
    assert isinstance(got, np.ndarray) and got.dtype == np.float32 and got.shape == (len(origins) * 2048 * 4,)
    ref = oracle.ray_query(v, f, origins, dirs)
    n, mism, _ = S.compare_hits(v, f, origins, dirs, got, ref)
    assert mism <= 0.002 * n
    hits = (ref[..., 0] >= 0).mean()
    assert 0.2 < hits < 0.95  # the scene is neither empty nor closed around every origin
    assert app.status() == 0


def test_triangle_soup_matches_oracle(pkg, cuda, oracle):
    v, f = S.triangle_soup(20000, seed=3)
    app = _app(pkg, v, f)
    origins = np.array([[0, 0, 0], [8, 8, 8], [-2, 3, 1]], np.float32)
    dirs = np.stack([S.random_dirs(1500, seed=10 + s) for s in range(3)])
    got = app.QueryForNLOS(origins, dirs)
    ref = oracle.ray_query(v, f, origins, dirs)
    n, mism, _ = S.compare_hits(v, f, origins, dirs, got, ref)
    assert mism <= 0.002 * n
    assert app.status() == 0


def test_los_query_matches_oracle(pkg, cuda, oracle):
    v, f = S.scene_spheres_and_ground(2)
    app = _app(pkg, v, f)
    rng = np.random.default_rng(5)
    txs = rng.uniform(-4, 4, (7, 3)).astype(np.float32)
    rxs = rng.uniform(-4, 4, (7, 33, 3)).astype(np.float32)
    got = app.QueryForLOS(txs.reshape(-1).tolist(), rxs.reshape(-1).tolist())  # plain lists
    dirs = rxs - txs[:, None, :]
    ref = oracle.ray_query(v, f, txs, dirs)
    S.compare_hits(v, f, txs, dirs, got, ref)
    # device tensors stay on the device
    dev = app.QueryForLOS(torch.from_numpy(txs).cuda(), torch.from_numpy(rxs).cuda())
    assert dev.is_cuda and torch.equal(dev.cpu(), torch.from_numpy(np.asarray(got)))


def test_single_triangle_and_axis_aligned_rays(pkg, cuda, oracle):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    f = np.array([[0, 1, 2]], np.int32)
    app = _app(pkg, v, f)
    o = np.array([[0.2, 0.2, 1.0], [0.2, 0.2, -1.0], [0.9, 0.9, 1.0], [0.2, 0.2, 1.0]], np.float32)
    d = np.array([[[0, 0, -1]], [[0, 0, 1]], [[0, 0, -1]], [[0, 0, 1]]], np.float32)
    got = np.asarray(app.QueryForNLOS(o, d)).reshape(4, 4)
    np.testing.assert_array_equal(got[:, 0], [0, 0, -1, -1])
    np.testing.assert_allclose(got[:2, 3], [1.0, 1.0], rtol=1e-6)
    np.testing.assert_array_equal(got[2:, 3], [-1, -1])
    np.testing.assert_array_equal(got, oracle.ray_query(v, f, o, d).reshape(4, 4).astype(np.float32))


def test_coincident_faces_and_equal_keys(pkg, cuda, oracle):
    """Duplicated faces share Morton keys (index tie-break in the tree); ties keep the lower id."""
    v, f = S.grid(8, 8, -1.0, -1.0, 2.0)
    f2 = np.concatenate([f[::-1], f, f]).astype(np.int32)
    app = _app(pkg, v, f2)
    rng = np.random.default_rng(7)
    xy = rng.uniform(-0.99, 0.99, (500, 2))
    o = np.concatenate([xy, np.full((500, 1), 2.0)], 1).astype(np.float32)
    d = np.tile(np.array([0, 0, -1], np.float32), (500, 1, 1))
    got = np.asarray(app.QueryForNLOS(o, d)).reshape(500, 4)
    ref = oracle.ray_query(v, f2, o, d).reshape(500, 4)
    S.compare_hits(v, f2, o, d, got, ref)
    inside = got[:, 0] >= 0
    assert inside.mean() > 0.99
    assert np.all(got[inside, 0] < len(f))  # the reversed copy (lowest ids) always wins


def test_empty_queries_and_degenerate_rays(pkg, cuda):
    v, f = S.grid(4, 4)
    app = _app(pkg, v, f)
    z = app.query(torch.zeros(0, 3, device=cuda), torch.zeros(0, 5, 3, device=cuda))
    assert z.shape == (0, 5, 4)
    z = app.query(torch.zeros(3, 3, device=cuda), torch.zeros(3, 0, 3, device=cuda))
    assert z.shape == (3, 0, 4)
    # a zero direction normalises to NaN: no hit, no error
    r = app.query(torch.tensor([[0.3, 0.3, 1.0]], device=cuda), torch.zeros(1, 1, 3, device=cuda))
    assert r[0, 0, 0].item() == -1 and r[0, 0, 3].item() == -1
    assert app.status() == 0


def test_tmin_tmax(pkg, cuda, oracle):
    v, f = S.grid(4, 4, -1.0, -1.0, 2.0)
    app = _app(pkg, v, f)
    o = torch.tensor([[0.13, 0.21, 0.0], [0.13, 0.21, 0.5]], device=cuda)
    d = torch.tensor([[[0, 0, -1.0]], [[0, 0, -1.0]]], device=cuda)
    r = app.query(o, d)
    assert r[0, 0, 0].item() == -1 and r[1, 0, 0].item() >= 0
    assert app.query(o, d, tmax=0.4)[1, 0, 0].item() == -1
    assert app.query(o, d, tmin=0.6)[1, 0, 0].item() == -1


def test_full_size_height_field_exact(pkg, cuda):
    """512 x 512 cells (524 288 faces), 512 x 256 vertical rays: face and depth known exactly."""
    nx = ny = 512
    height = lambda X, Y: 0.05 * np.sin(3 * X) * np.cos(2 * Y)  # noqa: E731
    v, f = S.grid(nx, ny, 0.0, 0.0, 1.0, height=height)
    app = _app(pkg, v, f)
    rng = np.random.default_rng(11)
    n = 512 * 256
    cell = rng.integers(0, nx * ny, n)
    i, j = cell // ny, cell % ny
    a, b = rng.uniform(0.05, 0.9, n), rng.uniform(0.05, 0.9, n)
    keep = np.abs(a + b - 1) > 0.05
    x, y = (i + a) / nx, (j + b) / ny
    o = np.stack([x, y, np.full(n, 1.0)], 1).astype(np.float32)
    got = app.query(torch.from_numpy(o).cuda(),
                    torch.tensor([0, 0, -1.0], device=cuda).expand(n, 1, 3).contiguous()).cpu().numpy()
    face = S.grid_face_at(o[:, 0].astype(np.float64), o[:, 1].astype(np.float64), nx, ny)
    assert np.array_equal(got[keep, 0, 0].astype(np.int64), face[keep])
    # depth = 1 - plane height of that face at (x, y)
    tri = v[f[face[keep]]].astype(np.float64)
    nrm = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    px = o[keep].astype(np.float64)
    zp = tri[:, 0, 2] - (nrm[:, 0] * (px[:, 0] - tri[:, 0, 0]) + nrm[:, 1] * (px[:, 1] - tri[:, 0, 1])) / nrm[:, 2]
    np.testing.assert_allclose(got[keep, 0, 3], 1.0 - zp, atol=2e-6)
    assert app.status() == 0


def test_depth_map_helpers(pkg, cuda):
    RQ = pkg.ray_query
    verts, faces = pkg.meshes.icosphere(3, 2.0)
    app = RQ.initialize_vulkan_ray_querier(torch.tensor(verts, device=cuda), torch.tensor(faces, device=cuda))
    d, th, ph, _, _ = RQ.SampleSkydomRays(2 * 16 * 16, device=cuda)
    o = torch.tensor([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0], [0.0, 0.0, 9.0]], device=cuda)
    depth, face = RQ.GetRayQueryDepthMap(app, o, d, keepdim=False)
    assert depth.shape == (3, 512) and face.shape == (3, 512, 1) and face.dtype == torch.int32
    assert torch.all(face[:2] >= 0) and torch.all((depth[:2] > 1.4) & (depth[:2] < 2.6))
    assert torch.all((face[2] >= 0) == (depth[2] > 0).unsqueeze(-1))
