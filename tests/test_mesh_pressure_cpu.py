"""Geometry helpers of the pressure projection (cotangent Laplacian, surface gradients)."""
import numpy as np
import torch


def test_cot_laplacian_flat_patch_and_sphere(pkg):
    U = pkg.utils
    # flat regular grid: the cotangent Laplacian of the coordinates vanishes at interior vertices
    n = 6
    xs = np.linspace(0, 1, n + 1)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    v = torch.tensor(np.stack([X, Y, 0 * X], -1).reshape(-1, 3))
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a = (i * (n + 1) + j).ravel()
    f = torch.tensor(np.concatenate([np.stack([a, a + n + 1, a + 1], 1), np.stack([a + n + 1, a + n + 2, a + 1], 1)]))
    L, inv = U.cot_laplacian(v, f)
    Ld = L.to_dense()
    assert torch.allclose(Ld, Ld.T)
    lap = Ld @ v - Ld.sum(1, keepdim=True) * v
    interior = ((v[:, 0] > 0) & (v[:, 0] < 1) & (v[:, 1] > 0) & (v[:, 1] < 1))
    assert lap[interior].abs().max() < 1e-12
    # right isoceles triangles: cot of the 45-degree angles is 1, of the right angle 0
    assert set(np.round(np.unique(Ld.numpy()[Ld.numpy() != 0]), 12)) <= {1.0, 2.0}
    # inverse areas: interior vertex touches 6 triangles of area 1/(2 n^2)
    k = int(np.nonzero(interior.numpy())[0][0])
    assert abs(inv[k, 0].item() - 1.0 / (6 * 0.5 / n ** 2)) < 1e-9


def test_signed_mean_curvature_on_sphere(pkg):
    """The reference's formula gives -H/3 on a sphere (areas of whole incident faces, L x inward)."""
    v, f = pkg.meshes.icosphere(3, 2.0)
    v, f = torch.tensor(v), torch.tensor(f)
    mp = pkg.MeshPressure.__new__(pkg.MeshPressure)
    k = pkg.MeshPressure.signed_mean_curvature(mp, v, f, pkg.utils.compute_vert_normals(v, f))
    assert abs(k.mean().item() + 0.5 / 3) < 0.003 and k.std().item() < 0.01


def test_tangent_gradient_exact_for_linear_data(pkg):
    U = pkg.utils
    v, f = pkg.meshes.icosphere(2, 1.0)
    v, f = torch.tensor(v), torch.tensor(f)
    g = torch.tensor([0.3, -1.2, 0.7], dtype=torch.float64)
    p = (v @ g).reshape(1, -1, 1)
    fg = U.compute_mesh_face_tangent_gradient(p, v, f)[0]
    n = U.compute_face_normals(v, f)
    expect = g - (n @ g)[:, None] * n  # tangential part of the constant gradient
    assert (fg - expect).abs().max() < 1e-12
    vg = U.compute_mesh_vert_tangent_gradient(p, v, f)
    assert vg.shape == (1, v.shape[0], 3)
