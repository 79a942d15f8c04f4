"""GPU near-pair list (mb_shared_vertex_pairs_*) against the dense shared-vertex relation:
the ordered face pairs sharing a vertex, sorted by first face then second, bit-exact."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _dense_pairs(f):
    dense = np.zeros((f.shape[0], f.shape[0]), bool)
    for a in range(3):
        for b in range(3):
            dense |= f[:, a][:, None] == f[:, b][None, :]
    return np.argwhere(dense).astype(np.int32)


def _cases(pkg):
    rng = np.random.default_rng(7)
    ico = pkg.meshes.icosphere(3)[1]
    perm = ico[rng.permutation(ico.shape[0])]
    # a fan of 300 faces around vertex 0 (valence far above a surface mesh's)
    n = 300
    fan = np.stack([np.zeros(n, np.int64), 1 + np.arange(n), 1 + (np.arange(n) + 1) % n], 1).astype(np.int32)
    degenerate = np.array([[0, 1, 2], [1, 0, 3], [0, 1, 4], [5, 6, 7], [2, 2, 3], [8, 9, 9]], np.int32)
    return [ico, perm, pkg.meshes.star_shape(2, seed=4)[1], pkg.meshes.ellipsoid(1)[1], fan, degenerate]


def test_near_pairs_match_dense_relation(pkg, cuda):
    for f in _cases(pkg):
        ft = torch.tensor(f, dtype=torch.int32, device=cuda)
        got = pkg.utils.shared_vertex_pairs(ft, int(f.max()) + 1)
        assert got.dtype == torch.int32 and got.is_cuda
        assert np.array_equal(got.cpu().numpy(), _dense_pairs(f))
        # unused trailing vertices and the default vertex count give the same list
        assert torch.equal(pkg.utils.shared_vertex_pairs(ft, int(f.max()) + 11), got)
        assert torch.equal(pkg.utils.shared_vertex_pairs(ft), got)


def test_near_pairs_full_size_properties(pkg, cuda):
    """icosphere L6 (81 920 faces): every face paired with itself, rows sorted and unique,
    the list symmetric, and each face of a closed triangle mesh with valence-6 vertices has
    1 + 3 + 9 neighbours (self, edge and vertex neighbours) except near the 12 valence-5
    vertices."""
    f = pkg.meshes.icosphere(6)[1]
    ft = torch.tensor(f, dtype=torch.int32, device=cuda)
    p = pkg.utils.shared_vertex_pairs(ft, int(f.max()) + 1).cpu().numpy().astype(np.int64)
    key = p[:, 0] * f.shape[0] + p[:, 1]
    assert np.all(np.diff(key) > 0)
    assert np.array_equal(np.sort(p[:, 1] * f.shape[0] + p[:, 0]), key)
    assert np.all(np.isin(np.arange(f.shape[0]) * (f.shape[0] + 1), key))
    counts = np.bincount(p[:, 0], minlength=f.shape[0])
    assert np.median(counts) == 13 and counts.min() >= 11


def test_near_pairs_reject_bad_ids(pkg, cuda):
    ft = torch.tensor([[0, 1, 2], [1, 2, 7]], dtype=torch.int32, device=cuda)
    with pytest.raises(Exception, match="outside"):
        pkg.utils.shared_vertex_pairs(ft, 5)
    assert pkg.utils.shared_vertex_pairs(torch.zeros((0, 3), dtype=torch.int32, device=cuda), 4).shape == (0, 2)
