"""The symmetric-rule Laplace oracle pinned by the sphere's analytic spectra and solutions.

On the unit sphere the spherical harmonics of degree l are eigenfunctions of the boundary
operators: V Y = Y/(2l+1), K Y = -Y/(2(2l+1)) (interior trace convention of the
reference's double layer n_y.(x - y)/(4 pi R^3)), D Y = l(l+1)/(2l+1) Y.  With u = z
(l = 1, harmonic inside, du/dn = z) the Dirichlet, Neumann and mixed problems have known
solutions, and the single-layer collocation system V sigma = 1 has sigma = 1/a.  The
oracle (oracle/mesh_bem_oracle.c, double) must converge to all of these.
"""
import numpy as np
import pytest


def _pack(M, f, nv):
    P = np.zeros((nv, nv))
    np.add.at(P, (f[:, None, :, None], f[None, :, None, :]), M)
    return P


def _operators(pkg, oracle, level):
    v, f = pkg.meshes.icosphere(level, 1.0)
    nv = v.shape[0]
    V = _pack(oracle.laplace_sym(v, f, 1, 1), f, nv)
    K = _pack(oracle.laplace_sym(v, f, 2, 1), f, nv)
    V0 = oracle.laplace_sym(v, f, 1, 0)[:, :, 0, 0]
    p0, p1, p2 = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    a = 0.5 * np.linalg.norm(np.cross(p1 - p0, p2 - p1), axis=1)
    c = np.stack([p1 - p2, p2 - p0, p0 - p1], 1) / (2 * a[:, None, None])
    D = _pack(np.einsum("yad,xbd->yxab", c, c) * V0[:, :, None, None], f, nv)
    M = np.zeros((nv, nv))
    np.add.at(M, (f[:, :, None], f[:, None, :]), a[:, None, None] * (np.ones((3, 3)) + np.eye(3)) / 12)
    return v, f, V, K, D, M


@pytest.fixture(scope="module")
def ops(pkg, oracle):
    return {lv: _operators(pkg, oracle, lv) for lv in (1, 2)}


def test_spectra_on_sphere(ops):
    errs = []
    for lv in (1, 2):
        v, f, V, K, D, M = ops[lv]
        z = v[:, 2]
        zz = z @ M @ z
        e = [abs(z @ V @ z / zz - 1 / 3) * 3, abs(z @ K.T @ z / zz + 1 / 6) * 6, abs(z @ D @ z / zz - 2 / 3) * 1.5]
        errs.append(e)
        assert np.abs(V - V.T).max() < 3e-5 * np.abs(V).max()  # near pairs: inner closed form, outer rule
        assert np.abs(D.sum(1)).max() < 1e-12  # D annihilates constants exactly
        one = np.ones(len(z))
        np.testing.assert_allclose(K.T @ one, -0.5 * (M @ one), rtol=1e-4)  # Gauss: K 1 = -1/2
    assert max(errs[1]) < 0.02
    assert all(b <= a for a, b in zip(errs[0], errs[1]))  # converging


def test_dirichlet_neumann_mixed_solutions(ops):
    v, f, V, K, D, M = ops[2]
    z = v[:, 2]
    Ks = K.T
    t = np.linalg.solve(V, 0.5 * M @ z + Ks @ z)
    assert np.linalg.norm(t - z) / np.linalg.norm(z) < 0.025
    a = M @ np.ones(len(z))
    u = np.linalg.solve(D + np.outer(a, a), 0.5 * M @ z - Ks.T @ z)
    assert np.linalg.norm(u - z) / np.linalg.norm(z) < 0.03
    d = z > 0
    n = ~d
    A = np.block([[V[np.ix_(d, d)], -Ks[np.ix_(d, n)]], [Ks.T[np.ix_(n, d)], D[np.ix_(n, n)]]])
    g, fn = np.where(d, z, 0.0), np.where(n, z, 0.0)
    x = np.linalg.solve(A, np.concatenate([(0.5 * M @ g + Ks @ g - V @ fn)[d], (0.5 * M @ fn - Ks.T @ fn - D @ g)[n]]))
    assert np.linalg.norm(x[d.sum():] - z[n]) / np.linalg.norm(z[n]) < 0.02
    far = d & (z > 0.3)  # away from the Dirichlet / Neumann interface
    assert np.linalg.norm(x[:d.sum()][far[d]] - z[far]) / np.linalg.norm(z[far]) < 0.1


def test_collocation_sphere_density(pkg, oracle):
    for lv, tol in ((1, 0.05), (2, 0.02)):
        v, f = pkg.meshes.icosphere(lv, 2.0)
        C = oracle.laplace_colloc_sl(v, f)
        sig = np.linalg.solve(C, np.ones(f.shape[0]))
        assert np.abs(sig * 2.0 - 1).max() < tol  # sigma = 1/a


def test_dl_closed_form_matches_quadrature_far_away(pkg, oracle):
    """Off-surface the near formulas must agree with the 7-point rule on a distant pair."""
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [5, 5, 3], [6, 5, 3.2], [5, 6, 2.7]], float)
    f = np.array([[0, 1, 2], [3, 4, 5]], np.int32)
    # faces do not share a vertex: the oracle uses 7 x 7 points; check against a fine rule
    out = oracle.laplace_sym(v, f, 2, 1)[1, 0]
    # brute force: 40 x 40 midpoint rule in barycentric sub-triangles
    def pts(P, n):
        xs, ws, bs = [], [], []
        for i in range(n):
            for j in range(n - i):
                for up in (0, 1):
                    if up and i + j == n - 1:
                        continue
                    b = np.array([(i + (1 + up) / 3) / n, (j + (1 + up) / 3) / n]) if not up else \
                        np.array([(i + 2 / 3) / n, (j + 2 / 3) / n])
                    xs.append(P[0] + b[0] * (P[1] - P[0]) + b[1] * (P[2] - P[0]))
                    bs.append([1 - b[0] - b[1], b[0], b[1]])
        A = 0.5 * np.linalg.norm(np.cross(P[1] - P[0], P[2] - P[0]))
        return np.array(xs), np.full(len(xs), A / len(xs)), np.array(bs)
    Y, wy, by = pts(v[f[1]], 40)
    X, wx, bx = pts(v[f[0]], 40)
    ny = np.cross(v[4] - v[3], v[5] - v[4]); ny /= np.linalg.norm(ny)
    d = X[None, :, :] - Y[:, None, :]
    R = np.linalg.norm(d, axis=-1)
    k = (d @ ny) / (4 * np.pi * R ** 3)
    ref = np.einsum("y,ya,yx,x,xb->ab", wy, by, k, wx, bx)
    np.testing.assert_allclose(out, ref, rtol=2e-3)
