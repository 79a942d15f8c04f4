"""Host-side logic on the CPU: tables, mesh helpers, rule flattening, the C ABI surface."""
import ctypes
import importlib
import os
import re

import numpy as np
import pytest
import torch

from conftest import REPO, rel_err


def test_gauss_tables_match_reference(pkg, gauss_golden):
    U = pkg.utils
    prev = torch.get_default_dtype()
    torch.set_default_dtype(torch.float64)
    try:
        for n in (1, 2, 3, 4, 5, 6, 7, 8, 12):
            p, w = U.get_gaussion_integration_points_and_weights(n, dtype=torch.float64)
            assert np.abs(p.numpy() - gauss_golden[f"p{n}"]).max() < 1e-15
            assert np.abs(w.numpy() - gauss_golden[f"w{n}"]).max() < 1e-15
    finally:
        torch.set_default_dtype(prev)
    # with the default float32 dtype the reference's tables are float32-rounded before the
    # map to [0, 1] (done in the solver dtype)
    torch.set_default_dtype(torch.float32)
    p, _ = U.get_gaussion_integration_points_and_weights(4, dtype=torch.float64)
    x32 = (np.polynomial.legendre.leggauss(4)[0].astype(np.float32).astype(np.float64) + 1.0) / 2.0
    assert np.array_equal(p.numpy(), x32)
    torch.set_default_dtype(prev)
    with pytest.raises(NotImplementedError):
        U.get_gaussion_integration_points_and_weights(9)


@pytest.mark.parametrize("name", ["ico0", "ico1", "ell1"])
def test_mesh_helpers_match_reference(pkg, golden, name):
    U = pkg.utils
    g = golden[name]
    v = torch.tensor(g["verts"])
    f = torch.tensor(g["faces"])
    assert np.array_equal(U.compute_face_areas(v, f).numpy(), g["face_areas"])
    assert np.array_equal(U.compute_face_normals(v, f).numpy(), g["face_normals"])
    assert np.abs(U.compute_vert_areas(v, f).numpy() - g["vert_areas"]).max() < 1e-15
    edges, fei, adj = U.get_edge_unique(v, f)
    assert np.array_equal(edges.numpy(), g["edges"])
    assert np.array_equal(fei.numpy(), g["face_edge_indices"])
    assert np.array_equal(adj.numpy(), g["edge_adjacent_faces"])


def test_rule_table_reproduces_reference_panels(pkg, golden, oracle):
    """The flattened sub-domain table, walked on the host, reproduces the reference's V."""
    U = pkg.utils
    g = golden["ico0"]
    rands = torch.tensor(g["lap_gq2_o1_rands"])
    w = torch.tensor(g["lap_gq2_o1_weights"])
    table, seg = U.panel_rule_table(rands, rands, w, w)
    assert seg[0] == 0 and seg[-1] == table.shape[0] == 16 * (1 + 2 + 5 + 3)
    tab = table.numpy()
    verts, faces, areas = g["verts"], g["faces"], g["face_areas"].reshape(-1)
    rel = g["panel_relations"]
    out = np.zeros((20, 20, 3, 3))
    for fy in range(20):
        Y = verts[faces[fy]]
        for fx in range(20):
            X = verts[faces[fx]]
            r = rel[fy, fx]
            t = tab[seg[r]:seg[r + 1]]
            x = (1 - t[:, 0:1]) * X[0] + (t[:, 0:1] - t[:, 1:2]) * X[1] + t[:, 1:2] * X[2]
            y = (1 - t[:, 2:3]) * Y[0] + (t[:, 2:3] - t[:, 3:4]) * Y[1] + t[:, 3:4] * Y[2]
            G = 1 / (4 * np.pi * np.linalg.norm(x - y, axis=1))
            py = np.stack([1 - t[:, 2], t[:, 2] - t[:, 3], t[:, 3]], 1)
            px = np.stack([1 - t[:, 0], t[:, 0] - t[:, 1], t[:, 1]], 1)
            out[fy, fx] = np.einsum("q,qa,qb->ab", G * t[:, 4], py, px) * 4 * areas[fy] * areas[fx]
    assert rel_err(out, g["lap_gq2_o1_V_unpacked"]) < 1e-12


def test_meshes_are_closed_and_outward(pkg):
    for lvl in range(4):
        v, f = pkg.meshes.icosphere(lvl)
        assert f.shape[0] == 20 * 4 ** lvl and v.shape[0] == 10 * 4 ** lvl + 2
        vt, ft = torch.tensor(v), torch.tensor(f)
        edges, fei, adj = pkg.utils.get_edge_unique(vt, ft)
        assert edges.shape[0] == 30 * 4 ** lvl
        counts = np.bincount(fei.numpy(), minlength=edges.shape[0])
        assert np.all(counts == 2)
        n = pkg.utils.compute_face_normals(vt, ft).numpy()
        c = v[f].mean(axis=1)
        assert np.all((n * c).sum(1) > 0)
    v, f = pkg.meshes.ellipsoid(2, seed=0)
    v2, _ = pkg.meshes.ellipsoid(2, seed=0)
    assert np.array_equal(v, v2)
    v, f = pkg.meshes.star_shape(2, seed=5)
    r = np.linalg.norm(v, axis=1)
    assert r.min() > 0.3 and np.isfinite(r).all()
    d = pkg.meshes.fibonacci_lattice(256)
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0)


def _header_symbols():
    hdr = open(os.path.join(REPO, "include", "mesh_bem_gb300.h")).read()
    return sorted(set(re.findall(r"\b(mb_[a-z0-9_]+)\s*\(", hdr)))


def test_capi_library_exports_header_symbols(pkg):
    from importlib import import_module

    build = import_module("mesh-ferrofluid_gb300.build")
    if not os.path.exists(build.LIB):
        build.build()
    lib = ctypes.CDLL(build.LIB)
    syms = _header_symbols()
    assert len(syms) >= 19
    for s in syms:
        assert hasattr(lib, s), s
    lib.mb_abi_version.restype = ctypes.c_int
    assert lib.mb_abi_version() == 1
    # the Python binding declares exactly the header's entry points
    from importlib import import_module as im

    bound = set(im("mesh-ferrofluid_gb300._lib").exported_symbols())
    assert bound == set(syms)


def test_ops_reject_cpu_tensors(pkg):
    """No CPU fallback: host tensors are refused before any launch."""
    v = torch.zeros((3, 3))
    f = torch.zeros((1, 3), dtype=torch.int32)
    a = torch.ones((1, 1))
    n = torch.zeros((1, 3))
    p, w = pkg.utils.get_gaussion_integration_points_and_weights(2)
    z = torch.zeros((1, 3, 3))
    with pytest.raises(ValueError, match="CUDA"):
        pkg.mesh_MOM_3d.create_MOM_Zmat_3d_forward(v, f, a, n, p, w, p, w, z, z.clone(), 1.0)


def test_shared_vertex_pairs_equal_dense_relation(pkg):
    """The O(F) near-pair builder returns exactly the nonzeros of the dense shared-vertex
    relation, in row-major order (closed meshes, a non-manifold fan and an empty mesh)."""
    meshes = [pkg.meshes.icosphere(2), pkg.meshes.star_shape(2, seed=4), pkg.meshes.ellipsoid(1),
              (None, np.array([[0, 1, 2], [1, 0, 3], [0, 1, 4], [5, 6, 7]], np.int32))]
    for _, f in meshes:
        got = pkg.utils.shared_vertex_pairs(torch.tensor(f, dtype=torch.int32)).numpy()
        dense = np.zeros((f.shape[0], f.shape[0]), bool)
        for a in range(3):
            for b in range(3):
                dense |= f[:, a][:, None] == f[:, b][None, :]
        assert np.array_equal(got, np.argwhere(dense))
    assert pkg.utils.shared_vertex_pairs(torch.zeros((0, 3), dtype=torch.int32)).shape == (0, 2)


def test_schur_solve_matches_dense_block_solve(pkg):
    """The mixed block system [[V, -B], [B^T, D]] solved by Cholesky factors (solver="schur")."""
    m = importlib.import_module("mesh-ferrofluid_gb300.mesh_BEM_solver_3d")
    g = torch.Generator().manual_seed(0)
    nd, nn = 30, 20
    X = torch.randn(nd, nd, generator=g, dtype=torch.float64)
    Y = torch.randn(nn, nn, generator=g, dtype=torch.float64)
    V = X @ X.T + nd * torch.eye(nd, dtype=torch.float64)
    D = Y @ Y.T + torch.eye(nn, dtype=torch.float64)
    B = torch.randn(nd, nn, generator=g, dtype=torch.float64)
    r1 = torch.randn(nd, generator=g, dtype=torch.float64)
    r2 = torch.randn(nn, generator=g, dtype=torch.float64)
    A = torch.cat((torch.cat((V, -B), 1), torch.cat((B.T, D), 1)), 0)
    x = torch.linalg.solve(A, torch.cat((r1, r2)))
    assert (m._schur_solve(V, B, D, r1, r2) - x).abs().max().item() < 1e-12
    assert (m._spd_solve(V, r1) - torch.linalg.solve(V, r1)).abs().max().item() < 1e-12
    with pytest.raises(RuntimeError):
        m._spd_solve(-V, r1)


def test_rule_table_cache_keys_on_values(pkg):
    """The flattened sub-domain rule table is reused for equal rules (even new tensors) and
    rebuilt when a rule value, the dtype or the rule size changes."""
    L, U = pkg.layers, pkg.utils

    def rule(q, dt):
        p, w1 = U.get_gaussion_integration_points_and_weights(q, device="cpu", dtype=dt)
        r, w = U.collapsed_rule_2d(p, w1)
        return r, w

    r, w = rule(2, torch.float64)
    t1, s1 = L._cached_rule_table(r, r, w, w, torch.float64, torch.device("cpu"))
    t2, s2 = L._cached_rule_table(r.clone(), r.clone(), w.clone(), w.clone(), torch.float64, torch.device("cpu"))
    assert t2 is t1 and s2 == s1
    ref, seg = U.panel_rule_table(r, r, w, w)
    assert torch.equal(t1, ref) and s1 == seg
    r2 = r.clone()
    r2[0, 0] += 1e-3
    t3, _ = L._cached_rule_table(r2, r2, w, w, torch.float64, torch.device("cpu"))
    assert t3 is not t1 and torch.equal(t3, U.panel_rule_table(r2, r2, w, w)[0])
    t4, _ = L._cached_rule_table(r, r, w, w, torch.float32, torch.device("cpu"))
    assert t4.dtype == torch.float32
    r3, w3 = rule(3, torch.float64)
    t5, s5 = L._cached_rule_table(r3, r3, w3, w3, torch.float64, torch.device("cpu"))
    assert t5.shape[0] != t1.shape[0] and s5 == U.panel_rule_table(r3, r3, w3, w3)[1]
    # an in-place change of a rule tensor already found by identity rebuilds the table
    r4 = r.clone()
    t6, _ = L._cached_rule_table(r4, r4, w, w, torch.float64, torch.device("cpu"))
    assert t6 is t1
    r4[1, 1] += 1e-3
    t7, _ = L._cached_rule_table(r4, r4, w, w, torch.float64, torch.device("cpu"))
    assert t7 is not t1 and torch.equal(t7, U.panel_rule_table(r4, r4, w, w)[0])


def test_face_range_check_is_cached_per_tensor_version(pkg):
    """check_face_range reduces a face tensor once, then trusts it until it is modified in
    place (its version counter moves) or checked against another vertex count."""
    M = pkg.mesh_MOM_3d
    f = torch.tensor([[0, 1, 2], [2, 1, 3]], dtype=torch.int32)
    M.check_face_range(f, 4)
    M.check_face_range(f, 4)
    with pytest.raises(ValueError):
        M.check_face_range(f, 3)
    f[1, 2] = 7
    with pytest.raises(ValueError):
        M.check_face_range(f, 4)
    f[1, 2] = -1
    with pytest.raises(ValueError):
        M.check_face_range(f, 8)
