"""GPU parity of the Laplace single/double-layer path against the reference's own results.

The golden fixtures come from the reference's ``MeshBEMSolver3d.solve`` run in float64
(tests/golden/make_golden.py).  Tolerances: 1e-10 (float64), 1e-5 (float32 vs float64
oracle), relative Frobenius.
"""
import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _mesh(g, dev, dt):
    v = torch.tensor(g["verts"], dtype=dt, device=dev)
    f = torch.tensor(g["faces"], dtype=torch.int32, device=dev)
    a = torch.tensor(g["face_areas"], dtype=dt, device=dev)
    n = torch.tensor(g["face_normals"], dtype=dt, device=dev)
    return v, f, a, n


CASES = [("ico0", 2, 1), ("ico0", 3, 1), ("ico0", 2, 0), ("ell1", 2, 1)]


@pytest.mark.parametrize("name,gq,order", CASES)
@pytest.mark.parametrize("layer", [1, 2])
def test_panels_f64_match_reference(pkg, cuda, golden, name, gq, order, layer):
    g = golden[name]
    v, f, a, n = _mesh(g, cuda, torch.float64)
    tag = f"lap_gq{gq}_o{order}"
    rands = torch.tensor(g[f"{tag}_rands"], device=cuda)
    w = torch.tensor(g[f"{tag}_weights"], device=cuda)
    rel = torch.tensor(g["panel_relations"], device=cuda)
    out = pkg.double_integration_on_panels_3d(int(pkg.BEMType.LAPLACE), order, v, f, a, n, w, w, rands,
                                              rands, rel, 1.0, layer)
    key = f"{tag}_{'V' if layer == 1 else 'K'}_unpacked"
    got = out.cpu().numpy()
    if key in g:
        assert rel_err(got, g[key]) < 1e-10
    elif key + "_rows" in g:
        ref = g[key + "_rows"]
        assert rel_err(got[: ref.shape[0]], ref) < 1e-10
    fro = float(g[f"{tag}_{'V' if layer == 1 else 'K'}_fro"])
    assert abs(np.linalg.norm(got) / fro - 1) < 1e-10
    # packing (pack_matrix_tight) of the same matrix
    packed = pkg.utils.pack_matrix_tight(order, out, v, f).cpu().numpy()
    assert rel_err(packed, g[f"{tag}_{'V' if layer == 1 else 'K'}_packed"]) < 1e-10


@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
def test_panels_relation_derived_on_device(pkg, cuda, golden, dt):
    g = golden["ell1"]
    v, f, a, n = _mesh(g, cuda, dt)
    rel = pkg.utils.compute_panel_relation(f)
    assert np.array_equal(rel.cpu().numpy(), g["panel_relations"])
    rands = torch.tensor(g["lap_gq2_o1_rands"], device=cuda, dtype=dt)
    w = torch.tensor(g["lap_gq2_o1_weights"], device=cuda, dtype=dt)
    a1 = pkg.double_integration_on_panels_3d(0, 1, v, f, a, n, w, w, rands, rands, rel, 1.0, 1)
    a2 = pkg.double_integration_on_panels_3d(0, 1, v, f, a, n, w, w, rands, rands, None, 1.0, 1)
    assert torch.equal(a1, a2)


@pytest.mark.parametrize("layer", [1, 2])
@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("gq", [2, 3])
def test_panels_f32_vs_oracle(pkg, cuda, oracle, layer, order, gq):
    v_np, f_np = pkg.meshes.ellipsoid(2, jitter=0.02, seed=1)
    v = torch.tensor(v_np, dtype=torch.float32, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    a = pkg.utils.compute_face_areas(v, f).contiguous()
    n = pkg.utils.compute_face_normals(v, f).contiguous()
    p, w1 = pkg.utils.get_gaussion_integration_points_and_weights(gq, device=cuda)
    rands, w = pkg.utils.collapsed_rule_2d(p, w1)
    rel = pkg.utils.compute_panel_relation(f)
    out = pkg.double_integration_on_panels_3d(0, order, v, f, a, n, w, w, rands, rands, rel, 1.0, layer)
    h = lambda t: t.cpu().double().numpy()  # noqa: E731
    ref = oracle.laplace_panels(h(v), f_np, h(a), h(n), h(rands), h(w), rel.cpu().numpy(), layer, order)
    assert rel_err(out.cpu().numpy(), ref) < 1e-5


@pytest.mark.parametrize("layer", [1, 2])
def test_panels_helmholtz_f64_vs_oracle(pkg, cuda, oracle, layer):
    v_np, f_np = pkg.meshes.icosphere(1)
    v = torch.tensor(v_np, dtype=torch.float64, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    a = pkg.utils.compute_face_areas(v, f).contiguous()
    n = pkg.utils.compute_face_normals(v, f).contiguous()
    p, w1 = pkg.utils.get_gaussion_integration_points_and_weights(2, device=cuda, dtype=torch.float64)
    rands, w = pkg.utils.collapsed_rule_2d(p, w1)
    rel = pkg.utils.compute_panel_relation(f)
    out = pkg.double_integration_on_panels_3d(int(pkg.BEMType.HELMHOLTZ_BEM), 1, v, f, a, n, w, w, rands,
                                              rands, rel, 3.0, layer)
    h = lambda t: t.cpu().double().numpy()  # noqa: E731
    ref = oracle.laplace_panels(h(v), f_np, h(a), h(n), h(rands), h(w), rel.cpu().numpy(), layer, 1,
                                kind=1, k=3.0)
    assert rel_err(out.cpu().numpy(), ref) < 1e-10


@pytest.mark.parametrize("name,gq,order", [("ico0", 2, 1), ("ico1", 2, 1), ("ico1", 3, 1),
                                           ("ell1", 2, 1), ("ell1", 2, 0)])
def test_solve_f64_matches_reference(pkg, cuda, golden, name, gq, order):
    g = golden[name]
    torch.set_default_dtype(torch.float64)
    try:
        solver = pkg.MeshBEMSolver3d(gaussQR=gq, order_type=order, BEM_type=int(pkg.BEMType.LAPLACE),
                                     wavenumber=1.0, logger=None, dtype=torch.float64, device=cuda)
    finally:
        torch.set_default_dtype(torch.float32)
    v = torch.tensor(g["verts"], dtype=torch.float64, device=cuda)
    f = torch.tensor(g["faces"], dtype=torch.int32, device=cuda)
    fv = (v[:, 0] ** 2 - v[:, 1] ** 2).reshape(1, -1, 1)
    flags = torch.zeros_like(fv, dtype=torch.uint8)
    neu, dirv = solver.solve(v, f, fv, torch.zeros_like(fv), flags)
    tag = f"lap_gq{gq}_o{order}"
    assert rel_err(solver.rhs_layer.get_rhs_vec().cpu().numpy(), g[f"{tag}_rhs"]) < 1e-10
    assert rel_err(neu.cpu().numpy(), g[f"{tag}_neumann"]) < 1e-9
    assert rel_err(dirv.cpu().numpy(), g[f"{tag}_dirichlet"]) == 0.0


@pytest.mark.parametrize("with_rel", [False, True])
@pytest.mark.parametrize("gq", [2, 3])
def test_panels_row_window_equals_full(pkg, cuda, gq, with_rel):
    """Rows [3, 250) through the C ABI equal the same rows of the whole matrix.  With the
    relation matrix the tiled kernel takes its tiles from the window's first row and the
    near-pair kernel overwrites the window's vertex-sharing pairs; without it the per-pair
    kernel derives each relation from the faces."""
    v_np, f_np = pkg.meshes.icosphere(2)
    v = torch.tensor(v_np, dtype=torch.float32, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    a = pkg.utils.compute_face_areas(v, f).contiguous()
    n = pkg.utils.compute_face_normals(v, f).contiguous()
    p, w1 = pkg.utils.get_gaussion_integration_points_and_weights(gq, device=cuda)
    rands, w = pkg.utils.collapsed_rule_2d(p, w1)
    full = pkg.double_integration_on_panels_3d(0, 1, v, f, a, n, w, w, rands, rands, None, 1.0, 2)
    table, seg = pkg.layers._cached_rule_table(rands, rands, w, w, torch.float32, cuda)
    seg_c = np.asarray(seg, dtype=np.int32)
    nf = f.shape[0]
    r0, r1 = 3, 250
    win = torch.full((r1 - r0, nf, 3, 3), float("nan"), dtype=torch.float32, device=cuda)
    rel = pkg.utils.compute_panel_relation(f)
    L = pkg._lib
    L.call("mb_laplace_panels_f32", L.ptr(v), v.shape[0], L.ptr(f), nf, L.ptr(a), L.ptr(n), L.ptr(table),
           seg_c.ctypes.data_as(__import__("ctypes").c_void_p),
           L.ptr(rel) if with_rel else None, 2, 1, 0, 1.0, r0, r1, L.ptr(win),
           None, L.stream_of(v))
    torch.cuda.synchronize()
    assert rel_err(win.cpu().numpy(), full[r0:r1].cpu().numpy()) < 1e-6


@pytest.mark.parametrize("n_fan", [300, 301])
@pytest.mark.parametrize("layer", [1, 2])
def test_panels_high_valence_rows(pkg, cuda, n_fan, layer):
    """A fan of n_fan triangles around one apex: every row has n_fan - 1 pairs sharing a vertex
    (more than the near-pair kernel's list holds, so it rescans the row).  With the relation
    matrix (tiled kernel + near-pair kernel; 300 faces: 32-bit relation scans and bulk row
    stores, 301: byte scans and plain stores) the panels equal the per-pair kernel's, which
    derives each relation from the faces."""
    ang = np.linspace(0.0, 2.0 * np.pi, n_fan, endpoint=False)
    rim = np.stack([np.cos(ang), np.sin(ang), 0.3 * np.sin(3.0 * ang)], axis=1)
    v_np = np.concatenate([[[0.0, 0.0, 0.8]], rim])
    f_np = np.array([[0, 1 + i, 1 + (i + 1) % n_fan] for i in range(n_fan)], dtype=np.int32)
    v = torch.tensor(v_np, dtype=torch.float32, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    a = pkg.utils.compute_face_areas(v, f).contiguous()
    n = pkg.utils.compute_face_normals(v, f).contiguous()
    p, w1 = pkg.utils.get_gaussion_integration_points_and_weights(2, device=cuda)
    rands, w = pkg.utils.collapsed_rule_2d(p, w1)
    rel = pkg.utils.compute_panel_relation(f)
    assert int((rel[0] > 0).sum()) == n_fan
    full = pkg.double_integration_on_panels_3d(0, 1, v, f, a, n, w, w, rands, rands, rel, 1.0, layer)
    table, seg = pkg.layers._cached_rule_table(rands, rands, w, w, torch.float32, cuda)
    seg_c = np.asarray(seg, dtype=np.int32)
    nf = f.shape[0]
    ref = torch.empty((nf, nf, 3, 3), dtype=torch.float32, device=cuda)
    L = pkg._lib
    L.call("mb_laplace_panels_f32", L.ptr(v), v.shape[0], L.ptr(f), nf, L.ptr(a), L.ptr(n), L.ptr(table),
           seg_c.ctypes.data_as(__import__("ctypes").c_void_p), None, layer, 1, 0, 1.0, 0, nf, L.ptr(ref),
           None, L.stream_of(v))
    torch.cuda.synchronize()
    assert torch.isfinite(full).all()
    assert rel_err(full.cpu().numpy(), ref.cpu().numpy()) < 1e-5
