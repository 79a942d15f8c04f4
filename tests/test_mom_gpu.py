"""GPU parity of the RWG MoM operators against the reference's own results and the oracle.

Tolerances (relative Frobenius): 1e-10 for float64 paths, 1e-5 for float32 paths against
the float64 oracle (the reference's FP32 build is itself ~1e-6 away from its FP64 result).
"""
import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL32 = 1e-5


def _dev_mesh(g, dev, dt):
    v = torch.tensor(g["verts"], dtype=dt, device=dev)
    f = torch.tensor(g["faces"], dtype=torch.int32, device=dev)
    a = torch.tensor(g["face_areas"], dtype=dt, device=dev)
    n = torch.tensor(g["face_normals"], dtype=dt, device=dev)
    return v, f, a, n


def _rules(pkg, gq, dev, dt):
    U = pkg.utils
    torch.set_default_dtype(torch.float64)  # the golden run used float64 literal tables
    try:
        px, wx = U.get_gaussion_integration_points_and_weights(gq, device=dev, dtype=dt)
        py, wy = U.get_gaussion_integration_points_and_weights(gq - 1, device=dev, dtype=dt)
    finally:
        torch.set_default_dtype(torch.float32)
    return px, wx, py, wy


@pytest.mark.parametrize("name", ["ico0", "ico1", "ell1"])
@pytest.mark.parametrize("gq", [4, 3])
def test_zmat_fe_f64_matches_reference(pkg, cuda, golden, name, gq):
    g = golden[name]
    v, f, a, n = _dev_mesh(g, cuda, torch.float64)
    px, wx, py, wy = _rules(pkg, gq, cuda, torch.float64)
    nf = f.shape[0]
    zr = torch.zeros((1, 3 * nf, 3 * nf), dtype=torch.float64, device=cuda)
    zi = torch.zeros_like(zr)
    k = float(g[f"mom_gq{gq}_k"])
    pkg.mesh_MOM_3d.create_MOM_Zmat_3d_forward(v, f, a, n, px, wx, py, wy, zr, zi, k)
    z = (zr + 1j * zi)[0].cpu().numpy()
    if f"mom_gq{gq}_zfe" in g:
        assert rel_err(z, g[f"mom_gq{gq}_zfe"]) < TOL64
    else:
        ref_rows = g[f"mom_gq{gq}_zfe_rows"]
        assert rel_err(z[: ref_rows.shape[0]], ref_rows) < TOL64
    assert abs(np.linalg.norm(z) / float(g[f"mom_gq{gq}_zfe_fro"]) - 1) < TOL64


def test_zmat_fe_batch_copies(pkg, cuda, golden):
    g = golden["ico0"]
    v, f, a, n = _dev_mesh(g, cuda, torch.float64)
    px, wx, py, wy = _rules(pkg, 4, cuda, torch.float64)
    nf = f.shape[0]
    zr = torch.zeros((2, 3 * nf, 3 * nf), dtype=torch.float64, device=cuda)
    zi = torch.zeros_like(zr)
    pkg.mesh_MOM_3d.create_MOM_Zmat_3d_forward(v, f, a, n, px, wx, py, wy, zr, zi, 2.0)
    assert torch.equal(zr[0], zr[1]) and torch.equal(zi[0], zi[1])
    assert rel_err((zr[1] + 1j * zi[1]).cpu().numpy(), g["mom_gq4_zfe"]) < TOL64


@pytest.mark.parametrize("level,k", [(1, 2.0), (2, 6.0)])
def test_zmat_fe_f32_vs_oracle(pkg, cuda, oracle, level, k):
    v_np, f_np = pkg.meshes.icosphere(level)
    v = torch.tensor(v_np, dtype=torch.float32, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    a = pkg.utils.compute_face_areas(v, f).contiguous()
    n = pkg.utils.compute_face_normals(v, f).contiguous()
    px, wx = pkg.utils.get_gaussion_integration_points_and_weights(4, device=cuda)
    py, wy = pkg.utils.get_gaussion_integration_points_and_weights(3, device=cuda)
    nf = f.shape[0]
    zr = torch.zeros((1, 3 * nf, 3 * nf), dtype=torch.float32, device=cuda)
    zi = torch.zeros_like(zr)
    pkg.mesh_MOM_3d.create_MOM_Zmat_3d_forward(v, f, a, n, px, wx, py, wy, zr, zi, k)
    z = (zr[0].double() + 1j * zi[0].double()).cpu().numpy()
    h = lambda t: t.cpu().double().numpy()  # noqa: E731
    ref = oracle.mom_zmat_fe(h(v), f_np, h(a), h(n), h(px), h(wx), h(py), h(wy), k)
    assert rel_err(z, ref) < TOL32


def test_zmat_fe_f32_high_k_row_slice_vs_oracle(pkg, cuda, oracle):
    """ka = 10 on the 1280-face sphere: phases kR up to ~20 rad through the SFU sin/cos."""
    v_np, f_np = pkg.meshes.icosphere(3)
    k = 10.0
    v = torch.tensor(v_np, dtype=torch.float32, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    a = pkg.utils.compute_face_areas(v, f).contiguous()
    n = pkg.utils.compute_face_normals(v, f).contiguous()
    px, wx = pkg.utils.get_gaussion_integration_points_and_weights(4, device=cuda)
    py, wy = pkg.utils.get_gaussion_integration_points_and_weights(3, device=cuda)
    nf = f.shape[0]
    zr = torch.zeros((1, 3 * nf, 3 * nf), dtype=torch.float32, device=cuda)
    zi = torch.zeros_like(zr)
    pkg.mesh_MOM_3d.create_MOM_Zmat_3d_forward(v, f, a, n, px, wx, py, wy, zr, zi, k)
    rows = (1200, 1500)
    z = (zr[0, rows[0]:rows[1]].double() + 1j * zi[0, rows[0]:rows[1]].double()).cpu().numpy()
    h = lambda t: t.cpu().double().numpy()  # noqa: E731
    ref = oracle.mom_zmat_fe(h(v), f_np, h(a), h(n), h(px), h(wx), h(py), h(wy), k, rows=rows)
    assert rel_err(z, ref) < TOL32


@pytest.mark.parametrize("dt,tol", [(torch.float32, TOL32), (torch.float64, TOL64)])
def test_zmat_rwg_equals_scattered_face_edge(pkg, cuda, golden, oracle, dt, tol):
    g = golden["ell1"]
    v, f, a, n = _dev_mesh(g, cuda, dt)
    px, wx, py, wy = _rules(pkg, 4, cuda, dt)
    fei = torch.tensor(g["face_edge_indices"], dtype=torch.int32, device=cuda)
    ne = g["edges"].shape[0]
    Z = pkg.mesh_MOM_3d.assemble_Z_rwg(v, f, a, n, fei, ne, px, wx, py, wy, 2.0)
    h = lambda t: t.cpu().double().numpy()  # noqa: E731
    zfe = oracle.mom_zmat_fe(h(v), g["faces"], h(a), h(n), h(px), h(wx), h(py), h(wy), 2.0)
    e = g["face_edge_indices"].astype(np.int64)
    zref = np.zeros((ne, ne), np.complex128)
    np.add.at(zref, (e[:, None], e[None, :]), zfe)
    assert rel_err(Z.cpu().numpy(), zref) < tol


def test_zmat_rwg_row_chunks_sum_to_full(pkg, cuda):
    v_np, f_np = pkg.meshes.icosphere(2)
    v = torch.tensor(v_np, dtype=torch.float32, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    edges, fei, _ = pkg.utils.get_edge_unique(v, f)
    a = pkg.utils.compute_face_areas(v, f).contiguous()
    n = pkg.utils.compute_face_normals(v, f).contiguous()
    px, wx = pkg.utils.get_gaussion_integration_points_and_weights(4, device=cuda)
    py, wy = pkg.utils.get_gaussion_integration_points_and_weights(3, device=cuda)
    ne = edges.shape[0]
    full = pkg.mesh_MOM_3d.assemble_Z_rwg(v, f, a, n, fei, ne, px, wx, py, wy, 3.0)
    part = torch.zeros_like(full)
    nrow = 3 * f.shape[0]
    for r0 in range(0, nrow, 257):
        pkg.mesh_MOM_3d.assemble_Z_rwg(v, f, a, n, fei, ne, px, wx, py, wy, 3.0, out=part,
                                       rows=(r0, min(nrow, r0 + 257)))
    assert rel_err(part.cpu().numpy(), full.cpu().numpy()) < 1e-6


def _ico_setup(pkg, cuda, level):
    v_np, f_np = pkg.meshes.icosphere(level)
    v = torch.tensor(v_np, dtype=torch.float32, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    edges, fei, _ = pkg.utils.get_edge_unique(v, f)
    a = pkg.utils.compute_face_areas(v, f).contiguous()
    n = pkg.utils.compute_face_normals(v, f).contiguous()
    px, wx = pkg.utils.get_gaussion_integration_points_and_weights(4, device=cuda)
    py, wy = pkg.utils.get_gaussion_integration_points_and_weights(3, device=cuda)
    return v, f, a, n, fei, edges.shape[0], (px, wx, py, wy)


def test_edge_rows_map(pkg, cuda):
    v, f, a, n, fei, ne, _ = _ico_setup(pkg, cuda, 2)
    er = pkg.mesh_MOM_3d.edge_rows(fei, f.shape[0], ne).cpu().numpy()
    e = fei.cpu().numpy().reshape(-1).astype(np.int64)
    ref = np.full((ne, 2), -1, np.int64)
    for r in np.argsort(e, kind="stable"):  # rows of each edge in increasing order
        m = e[r]
        ref[m, 0 if ref[m, 0] < 0 else 1] = r
    assert er[-1] == 0
    assert np.array_equal(er[:-1].reshape(ne, 2), ref)


def test_edge_rows_reject_more_than_two_faces(pkg, cuda):
    # three triangles on one edge (0, 1)
    v = torch.tensor([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1]], dtype=torch.float32, device=cuda)
    f = torch.tensor([[0, 1, 2], [1, 0, 3], [0, 1, 4]], dtype=torch.int32, device=cuda)
    edges, fei, _ = pkg.utils.get_edge_unique(v, f)
    with pytest.raises(ValueError):
        pkg.mesh_MOM_3d.edge_rows(fei, 3, edges.shape[0])


@pytest.mark.parametrize("level,k", [(2, 3.0), (3, 8.0)])
def test_zmat_rwg_edge_order_equals_face_order(pkg, cuda, level, k):
    v, f, a, n, fei, ne, rules = _ico_setup(pkg, cuda, level)
    M = pkg.mesh_MOM_3d
    zf = M.assemble_Z_rwg(v, f, a, n, fei, ne, *rules, k)
    ze = M.assemble_Z_rwg(v, f, a, n, fei, ne, *rules, k, order="edges")
    assert rel_err(ze.cpu().numpy(), zf.cpu().numpy()) < 1e-6
    part = torch.zeros_like(ze)
    for m0 in range(0, ne, 101):  # Z-row chunks sum to the whole
        M.assemble_Z_rwg(v, f, a, n, fei, ne, *rules, k, out=part, order="edges", rows=(m0, min(ne, m0 + 101)))
    assert torch.equal(part, ze)


@pytest.mark.parametrize("chunks", [1, 7])
def test_zmat_rwg_to_host_equals_device(pkg, cuda, chunks):
    v, f, a, n, fei, ne, rules = _ico_setup(pkg, cuda, 3)
    M = pkg.mesh_MOM_3d
    zd = M.assemble_Z_rwg(v, f, a, n, fei, ne, *rules, 5.0, order="edges")  # the host path's kernel
    h = torch.empty((ne, ne), dtype=torch.complex64, pin_memory=True)
    scratch = torch.full((ne, ne), float("nan"), dtype=torch.complex64, device=cuda)  # overwritten
    M.assemble_Z_rwg(v, f, a, n, fei, ne, *rules, 5.0, out=scratch, out_host=h, chunks=chunks)
    torch.cuda.synchronize()
    assert torch.equal(h, zd.cpu())


@pytest.mark.parametrize("name", ["ico0", "ell1"])
def test_rhs_fe_matches_reference(pkg, cuda, golden, name):
    g = golden[name]
    v, f, a, n = _dev_mesh(g, cuda, torch.float64)
    px, wx, _, _ = _rules(pkg, 4, cuda, torch.float64)
    nf = f.shape[0]
    rr = torch.zeros((1, nf, 3, 1), dtype=torch.float64, device=cuda)
    ri = torch.zeros_like(rr)
    pkg.mesh_MOM_3d.create_MOM_rhs_3d_forward(v, f, a, n, px, wx, rr, ri, 2.0)
    r = (rr + 1j * ri)[0, :, :, 0].cpu().numpy()
    assert rel_err(r, g["mom_gq4_rhsfe"]) < TOL64


def test_rhs_rwg_multi_wave(pkg, cuda, golden, oracle):
    g = golden["ell1"]
    v, f, a, n = _dev_mesh(g, cuda, torch.float32)
    px, wx, _, _ = _rules(pkg, 4, cuda, torch.float32)
    fei = torch.tensor(g["face_edge_indices"], dtype=torch.int32, device=cuda)
    ne = g["edges"].shape[0]
    dirs = pkg.meshes.fibonacci_lattice(6)
    pol = np.cross(dirs, [0.3, 0.5, 0.81])
    pol /= np.linalg.norm(pol, axis=1, keepdims=True)
    waves = pkg.mesh_MOM_3d.plane_waves(2.0, dirs, pol, device=cuda)
    R = pkg.mesh_MOM_3d.assemble_rhs_rwg(v, f, a, n, fei, ne, px, wx, waves).cpu().numpy()
    h = lambda t: t.cpu().double().numpy()  # noqa: E731
    e = g["face_edge_indices"].astype(np.int64)
    for i in range(6):
        fe = oracle.mom_rhs_fe(h(v), g["faces"], h(a), h(n), h(px), h(wx), 2.0, khat=dirs[i],
                               e0=pol[i]).reshape(-1)
        ref = np.zeros(ne, np.complex128)
        np.add.at(ref, e, fe)
        assert rel_err(R[:, i], ref) < TOL32
    # the packed reference wave reproduces the face-edge op after scattering
    w0 = pkg.mesh_MOM_3d.reference_plane_wave(2.0, device=cuda)
    R0 = pkg.mesh_MOM_3d.assemble_rhs_rwg(v, f, a, n, fei, ne, px, wx, w0).cpu().numpy()[:, 0]
    ref0 = np.zeros(ne, np.complex128)
    np.add.at(ref0, e, g["mom_gq4_rhsfe"].reshape(-1))
    assert rel_err(R0, ref0) < TOL32


@pytest.mark.parametrize("name", ["ico0", "ell1"])
def test_interp_matches_reference(pkg, cuda, golden, name):
    g = golden[name]
    v, f, a, _ = _dev_mesh(g, cuda, torch.float64)
    fei = torch.tensor(g["face_edge_indices"], dtype=torch.int32, device=cuda)
    ic = torch.tensor(g["mom_gq4_icoeff"], device=cuda)
    nf = f.shape[0]
    jr = torch.zeros((1, 3 * nf, 3), dtype=torch.float64, device=cuda)
    ji = torch.zeros_like(jr)
    pkg.mesh_MOM_3d.interpolate_Icoeff_to_Js_3d_forward(v, f, fei, a, ic.real.contiguous(),
                                                        ic.imag.contiguous(), jr, ji)
    assert rel_err((jr + 1j * ji).cpu().numpy(), g["mom_gq4_face_vert_js"]) < TOL64
    vj = pkg.mesh_MOM_3d.interpolate_vert_js(v, f, fei, a, ic)
    assert rel_err(vj.cpu().numpy(), g["mom_gq4_vert_js"]) < TOL64


@pytest.mark.parametrize("name", ["ico0", "ico1", "ell1"])
def test_solve_MOM_f64_matches_reference(pkg, cuda, golden, name):
    g = golden[name]
    torch.set_default_dtype(torch.float64)
    try:
        solver = pkg.MeshBEMSolver3d(gaussQR=4, order_type=1, BEM_type=int(pkg.BEMType.HELMHOLTZ_MOM),
                                     wavenumber=float(g["mom_gq4_k"]), logger=None,
                                     dtype=torch.float64, device=cuda)
    finally:
        torch.set_default_dtype(torch.float32)
    v = torch.tensor(g["verts"], dtype=torch.float64, device=cuda)
    f = torch.tensor(g["faces"], dtype=torch.int32, device=cuda)
    edges = torch.tensor(g["edges"], device=cuda)
    fei = torch.tensor(g["face_edge_indices"], dtype=torch.int32, device=cuda)
    js = solver.solve_MOM(v, f, edges, fei)
    assert js.shape == (1, v.shape[0], 3)
    assert rel_err(js.cpu().numpy(), g["mom_gq4_vert_js"]) < 1e-9


def test_solve_MOM_f32_close_to_reference(pkg, cuda, golden):
    g = golden["ell1"]
    torch.set_default_dtype(torch.float64)
    try:
        solver = pkg.MeshBEMSolver3d(gaussQR=4, order_type=1, BEM_type=int(pkg.BEMType.HELMHOLTZ_MOM),
                                     wavenumber=float(g["mom_gq4_k"]), logger=None,
                                     dtype=torch.float32, device=cuda)
    finally:
        torch.set_default_dtype(torch.float32)
    v = torch.tensor(g["verts"], dtype=torch.float32, device=cuda)
    f = torch.tensor(g["faces"], dtype=torch.int32, device=cuda)
    edges = torch.tensor(g["edges"], device=cuda)
    fei = torch.tensor(g["face_edge_indices"], dtype=torch.int32, device=cuda)
    js = solver.solve_MOM(v, f, edges, fei)
    # FP32 assembly + complex64 LU: the current inherits cond(Z) * 1e-7-level input error.
    assert rel_err(js.cpu().numpy(), g["mom_gq4_vert_js"]) < 1e-4


def test_bad_inputs_raise(pkg, cuda):
    v = torch.zeros((3, 3), device=cuda)
    f = torch.zeros((1, 3), dtype=torch.int64, device=cuda)
    a = torch.ones((1, 1), device=cuda)
    n = torch.zeros((1, 3), device=cuda)
    p, w = pkg.utils.get_gaussion_integration_points_and_weights(2, device=cuda)
    zr = torch.zeros((1, 3, 3), device=cuda)
    with pytest.raises(TypeError):
        pkg.mesh_MOM_3d.create_MOM_Zmat_3d_forward(v, f, a, n, p, w, p, w, zr, zr.clone(), 1.0)
    with pytest.raises(ValueError):
        pkg.mesh_MOM_3d.create_MOM_Zmat_3d_forward(v.cpu(), f.int().cpu(), a, n, p, w, p, w, zr,
                                                   zr.clone(), 1.0)
    with pytest.raises(pkg.MeshBEMError):
        pkg.mesh_MOM_3d.create_MOM_Zmat_3d_forward(v, f.int(), a, n, p, w, p, w, zr, zr.clone(), 0.0)


def test_empty_mesh_is_noop(pkg, cuda):
    v = torch.zeros((0, 3), device=cuda)
    f = torch.zeros((0, 3), dtype=torch.int32, device=cuda)
    a = torch.zeros((0, 1), device=cuda)
    n = torch.zeros((0, 3), device=cuda)
    p, w = pkg.utils.get_gaussion_integration_points_and_weights(2, device=cuda)
    zr = torch.zeros((1, 0, 0), device=cuda)
    pkg.mesh_MOM_3d.create_MOM_Zmat_3d_forward(v, f, a, n, p, w, p, w, zr, zr.clone(), 1.0)


@pytest.mark.parametrize("name", ["ico0", "ico1", "ell1"])
def test_radiate_H_f64_matches_reference(pkg, cuda, golden, name):
    g = golden[name]
    v = torch.tensor(g["verts"], device=cuda)
    H = pkg.mesh_MOM_3d.radiate_H(torch.tensor(g["field_points"], device=cuda), v,
                                  torch.tensor(g["vert_areas"], device=cuda),
                                  torch.tensor(g["mom_gq4_vert_js"][0], device=cuda), float(g["mom_gq4_k"]))
    assert rel_err(H.cpu().numpy(), g["field_H"]) < TOL64


def test_radiate_H_f32_large_vs_oracle(pkg, cuda, oracle):
    """A 64 x 64 observation grid around the 2562-vertex sphere, float32 against float64."""
    v_np, f_np = pkg.meshes.icosphere(4)
    rng = np.random.default_rng(0)
    js = rng.normal(size=(v_np.shape[0], 3)) + 1j * rng.normal(size=(v_np.shape[0], 3))
    va = rng.uniform(0.5, 1.5, size=v_np.shape[0]) * 1e-3
    g1 = np.linspace(-3, 3, 64)
    gx, gz = np.meshgrid(g1, g1, indexing="ij")
    pts = np.stack([gx.ravel(), 0.05 * np.ones(gx.size), gz.ravel()], -1)
    H = pkg.mesh_MOM_3d.radiate_H(torch.tensor(pts, dtype=torch.float32, device=cuda),
                                  torch.tensor(v_np, dtype=torch.float32, device=cuda),
                                  torch.tensor(va, dtype=torch.float32, device=cuda),
                                  torch.tensor(js, dtype=torch.complex64, device=cuda), 10.0)
    f32 = lambda a: a.astype(np.float32).astype(np.float64)  # noqa: E731
    ref = oracle.radiate_h(f32(pts), f32(v_np), f32(va), f32(js.real) + 1j * f32(js.imag), 10.0)
    assert rel_err(H.cpu().numpy(), ref) < TOL32


# ---- the benched kernel at the benched phases ---------------------------------------------
# The bench assembles Z by Z rows (order="edges", float32, gaussQR 4) at ka = 10, so phases
# kR up to ~20 rad go through the SFU sine / cosine.  These compare that exact code path with
# the float64 oracle: the whole matrix on the 1280-face sphere and Z-row windows of the
# 20480-face sphere of the bench itself.

def _scatter_rows(zfe_rows, row_ids, e, ne):
    """Z rows of the face-edge rows `row_ids` (rows of zfe_rows), columns scattered by e."""
    out = np.zeros((len(row_ids), ne), np.complex128)
    for i, r in enumerate(row_ids):
        np.add.at(out[i], e, zfe_rows[r])
    return out


@pytest.mark.parametrize("order", ["edges", "gather"])
def test_zmat_rwg_edges_ka10_full_L3_vs_oracle(pkg, cuda, oracle, order):
    v, f, a, n, fei, ne, rules = _ico_setup(pkg, cuda, 3)
    k = 10.0
    Z = pkg.mesh_MOM_3d.assemble_Z_rwg(v, f, a, n, fei, ne, *rules, k, order=order)
    h = lambda t: t.cpu().double().numpy()  # noqa: E731
    zfe = oracle.mom_zmat_fe(h(v), f.cpu().numpy(), h(a), h(n), *(h(t) for t in rules), k)
    e = fei.cpu().numpy().reshape(-1).astype(np.int64)
    zrow = np.zeros((ne, zfe.shape[1]), np.complex128)
    np.add.at(zrow, e, zfe)
    zref = np.zeros((ne, ne), np.complex128)
    np.add.at(zref.T, e, zrow.T)
    assert rel_err(Z.cpu().numpy(), zref) < TOL32


def test_zmat_rwg_edges_ka10_L5_row_windows_vs_oracle(pkg, cuda, oracle):
    """The bench workload itself (icosphere L5, F = 20480, E = 30720, ka = 10): the whole Z,
    then the Z rows of three windows of 16 faces (the children of one level-3 face, 18 interior
    edges each) against the oracle's face-edge rows."""
    v, f, a, n, fei, ne, rules = _ico_setup(pkg, cuda, 5)
    k = 10.0
    er = pkg.mesh_MOM_3d.edge_rows(fei, f.shape[0], ne)
    Z = torch.full((ne, ne), float("nan"), dtype=torch.complex64, device=cuda)  # gather overwrites every entry
    pkg.mesh_MOM_3d.assemble_Z_rwg(v, f, a, n, fei, ne, *rules, k, out=Z, order="gather", edge_rows_map=er)
    torch.cuda.synchronize()
    er2 = er[:-1].cpu().numpy().reshape(ne, 2).astype(np.int64)
    e = fei.cpu().numpy().reshape(-1).astype(np.int64)
    h = lambda t: t.cpu().double().numpy()  # noqa: E731
    vh, fh, ah, nh = h(v), f.cpu().numpy(), h(a), h(n)
    rh = [h(t) for t in rules]
    nf = f.shape[0]
    compared = 0
    for f0 in (0, nf // 2 + 96, nf - 16):
        r0, r1 = 3 * f0, 3 * (f0 + 16)
        # Z rows whose two face-edge rows both lie in the window
        m = np.nonzero((er2[:, 0] >= r0) & (er2[:, 1] >= r0) & (er2[:, 0] < r1) & (er2[:, 1] < r1))[0]
        assert m.size >= 16
        zfe = oracle.mom_zmat_fe(vh, fh, ah, nh, *rh, k, rows=(r0, r1))
        ref = _scatter_rows(zfe, er2[m, 0] - r0, e, ne) + _scatter_rows(zfe, er2[m, 1] - r0, e, ne)
        got = Z[torch.as_tensor(m, device=cuda)].cpu().numpy()
        assert rel_err(got, ref) < TOL32, f0
        compared += m.size
    assert compared >= 48


# ---- the reference's own call sites ---------------------------------------------------------

def _check_zfe(z, g, gq):
    if f"mom_gq{gq}_zfe" in g:
        assert rel_err(z, g[f"mom_gq{gq}_zfe"]) < TOL64
    else:
        ref_rows = g[f"mom_gq{gq}_zfe_rows"]
        assert rel_err(z[: ref_rows.shape[0]], ref_rows) < TOL64
    assert abs(np.linalg.norm(z) / float(g[f"mom_gq{gq}_zfe_fro"]) - 1) < TOL64


@pytest.mark.parametrize("name", ["ico0", "ell1"])
def test_kernel_functions_apply_match_reference(pkg, cuda, golden, name):
    """MeshMOM{Zmat,Rhs,InterpolateJs}Kernel.apply -- the only way the reference reaches its
    kernels (src/mesh_BEM/kernel_functions.py:26-171) -- against the reference's results."""
    g = golden[name]
    v, f, a, n = _dev_mesh(g, cuda, torch.float64)
    px, wx, py, wy = _rules(pkg, 4, cuda, torch.float64)
    KF = pkg.kernel_functions
    k = float(g["mom_gq4_k"])
    nf = f.shape[0]
    Z = KF.MeshMOMZmatKernel.apply(v, f, a, n, px, wx, py, wy, k)
    assert Z.shape == (1, 3 * nf, 3 * nf) and Z.dtype == torch.complex128
    _check_zfe(Z[0].cpu().numpy(), g, 4)
    R = KF.MeshMOMRhsKernel.apply(v, f, a, n, px, wx, k)
    assert R.shape == (1, nf, 3, 1) and R.dtype == torch.complex128
    assert rel_err(R[0, :, :, 0].cpu().numpy(), g["mom_gq4_rhsfe"]) < TOL64
    fei = torch.tensor(g["face_edge_indices"], dtype=torch.int32, device=cuda)
    ic = torch.tensor(g["mom_gq4_icoeff"], device=cuda)
    J = KF.MeshMOMInterpolateJsKernel.apply(v, f, fei, a, ic)
    assert J.shape == (1, 3 * nf, 3) and J.dtype == torch.complex128
    assert rel_err(J.cpu().numpy(), g["mom_gq4_face_vert_js"]) < TOL64


def test_kernel_functions_float32_close_to_reference(pkg, cuda, golden):
    """The demo's dtype (float32): the same wrappers within the FP32 tolerance."""
    g = golden["ell1"]
    v, f, a, n = _dev_mesh(g, cuda, torch.float32)
    px, wx, py, wy = _rules(pkg, 4, cuda, torch.float32)
    KF = pkg.kernel_functions
    k = float(g["mom_gq4_k"])
    Z = KF.MeshMOMZmatKernel.apply(v, f, a, n, px, wx, py, wy, k)
    assert Z.dtype == torch.complex64
    ref_rows = g["mom_gq4_zfe_rows"]
    assert rel_err(Z[0, : ref_rows.shape[0]].cpu().numpy(), ref_rows) < TOL32
    R = KF.MeshMOMRhsKernel.apply(v, f, a, n, px, wx, k)
    assert rel_err(R[0, :, :, 0].cpu().numpy(), g["mom_gq4_rhsfe"]) < TOL32


def test_torch_ops_mesh_MOM_3d_match_reference(pkg, cuda, golden):
    """torch.ops.mesh_MOM_3d.* (TORCH_LIBRARY(mesh_MOM_3d), mesh_MOM_3d.cpp:117-121) after
    register_torch_ops(): the three ops write their outputs in place like the reference's."""
    lib = pkg.mesh_MOM_3d.register_torch_ops()
    assert pkg.mesh_MOM_3d.register_torch_ops() is lib  # registering twice is a no-op
    ops = torch.ops.mesh_MOM_3d
    g = golden["ico0"]
    v, f, a, n = _dev_mesh(g, cuda, torch.float64)
    px, wx, py, wy = _rules(pkg, 4, cuda, torch.float64)
    k = float(g["mom_gq4_k"])
    nf = f.shape[0]
    zr = torch.zeros((1, 3 * nf, 3 * nf), dtype=torch.float64, device=cuda)
    zi = torch.zeros_like(zr)
    ops.create_MOM_Zmat_3d_forward(v, f, a, n, px, wx, py, wy, zr, zi, k)
    _check_zfe((zr + 1j * zi)[0].cpu().numpy(), g, 4)
    rr = torch.zeros((1, nf, 3, 1), dtype=torch.float64, device=cuda)
    ri = torch.zeros_like(rr)
    ops.create_MOM_rhs_3d_forward(v, f, a, n, px, wx, rr, ri, k)
    assert rel_err((rr + 1j * ri)[0, :, :, 0].cpu().numpy(), g["mom_gq4_rhsfe"]) < TOL64
    fei = torch.tensor(g["face_edge_indices"], dtype=torch.int32, device=cuda)
    ic = torch.tensor(g["mom_gq4_icoeff"], device=cuda)
    jr = torch.zeros((1, 3 * nf, 3), dtype=torch.float64, device=cuda)
    ji = torch.zeros_like(jr)
    ops.interpolate_Icoeff_to_Js_3d_forward(v, f, fei, a, ic.real.contiguous(), ic.imag.contiguous(), jr, ji)
    assert rel_err((jr + 1j * ji).cpu().numpy(), g["mom_gq4_face_vert_js"]) < TOL64


@pytest.mark.parametrize("level,k", [(2, 3.0), (3, 8.0)])
def test_zmat_rwg_gather_equals_edge_order(pkg, cuda, level, k):
    """Gather form: same entries as the atomic edge order; row windows overwrite exactly their rows."""
    v, f, a, n, fei, ne, rules = _ico_setup(pkg, cuda, level)
    M = pkg.mesh_MOM_3d
    ze = M.assemble_Z_rwg(v, f, a, n, fei, ne, *rules, k, order="edges")
    zg = torch.full_like(ze, float("nan"))
    M.assemble_Z_rwg(v, f, a, n, fei, ne, *rules, k, out=zg, order="gather")
    assert rel_err(zg.cpu().numpy(), ze.cpu().numpy()) < 1e-6
    part = torch.full_like(ze, float("nan"))
    for m0 in range(0, ne, 97):
        M.assemble_Z_rwg(v, f, a, n, fei, ne, *rules, k, out=part, order="gather", rows=(m0, min(ne, m0 + 97)))
    assert torch.equal(part, zg)
