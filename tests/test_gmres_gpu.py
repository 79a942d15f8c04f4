"""GPU checks of the dense iterative solver (replaces torch.linalg.solve of the reference)."""
import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _system(pkg, dev, level=2, k=3.0):
    v_np, f_np = pkg.meshes.icosphere(level)
    v = torch.tensor(v_np, dtype=torch.float32, device=dev)
    f = torch.tensor(f_np, dtype=torch.int32, device=dev)
    edges, fei, _ = pkg.utils.get_edge_unique(v, f)
    solver = pkg.MeshBEMSolver3d(gaussQR=4, order_type=1, BEM_type=int(pkg.BEMType.HELMHOLTZ_MOM),
                                 wavenumber=k, logger=None, dtype=torch.float32, device=dev)
    dirs = pkg.meshes.fibonacci_lattice(3)
    pol = np.cross(dirs, [0.0, 0.3, 1.0])
    pol /= np.linalg.norm(pol, axis=1, keepdims=True)
    waves = pkg.mesh_MOM_3d.plane_waves(k, dirs, pol, device=dev)
    Z, rhs, _ = solver.assemble_MOM(v, f, edges.shape[0], fei, waves=waves)
    return Z, rhs


def test_matvec_and_residual_match_torch(pkg, cuda):
    Z, rhs = _system(pkg, cuda)
    n = Z.shape[0]
    g = torch.Generator(device="cpu").manual_seed(0)
    x = torch.randn(n, dtype=torch.complex128, generator=g).to(cuda)
    y = pkg.mesh_MOM_3d.matvec(Z, x)
    ref = Z.to(torch.complex128) @ x.to(torch.complex64).to(torch.complex128)
    assert rel_err(y.cpu().numpy(), ref.cpu().numpy()) < 1e-6
    b = rhs[:, 0].to(torch.complex128)
    r = pkg.mesh_MOM_3d.residual(Z, x, b)
    ref_r = b - Z.to(torch.complex128) @ x
    assert rel_err(r.cpu().numpy(), ref_r.cpu().numpy()) < 1e-12


def test_matvec_accepts_an_8_byte_aligned_vector_view(pkg, cuda):
    """v = X[1:n+1] of a complex64 array starts 8 bytes past a 16-byte boundary; the product
    must read it element by element and equal the product with an aligned copy."""
    Z, _ = _system(pkg, cuda)
    n = Z.shape[0]
    g = torch.Generator(device="cpu").manual_seed(1)
    X = torch.randn(n + 1, dtype=torch.complex64, generator=g).to(cuda)
    v = X[1:n + 1]
    assert v.data_ptr() % 16 == 8
    y = pkg.mesh_MOM_3d.matvec(Z, v)
    y_aligned = pkg.mesh_MOM_3d.matvec(Z, v.clone())
    ref = Z.to(torch.complex128) @ v.to(torch.complex128)
    assert rel_err(y.cpu().numpy(), ref.cpu().numpy()) < 1e-6
    assert rel_err(y.cpu().numpy(), y_aligned.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("restart", [50, 7])
def test_gmres_matches_dense_solve(pkg, cuda, restart):
    Z, rhs = _system(pkg, cuda)
    x, infos = pkg.mesh_MOM_3d.gmres(Z, rhs, restart=restart, tol=1e-9, max_iters=3000)
    ref = torch.linalg.solve(Z.to(torch.complex128), rhs.to(torch.complex128))
    for c, info in enumerate(infos):
        assert info["converged"], info
        assert info["rel_residual"] <= 1e-9
        assert rel_err(x[:, c].cpu().numpy(), ref[:, c].cpu().numpy()) < 1e-6
    # the FP64 residual reported is the true one
    r = rhs[:, 0].to(torch.complex128) - Z.to(torch.complex128) @ x[:, 0]
    assert float(r.norm() / rhs[:, 0].to(torch.complex128).norm()) <= 2e-9


def test_gmres_iteration_cap_reports_status(pkg, cuda):
    Z, rhs = _system(pkg, cuda)
    x, infos = pkg.mesh_MOM_3d.gmres(Z, rhs[:, 0], restart=5, tol=1e-14, max_iters=3)
    assert infos[0]["iterations"] == 3 and not infos[0]["converged"]
    assert np.isfinite(x.cpu().numpy()).all()


def test_gmres_bad_arguments(pkg, cuda):
    Z, rhs = _system(pkg, cuda, level=1)
    with pytest.raises(pkg.MeshBEMError):
        pkg.mesh_MOM_3d.gmres(Z, rhs, restart=0)
    with pytest.raises(pkg.MeshBEMError):
        pkg.mesh_MOM_3d.gmres(Z, rhs, restart=200)
    with pytest.raises(ValueError):
        pkg.mesh_MOM_3d.gmres(Z, rhs, workspace=torch.empty(16, dtype=torch.uint8, device=cuda))


def test_solve_MOM_gmres_equals_lu(pkg, cuda, golden):
    g = golden["ell1"]
    kw = dict(gaussQR=4, order_type=1, BEM_type=int(pkg.BEMType.HELMHOLTZ_MOM),
              wavenumber=float(g["mom_gq4_k"]), logger=None, dtype=torch.float32, device=cuda)
    v = torch.tensor(g["verts"], dtype=torch.float32, device=cuda)
    f = torch.tensor(g["faces"], dtype=torch.int32, device=cuda)
    edges = torch.tensor(g["edges"], device=cuda)
    fei = torch.tensor(g["face_edge_indices"], dtype=torch.int32, device=cuda)
    js_lu = pkg.MeshBEMSolver3d(**kw).solve_MOM(v, f, edges, fei)
    s = pkg.MeshBEMSolver3d(solver="gmres", gmres_tol=1e-8, **kw)
    js_gm = s.solve_MOM(v, f, edges, fei)
    assert s.last_solve_info[0]["converged"]
    assert rel_err(js_gm.cpu().numpy(), js_lu.cpu().numpy()) < 1e-5
    assert rel_err(js_gm.cpu().numpy(), g["mom_gq4_vert_js"]) < 1e-4
