"""GPU parity of the symmetric-rule EFIE path (7-point rule, closed-form singular parts).

Against the float64 oracle restatement (oracle/mesh_bem_oracle.c, itself checked against
brute-force quadrature and the Mie series in tests/test_symmetric_rule_cpu.py):
1e-10 for float64, 1e-5 for float32 (relative Frobenius).
"""
import numpy as np
import pytest
import torch

import mie
from conftest import rel_err

pytestmark = pytest.mark.gpu


def _mesh(pkg, kind, dev, dt):
    v_np, f_np = pkg.meshes.icosphere(2) if kind == "ico2" else pkg.meshes.ellipsoid(2, jitter=0.03, seed=4)
    v = torch.tensor(v_np, dtype=dt, device=dev)
    f = torch.tensor(f_np, dtype=torch.int32, device=dev)
    edges, fei, _ = pkg.utils.get_edge_unique(v, f)
    return v_np, f_np, v, f, fei, edges.shape[0]


@pytest.mark.parametrize("kind", ["ico2", "ell2"])
@pytest.mark.parametrize("dt,tol", [(torch.float64, 1e-10), (torch.float32, 1e-5)])
def test_sym_zmat_matches_oracle(pkg, cuda, oracle, kind, dt, tol):
    v_np, f_np, v, f, fei, ne = _mesh(pkg, kind, cuda, dt)
    k = 4.0
    Z = pkg.mesh_MOM_3d.assemble_Z_rwg_sym(v, f, fei, ne, k)
    ref = oracle.mom_sym_zmat(v.cpu().double().numpy(), f_np, fei.cpu().numpy(), ne, k)
    assert rel_err(Z.cpu().numpy(), ref) < tol


@pytest.mark.parametrize("dt,tol", [(torch.float64, 1e-10), (torch.float32, 1e-5)])
def test_sym_rhs_matches_oracle(pkg, cuda, oracle, dt, tol):
    v_np, f_np, v, f, fei, ne = _mesh(pkg, "ell2", cuda, dt)
    dirs = pkg.meshes.fibonacci_lattice(4)
    pol = np.cross(dirs, [0.2, 0.1, 1.0])
    pol /= np.linalg.norm(pol, axis=1, keepdims=True)
    waves = pkg.mesh_MOM_3d.plane_waves(4.0, dirs, pol, device=cuda)
    R = pkg.mesh_MOM_3d.assemble_rhs_rwg_sym(v, f, fei, ne, waves)
    ref = oracle.mom_sym_rhs(v.cpu().double().numpy(), f_np, fei.cpu().numpy(), ne, waves.cpu().numpy())
    assert rel_err(R.cpu().numpy(), ref) < tol


def test_sym_near_pairs_cover_every_shared_vertex(pkg, cuda):
    v_np, f_np, v, f, fei, ne = _mesh(pkg, "ico2", cuda, torch.float32)
    pairs = pkg.mesh_MOM_3d.near_pairs(f).cpu().numpy()
    nf = f_np.shape[0]
    assert (pairs[:, 0] == pairs[:, 1]).sum() == nf  # every face with itself
    # icosphere: 3 edge neighbours + 9 vertex neighbours (fewer at the 12 valence-5 vertices)
    per_face = np.bincount(pairs[:, 0], minlength=nf)
    assert per_face.min() >= 11 and per_face.max() <= 13


def test_sym_gmres_current_matches_mie(pkg, cuda):
    """ka = 2 sphere, 1280 faces: the float32 GPU path (assembly + GMRES) within 5 % of Mie."""
    v_np, f_np = pkg.meshes.icosphere(3)
    v = torch.tensor(v_np, dtype=torch.float32, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    edges, fei, _ = pkg.utils.get_edge_unique(v, f)
    k = 2.0
    solver = pkg.MeshBEMSolver3d(gaussQR=4, order_type=1, BEM_type=int(pkg.BEMType.HELMHOLTZ_MOM),
                                 wavenumber=k, logger=None, dtype=torch.float32, device=cuda,
                                 rule="dunavant7", solver="gmres", gmres_tol=1e-7)
    waves = pkg.mesh_MOM_3d.plane_waves(k, [[0.0, 0.0, 1.0]], [[1.0, 0.0, 0.0]], device=cuda)
    Z, rhs, _ = solver.assemble_MOM(v, f, edges.shape[0], fei, waves=waves)
    I, info = pkg.mesh_MOM_3d.gmres(Z, rhs[:, 0], tol=1e-7)
    assert info[0]["converged"]
    I = I.cpu().numpy()
    fe = fei.cpu().numpy()
    P = v_np[f_np]
    c = P.mean(1)
    A = 0.5 * np.linalg.norm(np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 1]), axis=1)
    J = np.zeros((f_np.shape[0], 3), complex)
    for e in range(3):
        i1, i2 = f_np[:, (e + 1) % 3], f_np[:, (e + 2) % 3]
        l = np.linalg.norm(P[:, (e + 2) % 3] - P[:, (e + 1) % 3], axis=1)
        s = np.where(i1 < i2, 1.0, -1.0) * l / (2 * A)
        J += (s * I[fe.reshape(-1, 3)[:, e]])[:, None] * (c - P[:, e])
    assert rel_err(J, mie.surface_current(c, k, 1.0)) < 0.05


@pytest.mark.parametrize("chunks", [1, 5])
def test_sym_zmat_to_host_equals_device(pkg, cuda, chunks):
    """The overlapped host-output assembly returns the same Z as the device path."""
    v_np, f_np = pkg.meshes.icosphere(3)
    v = torch.tensor(v_np, dtype=torch.float32, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    edges, fei, _ = pkg.utils.get_edge_unique(v, f)
    ne = edges.shape[0]
    M = pkg.mesh_MOM_3d
    zd = M.assemble_Z_rwg_sym(v, f, fei, ne, 4.0)
    h = torch.empty((ne, ne), dtype=torch.complex64, pin_memory=True)
    M.assemble_Z_rwg_sym(v, f, fei, ne, 4.0, out_host=h, chunks=chunks)
    torch.cuda.synchronize()
    ref = zd.cpu()
    assert (torch.linalg.norm(h - ref) / torch.linalg.norm(ref)).item() < 1e-6


def test_sym_zmat_to_host_rejects_bad_buffers(pkg, cuda):
    """The host-output assembly refuses pageable host memory and near-pair lists that are not
    sorted by test face (the chunked schedule depends on that order)."""
    v_np, f_np = pkg.meshes.icosphere(1)
    v = torch.tensor(v_np, dtype=torch.float32, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    edges, fei, _ = pkg.utils.get_edge_unique(v, f)
    ne = edges.shape[0]
    M = pkg.mesh_MOM_3d
    with pytest.raises(ValueError):
        M.assemble_Z_rwg_sym(v, f, fei, ne, 2.0, out_host=torch.empty((ne, ne), dtype=torch.complex64))
    pairs = M.near_pairs(f)
    shuffled = pairs.flip(0).contiguous()
    h = torch.empty((ne, ne), dtype=torch.complex64, pin_memory=True)
    with pytest.raises(pkg._lib.MeshBEMError, match="sorted"):
        M.assemble_Z_rwg_sym(v, f, fei, ne, 2.0, pairs=shuffled, out_host=h)
