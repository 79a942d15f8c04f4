"""GPU checks of the near-field preconditioner (mb_spai_build_c64) and the device-resident
preconditioned GMRES (mb_pgmres_c64 / _c128).  Neither has a counterpart in the reference
(it factors Z densely, mesh_BEM_solver_3d.py:174); the checkers are the numpy restatement in
spai_reference.py and dense LU."""
import numpy as np
import pytest
import torch

import spai_reference as SR
from conftest import rel_err

pytestmark = pytest.mark.gpu


def _efie(pkg, dev, level, k):
    M = pkg.mesh_MOM_3d
    v_np, f_np = pkg.meshes.icosphere(level)
    v = torch.tensor(v_np, dtype=torch.float32, device=dev)
    f = torch.tensor(f_np, dtype=torch.int32, device=dev)
    edges, fei, _ = pkg.utils.get_edge_unique(v, f)
    ne = edges.shape[0]
    Z = M.assemble_Z_rwg_sym(v, f, fei, ne, k)
    waves = M.plane_waves(k, [[0.0, 0.0, 1.0]], [[1.0, 0.0, 0.0]], device=dev)
    b = M.assemble_rhs_rwg_sym(v, f, fei, ne, waves)[:, 0].to(torch.complex128)
    torch.cuda.synchronize()
    return v, f, fei, ne, Z, b


def test_spai_patterns_and_columns_match_restatement(pkg, cuda):
    v, f, fei, ne, Z, _ = _efie(pkg, cuda, 2, 3.0)
    P = pkg.mesh_MOM_3d.spai_preconditioner(Z, v, f, fei, ne)
    assert P.status == 0
    cols = P.cols.cpu().numpy()
    vals = P.vals.cpu().numpy()
    pats = SR.patterns(f.cpu().numpy(), fei.cpu().numpy(), ne)
    ref = SR.spai_columns(Z.cpu().numpy(), pats)
    Md = SR.dense_m(ref, ne)
    for i in range(ne):
        J_i = pats[i][0]
        k = int((cols[i] >= 0).sum())
        assert k == J_i.size and np.array_equal(np.sort(cols[i, :k]), J_i), i  # row pattern = J_i (symmetric)
        assert (cols[i, k:] == -1).all()
        got = np.zeros(ne, np.complex128)
        got[cols[i, :k]] = vals[i, :k]
        assert rel_err(got, Md[i]) < 2e-3, i


def test_spai_apply_is_the_row_product(pkg, cuda):
    v, f, fei, ne, Z, _ = _efie(pkg, cuda, 2, 3.0)
    P = pkg.mesh_MOM_3d.spai_preconditioner(Z, v, f, fei, ne)
    g = torch.Generator(device="cpu").manual_seed(0)
    x = torch.randn(ne, dtype=torch.complex64, generator=g).to(cuda)
    y = P.apply(x).cpu().numpy()
    cols, vals = P.cols.cpu().numpy(), P.vals.cpu().numpy()
    Mrow = np.zeros((ne, ne), np.complex128)
    for i in range(ne):
        k = int((cols[i] >= 0).sum())
        Mrow[i, cols[i, :k]] = vals[i, :k]
    assert rel_err(y, Mrow @ x.cpu().numpy().astype(np.complex128)) < 1e-6


def test_pgmres_without_preconditioner_equals_gmres(pkg, cuda):
    _, _, _, ne, Z, b = _efie(pkg, cuda, 2, 3.0)
    M = pkg.mesh_MOM_3d
    x0, i0 = M.gmres(Z, b, restart=30, tol=1e-9, max_iters=3000)
    x1, i1 = M.pgmres(Z, b, restart=30, tol=1e-9, max_iters=3000)
    assert i1[0]["converged"] and i1[0]["rel_residual"] <= 1e-9
    assert rel_err(x1.cpu().numpy(), x0.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("use_graph", [True, False])
def test_pgmres_preconditioned_efie_matches_lu_in_fewer_steps(pkg, cuda, use_graph):
    """7-point EFIE on the 1280-face sphere at ka = 10 (the config-2 wavenumber): the
    preconditioned solve reaches the dense-LU solution with a fraction of the steps."""
    v, f, fei, ne, Z, b = _efie(pkg, cuda, 3, 10.0)
    M = pkg.mesh_MOM_3d
    P = M.spai_preconditioner(Z, v, f, fei, ne)
    ref = torch.linalg.solve(Z.to(torch.complex128), b).cpu().numpy()
    xp, ip = M.pgmres(Z, b, M=P, restart=50, tol=1e-10, max_iters=4000, use_graph=use_graph)
    xn, inn = M.pgmres(Z, b, restart=50, tol=1e-10, max_iters=4000, use_graph=use_graph)
    assert ip[0]["converged"] and inn[0]["converged"]
    assert rel_err(xp.cpu().numpy(), ref) < 1e-6
    assert rel_err(xn.cpu().numpy(), ref) < 1e-6
    assert ip[0]["iterations"] * 5 < inn[0]["iterations"], (ip, inn)
    r = b - Z.to(torch.complex128) @ xp
    assert float(r.norm() / b.norm()) <= 2e-10


def test_pgmres_graph_and_direct_launches_are_bitwise_equal(pkg, cuda):
    v, f, fei, ne, Z, b = _efie(pkg, cuda, 2, 3.0)
    M = pkg.mesh_MOM_3d
    P = M.spai_preconditioner(Z, v, f, fei, ne)
    xa, ia = M.pgmres(Z, b, M=P, restart=20, tol=1e-10, use_graph=True)
    xb, ib = M.pgmres(Z, b, M=P, restart=20, tol=1e-10, use_graph=False)
    assert ia == ib
    assert torch.equal(xa, xb)


def test_pgmres_c128_reaches_fp64_accuracy(pkg, cuda):
    """complex128 Z with FP64 products: the FP64 reference solution of the same system."""
    v, f, fei, ne, Z, b = _efie(pkg, cuda, 2, 5.0)
    M = pkg.mesh_MOM_3d
    Z64 = M.assemble_Z_rwg_sym(v.double(), f, fei, ne, 5.0)
    waves = M.plane_waves(5.0, [[0.0, 0.0, 1.0]], [[1.0, 0.0, 0.0]], device=cuda)
    b64 = M.assemble_rhs_rwg_sym(v.double(), f, fei, ne, waves)[:, 0]
    P = M.spai_preconditioner(Z, v, f, fei, ne)
    x, info = M.pgmres(Z64, b64, M=P, restart=50, tol=1e-13, max_iters=2000)
    ref = torch.linalg.solve(Z64, b64)
    assert info[0]["converged"]
    assert rel_err(x.cpu().numpy(), ref.cpu().numpy()) < 1e-10


def test_pgmres_iteration_cap_and_bad_arguments(pkg, cuda):
    _, _, _, ne, Z, b = _efie(pkg, cuda, 1, 2.0)
    M = pkg.mesh_MOM_3d
    x, info = M.pgmres(Z, b, restart=5, tol=1e-15, max_iters=7)
    assert info[0]["iterations"] == 7 and not info[0]["converged"]
    assert np.isfinite(x.cpu().numpy()).all()
    with pytest.raises(pkg.MeshBEMError):
        M.pgmres(Z, b, restart=0)
    with pytest.raises(pkg.MeshBEMError):
        M.pgmres(Z, b, tol=0.0)


def test_half_copy_scales_and_rounds(pkg, cuda):
    _, _, _, ne, Z, _ = _efie(pkg, cuda, 2, 3.0)
    Zh, scale = pkg.mesh_MOM_3d.half_copy(Z)
    zr = torch.view_as_real(Z)
    amax = float(zr.abs().max())
    assert float(scale) == amax
    back = Zh.float().reshape(ne, ne, 2) * float(scale)
    err = (back - zr).abs().max().item()
    assert err <= amax * 2.0 ** -11  # half a unit in the last place of binary16 at the scale


@pytest.mark.parametrize("use_graph", [True, False])
def test_pgmres_half_inner_reaches_lu(pkg, cuda, use_graph):
    """Arnoldi products on the half-precision copy, refinement against complex64 Z: the
    solution still reaches the dense-LU solution of the complex64 system."""
    v, f, fei, ne, Z, b = _efie(pkg, cuda, 3, 10.0)
    M = pkg.mesh_MOM_3d
    P = M.spai_preconditioner(Z, v, f, fei, ne)
    ref = torch.linalg.solve(Z.to(torch.complex128), b).cpu().numpy()
    x, info = M.pgmres(Z, b, M=P, restart=50, tol=1e-9, max_iters=4000, use_graph=use_graph,
                       Z_half=M.half_copy(Z), inner_rtol=3e-3)
    assert info[0]["converged"] and info[0]["restarts"] >= 2
    assert rel_err(x.cpu().numpy(), ref) < 1e-6
    r = b - Z.to(torch.complex128) @ x
    assert float(r.norm() / b.norm()) <= 2e-9


def test_pgmres_half_graph_and_direct_bitwise_equal(pkg, cuda):
    v, f, fei, ne, Z, b = _efie(pkg, cuda, 2, 3.0)
    M = pkg.mesh_MOM_3d
    P = M.spai_preconditioner(Z, v, f, fei, ne)
    H = M.half_copy(Z)
    xa, ia = M.pgmres(Z, b, M=P, restart=20, tol=1e-10, use_graph=True, Z_half=H)
    xb, ib = M.pgmres(Z, b, M=P, restart=20, tol=1e-10, use_graph=False, Z_half=H)
    assert ia == ib
    assert torch.equal(xa, xb)
