"""Tensor-core (tcgen05, kind::tf32) path: self-test tile and the split-TF32 x 3 complex
multi-right-hand-side product against FP64 references."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_tcgen05_selftest_tile(pkg, cuda):
    L = pkg.load_library()
    err = ctypes.c_double(-1.0)
    pkg._lib.call("mb_tc_selftest", ctypes.byref(err), pkg._lib.stream_of(torch.empty(1, device=cuda)))
    assert 0.0 <= err.value < 1e-5, err.value


@pytest.mark.parametrize("n,m", [(256, 128), (1000, 200), (2046, 96), (512, 512)])
def test_multi_rhs_matmul_matches_fp64(pkg, cuda, n, m):
    """Split-TF32 x 3 keeps FP32-class accuracy (relative Frobenius error ~1e-7) on sizes that
    exercise partial tiles in every dimension (TMA zero fill, masked stores)."""
    M = pkg.mesh_MOM_3d
    g = torch.Generator(device="cpu").manual_seed(n * 7 + m)
    Z = torch.complex(torch.randn(n, n, generator=g), torch.randn(n, n, generator=g))
    X = torch.complex(torch.randn(n, m, generator=g), torch.randn(n, m, generator=g))
    Zd, Xd = Z.to(cuda), X.to(cuda)
    split = M.split_tf32(Zd)
    Y = M.multi_rhs_matmul(split, Xd, check=True)
    ref = Z.to(torch.complex128) @ X.to(torch.complex128)
    err = (torch.linalg.norm(Y.cpu().to(torch.complex128) - ref) / torch.linalg.norm(ref)).item()
    # plain FP32 (complex64, cuBLAS) product for scale: the split product is as accurate
    plain = (torch.linalg.norm((Zd @ Xd).cpu().to(torch.complex128) - ref) / torch.linalg.norm(ref)).item()
    assert err < max(2e-6, 4 * plain), (err, plain)


def test_multi_rhs_matmul_rejects_odd_n(pkg, cuda):
    M = pkg.mesh_MOM_3d
    Z = torch.zeros(5, 5, dtype=torch.complex64, device=cuda)
    with pytest.raises(pkg.MeshBEMError):
        M.multi_rhs_matmul(M.split_tf32(Z), torch.zeros(5, 3, dtype=torch.complex64, device=cuda))


@pytest.mark.parametrize("m", [64, 7, 1])
def test_gmres_multi_random_system(pkg, cuda, m):
    """Lockstep multi-RHS GMRES on a well-conditioned complex system against dense LU (odd
    column counts run on the internal even width with an inactive padding column)."""
    M = pkg.mesh_MOM_3d
    n = 512
    g = torch.Generator(device="cpu").manual_seed(3)
    Z = (torch.complex(torch.randn(n, n, generator=g), torch.randn(n, n, generator=g)) / n ** 0.5
         + 3 * torch.eye(n, dtype=torch.complex64))
    B = torch.complex(torch.randn(n, m, generator=g, dtype=torch.float64),
                      torch.randn(n, m, generator=g, dtype=torch.float64))
    X, info = M.gmres_multi(M.split_tf32(Z.to(cuda)), B.to(cuda), restart=30, tol=1e-6, max_iters=300)
    assert info["converged"] and info["max_rel_residual"] <= 1e-6
    ref = torch.linalg.solve(Z.to(torch.complex128), B)
    err = torch.linalg.norm(X.cpu() - ref, dim=0) / torch.linalg.norm(ref, dim=0)
    assert err.max().item() < 1e-5
    # FP64 residual of every column, independent of the solver's own estimate
    res = torch.linalg.norm(B - Z.to(torch.complex128) @ X.cpu(), dim=0) / torch.linalg.norm(B, dim=0)
    assert res.max().item() < 3e-6
    steps = info["column_iterations"].cpu()
    assert steps.shape[0] == m and int(steps.max()) <= info["iterations"]


def test_gmres_multi_matches_single_rhs_on_mom_system(pkg, cuda):
    """Many incidences on one mesh: the lockstep solve equals per-column GMRES."""
    M = pkg.mesh_MOM_3d
    v_np, f_np = pkg.meshes.icosphere(2, 1.0)
    v = torch.tensor(v_np, dtype=torch.float32, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    edges, fei, _ = pkg.utils.get_edge_unique(v, f)
    ne = edges.shape[0]
    Z = M.assemble_Z_rwg_sym(v, f, fei, ne, 2.0)
    dirs = pkg.meshes.fibonacci_lattice(8)
    pol = torch.tensor(np.cross(dirs, [0.3, 0.5, 0.8]), dtype=torch.float64)
    pol = pol / pol.norm(dim=1, keepdim=True)
    waves = M.plane_waves(2.0, torch.tensor(dirs), pol, device=cuda)
    B = M.assemble_rhs_rwg_sym(v, f, fei, ne, waves)
    X, info = M.gmres_multi(M.split_tf32(Z), B, restart=50, tol=1e-6, max_iters=2000)
    assert info["converged"]
    for c in range(B.shape[1]):
        x1, inf1 = M.gmres(Z, B[:, c], restart=50, tol=1e-6, max_iters=2000)
        assert inf1[0]["converged"]
        assert (torch.linalg.norm(X[:, c] - x1) / torch.linalg.norm(x1)).item() < 2e-5
