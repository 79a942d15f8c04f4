"""Tensor-core (tcgen05, kind::tf32) path: self-test tile and the split-TF32 x 3 complex
multi-right-hand-side product against FP64 references."""
import ctypes

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
