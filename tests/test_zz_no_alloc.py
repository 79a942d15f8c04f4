"""The allocation-free GMRES entry point, ``mb_gmres_c64_noalloc``, called through the C ABI.

Some callers of this library cannot allocate device memory: a host program or plugin that
budgets all GPU memory once at start-up, or a foreign-language caller (Go, Java, ...) that
reaches the library only through its C ABI and has no CUDA allocator of its own.  For them
the library offers a GMRES that takes no workspace and uses a fixed scratch array inside
the library instead.  This file checks it against the regular entry point
(``mb_gmres_c64`` with a caller-owned workspace) on the same system, on two calls in a row
(the scratch array keeps the previous call's contents), and that requests beyond the
array's stated limits are refused.  Its name makes pytest collect it last.
"""
import ctypes

import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-6  # the tolerance of the GMRES-vs-dense-solve tests


def _system(pkg, dev):
    v_np, f_np = pkg.meshes.icosphere(2)
    v = torch.tensor(v_np, dtype=torch.float32, device=dev)
    f = torch.tensor(f_np, dtype=torch.int32, device=dev)
    edges, fei, _ = pkg.utils.get_edge_unique(v, f)
    solver = pkg.MeshBEMSolver3d(gaussQR=4, order_type=1, BEM_type=int(pkg.BEMType.HELMHOLTZ_MOM),
                                 wavenumber=3.0, logger=None, dtype=torch.float32, device=dev)
    Z, rhs, _ = solver.assemble_MOM(v, f, edges.shape[0], fei)
    torch.cuda.synchronize()
    return Z.contiguous(), rhs[:, 0].to(torch.complex128).contiguous()


def _lib(pkg):
    lib = ctypes.CDLL(pkg._lib.lib_path())
    P, I64, I, D = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
    lib.mb_gmres_c64_noalloc.argtypes = [P, I64, P, P, I, I, D, P, P]
    lib.mb_gmres_c64_noalloc.restype = ctypes.c_int
    lib.mb_gmres_c64.argtypes = [P, I64, P, P, I, I, D, P, ctypes.c_size_t, P, P]
    lib.mb_gmres_c64.restype = ctypes.c_int
    lib.mb_gmres_workspace_bytes.argtypes = [I64, I]
    lib.mb_gmres_workspace_bytes.restype = ctypes.c_size_t
    lib.mb_last_error.restype = ctypes.c_char_p
    return lib


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _solve_both(lib, pkg, cuda, Z, b, restart, max_iters=3000, tol=1e-9):
    """Solve once with the workspace entry point and once with the allocation-free one."""
    n = Z.shape[0]
    stream = ctypes.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)
    ws = torch.empty(lib.mb_gmres_workspace_bytes(n, restart), dtype=torch.uint8, device=cuda)
    x_ref = torch.zeros(n, dtype=torch.complex128, device=cuda)
    info_ref = pkg._lib.GmresInfo()
    rc = lib.mb_gmres_c64(_p(Z), n, _p(b), _p(x_ref), restart, max_iters, tol, _p(ws), ws.numel(),
                          ctypes.byref(info_ref), stream)
    assert rc == 0, lib.mb_last_error()
    assert info_ref.status == 0
    x = torch.zeros(n, dtype=torch.complex128, device=cuda)
    info = pkg._lib.GmresInfo()
    rc = lib.mb_gmres_c64_noalloc(_p(Z), n, _p(b), _p(x), restart, max_iters, tol, ctypes.byref(info), stream)
    assert rc == 0, lib.mb_last_error()
    assert info.status == 0 and info.rel_residual <= tol
    return x, x_ref


def test_noalloc_gmres_matches_workspace_gmres_twice(pkg, cuda):
    lib = _lib(pkg)
    Z, b = _system(pkg, cuda)
    for _ in range(2):
        x, x_ref = _solve_both(lib, pkg, cuda, Z, b, restart=50)
        assert rel_err(x.cpu().numpy(), x_ref.cpu().numpy()) < TOL


def test_noalloc_gmres_smaller_system_after_larger(pkg, cuda):
    """The scratch keeps the previous call's contents, and the offsets of the solver's arrays
    inside it move with n and the restart length: a smaller, odd-sized system with a shorter
    restart right after a larger one must not read the larger call's leftovers."""
    lib = _lib(pkg)
    Z, b = _system(pkg, cuda)
    x, x_ref = _solve_both(lib, pkg, cuda, Z, b, restart=50)
    assert rel_err(x.cpu().numpy(), x_ref.cpu().numpy()) < TOL
    n2 = 97  # odd; a leading principal block of the Galerkin matrix is itself a Galerkin matrix
    Z2 = Z[:n2, :n2].contiguous()
    b2 = b[:n2].contiguous()
    x2, x2_ref = _solve_both(lib, pkg, cuda, Z2, b2, restart=13)
    assert rel_err(x2.cpu().numpy(), x2_ref.cpu().numpy()) < TOL
    # and back to the larger system
    x3, x3_ref = _solve_both(lib, pkg, cuda, Z, b, restart=31)
    assert rel_err(x3.cpu().numpy(), x3_ref.cpu().numpy()) < TOL


def test_noalloc_gmres_rejects_sizes_beyond_its_limits(pkg, cuda):
    lib = _lib(pkg)
    dummy = torch.zeros(16, dtype=torch.float64, device=cuda)
    stream = ctypes.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)
    info = pkg._lib.GmresInfo()
    rc = lib.mb_gmres_c64_noalloc(_p(dummy), 8193, _p(dummy), _p(dummy), 10, 10, 1e-6,
                                  ctypes.byref(info), stream)
    assert rc == 4 and b"8192" in lib.mb_last_error()
    rc = lib.mb_gmres_c64_noalloc(_p(dummy), 4, _p(dummy), _p(dummy), 51, 10, 1e-6,
                                  ctypes.byref(info), stream)
    assert rc == 4 and b"restart" in lib.mb_last_error()
