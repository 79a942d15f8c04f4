"""ctypes binding of libmeshbem_gb300.so (the C ABI in include/mesh_bem_gb300.h).

The library is built in-tree by ``build.py`` (``python -c "import __graft_entry__ as g;
g.build()"``).  There is no fallback: if the library is missing or fails to load, every
operator raises.  Helpers here turn torch tensors into (pointer, size) arguments after
checking device, dtype, shape and contiguity, and pass the caller's current CUDA stream.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

from . import build as _build

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I = ctypes.c_int
_D = ctypes.c_double

# name -> argtypes (restype is always c_int)
_SIGS = {
    "mb_abi_version": [],
    "mb_mom_zmat_fe_f32": [_P, _I64, _P, _I64, _P, _P, _P, _P, _I, _P, _P, _I, _D, _I64, _P, _P, _P],
    "mb_mom_zmat_fe_f64": [_P, _I64, _P, _I64, _P, _P, _P, _P, _I, _P, _P, _I, _D, _I64, _P, _P, _P],
    "mb_mom_rhs_fe_f32": [_P, _I64, _P, _I64, _P, _P, _P, _P, _I, _D, _I64, _P, _P, _P],
    "mb_mom_rhs_fe_f64": [_P, _I64, _P, _I64, _P, _P, _P, _P, _I, _D, _I64, _P, _P, _P],
    "mb_mom_interp_js_f32": [_P, _I64, _P, _I64, _P, _P, _P, _P, _I64, _I64, _P, _P, _P],
    "mb_mom_interp_js_f64": [_P, _I64, _P, _I64, _P, _P, _P, _P, _I64, _I64, _P, _P, _P],
    "mb_mom_zmat_rwg_c64": [_P, _I64, _P, _I64, _P, _P, _P, _I64, _P, _P, _I, _P, _P, _I, _D,
                            _I64, _I64, _P, _P],
    "mb_mom_zmat_rwg_c128": [_P, _I64, _P, _I64, _P, _P, _P, _I64, _P, _P, _I, _P, _P, _I, _D,
                             _I64, _I64, _P, _P],
    "mb_mom_edge_rows": [_P, _I64, _I64, _P, _P],
    "mb_shared_vertex_pairs_workspace_bytes": [_I64, _I64],
    "mb_shared_vertex_pairs_count": [_P, _I64, _I64, _P, _I64, _P, _P],
    "mb_shared_vertex_pairs_fill": [_P, _I64, _I64, _P, _P, _P],
    "mb_mom_sym_zmat_rwg_to_host_c64": [_P, _I64, _P, _I64, _P, _I64, _D, _P, _I64, _P, _P, _I, _P],
    "mb_gmres_blockdiag_column_steps": [_P, _I64, _I64, _I, _P, _P],
    "mb_gmres_multi_column_steps": [_P, _I64, _I64, _I, _P, _P],
    "mb_mom_zmat_rwg_edges_c64": [_P, _I64, _P, _I64, _P, _P, _P, _P, _I64, _P, _P, _I, _P, _P, _I, _D,
                                  _I64, _I64, _P, _P],
    "mb_mom_zmat_rwg_gather_c64": [_P, _I64, _P, _I64, _P, _P, _P, _I64, _P, _P, _I, _P, _P, _I, _D, _I64, _I64,
                                   _P, _P],
    "mb_mom_zmat_rwg_to_host_c64": [_P, _I64, _P, _I64, _P, _P, _P, _I64, _P, _P, _I, _P, _P, _I, _D,
                                    _P, _P, _P, _I, _P],
    "mb_mom_rhs_rwg_c64": [_P, _I64, _P, _I64, _P, _P, _P, _I64, _P, _P, _I, _P, _I, _P, _P],
    "mb_mom_rhs_rwg_c128": [_P, _I64, _P, _I64, _P, _P, _P, _I64, _P, _P, _I, _P, _I, _P, _P],
    "mb_mom_interp_vert_c64": [_P, _I64, _P, _I64, _P, _P, _P, _I64, _I64, _P, _P],
    "mb_mom_interp_vert_c128": [_P, _I64, _P, _I64, _P, _P, _P, _I64, _I64, _P, _P],
    "mb_laplace_panels_f32": [_P, _I64, _P, _I64, _P, _P, _P, _P, _P, _I, _I, _I, _D, _I64, _I64,
                              _P, _P, _P],
    "mb_laplace_panels_f64": [_P, _I64, _P, _I64, _P, _P, _P, _P, _P, _I, _I, _I, _D, _I64, _I64,
                              _P, _P, _P],
    "mb_pack_tight_f32": [_P, _P, _P, _I64, _I64, _I, _P, _P],
    "mb_pack_tight_f64": [_P, _P, _P, _I64, _I64, _I, _P, _P],
    "mb_panel_relation": [_P, _I64, _P, _P],
    "mb_mom_sym_zmat_rwg_c64": [_P, _I64, _P, _I64, _P, _I64, _D, _I64, _I64, _P, _P],
    "mb_mom_sym_zmat_rwg_c128": [_P, _I64, _P, _I64, _P, _I64, _D, _I64, _I64, _P, _P],
    "mb_mom_sym_near_c64": [_P, _I64, _P, _I64, _P, _I64, _P, _I64, _D, _P, _P],
    "mb_mom_sym_near_c128": [_P, _I64, _P, _I64, _P, _I64, _P, _I64, _D, _P, _P],
    "mb_mom_sym_rhs_rwg_c64": [_P, _I64, _P, _I64, _P, _I64, _P, _I, _P, _P],
    "mb_mom_sym_rhs_rwg_c128": [_P, _I64, _P, _I64, _P, _I64, _P, _I, _P, _P],
    "mb_laplace_hypersingular_f32": [_P, _I64, _P, _I64, _P, _P, _P],
    "mb_laplace_hypersingular_f64": [_P, _I64, _P, _I64, _P, _P, _P],
    "mb_laplace_hypersingular_tight_f32": [_P, _I64, _P, _I64, _P, _P, _P],
    "mb_laplace_hypersingular_tight_f64": [_P, _I64, _P, _I64, _P, _P, _P],
    "mb_laplace_sym_f32": [_P, _I64, _P, _I64, _I, _I, _P, _I64, _I64, _I64, _P, _P],
    "mb_laplace_sym_f64": [_P, _I64, _P, _I64, _I, _I, _P, _I64, _I64, _I64, _P, _P],
    "mb_laplace_sym_tight_f32": [_P, _I64, _P, _I64, _I, _P, _I64, _I64, _I64, _P, _P],
    "mb_laplace_sym_tight_f64": [_P, _I64, _P, _I64, _I, _P, _I64, _I64, _I64, _P, _P],
    "mb_laplace_colloc_sl_f32": [_P, _I64, _P, _I64, _P, _I64, _I64, _I64, _P, _P],
    "mb_laplace_colloc_sl_f64": [_P, _I64, _P, _I64, _P, _I64, _I64, _I64, _P, _P],
    "mb_tc_selftest": [_P, _P],
    "mb_split_tf32": [_P, _I64, _P, _P, _P],
    "mb_cgemm_workspace_bytes": [_I64, _I64],
    "mb_cgemm_tf32x3": [_P, _P, _I64, _P, _I64, _P, _P, ctypes.c_size_t, _P],
    "mb_cgemm_status": [_P, _I64, _I64, _P, _P],
    "mb_gmres_multi_workspace_bytes": [_I64, _I64, _I],
    "mb_mom_sym_zmat_batched_c64": [_P, _P, _P, _P, _P, _I, _I64, _P, _I64, _P, _P],
    "mb_mom_sym_zmat_batched_c128": [_P, _P, _P, _P, _P, _I, _I64, _P, _I64, _P, _P],
    "mb_mom_sym_rhs_batched_c64": [_P, _P, _P, _P, _I, _I64, _P, _I, _I64, _P, _P],
    "mb_mom_sym_rhs_batched_c128": [_P, _P, _P, _P, _I, _I64, _P, _I, _I64, _P, _P],
    "mb_mom_ref_zmat_batched_c64": [_P, _P, _P, _P, _P, _P, _P, _I64, _P, _I, _P, _P, _I, _P, _P, _I, _P, _P],
    "mb_mom_ref_zmat_batched_persistent_c64": [_P, _P, _P, _P, _P, _P, _P, _I64, _P, _I, _P, _P, _I, _P, _P, _I, _P,
                                               _P],
    "mb_mom_ref_rhs_batched_c64": [_P, _P, _P, _P, _P, _P, _I, _I64, _P, _P, _I, _P, _I, _I64, _P, _P],
    "mb_gnn_gemm": [_P, _I, _P, _I, _I, _P, _I64, _I, _I, _I, _P, _I, _P],
    "mb_gnn_gemm_tn": [_P, _I, _P, _I64, _I, _I, _P, _P],
    "mb_gnn_colsum": [_P, _I64, _I, _P, _P],
    "mb_gnn_aggregate": [_P, _P, _I64, _I, _P, _P],
    "mb_gnn_aggregate_bwd": [_P, _P, _I64, _I, _P, _P],
    "mb_gnn_relu_bwd": [_P, _P, _I64, _P, _P],
    "mb_gnn_adam": [_P, _P, _P, _P, _I64, _D, _D, _D, _D, _I, _P, _P],
    "mb_blockdiag_matvec_c64": [_P, _P, _P, _I, _I64, _P, _I64, _I, _I, _P, _P],
    "mb_gmres_blockdiag_workspace_bytes": [_I64, _I64, _I],
    "mb_gmres_blockdiag_aug_c64": [_P, _P, _P, _I, _I64, _I, _I, _I64, _P, _P, _P, _P, _P, _I, _P, _P, _I, _I, _D,
                                   _I, _P, ctypes.c_size_t, _P, _P],
    "mb_gmres_blockdiag_c64": [_P, _P, _P, _I, _I64, _I, _I, _I64, _P, _P, _I, _I, _D, _I, _P, ctypes.c_size_t,
                               _P, _P],
    "mb_gmres_multi_c64": [_P, _P, _I64, _P, _P, _I64, _I, _I, _D, _P, ctypes.c_size_t, _P, _P],
    "mb_ray_bvh_bytes": [_I64],
    "mb_ray_bvh_build_f32": [_P, _I64, _P, _I64, _P, ctypes.c_size_t, _P],
    "mb_ray_query_f32": [_P, _I64, _P, _P, _I64, _I64, _D, _D, _P, _P],
    "mb_ray_status": [_P, _I64, _P, _P],
    "mb_radiate_h_c64": [_P, _I64, _P, _P, _P, _I64, _D, _P, _P],
    "mb_radiate_h_c128": [_P, _I64, _P, _P, _P, _I64, _D, _P, _P],
    "mb_gmres_workspace_bytes": [_I64, _I],
    "mb_gmres_c64": [_P, _I64, _P, _P, _I, _I, _D, _P, ctypes.c_size_t, _P, _P],
    "mb_gmres_real_workspace_bytes": [_I64, _I],
    "mb_gmres_f32": [_P, _I64, _P, _P, _I, _I, _D, _P, ctypes.c_size_t, _P, _P],
    "mb_gmres_f64": [_P, _I64, _P, _P, _I, _I, _D, _P, ctypes.c_size_t, _P, _P],
    "mb_gmres_c64_noalloc": [_P, _I64, _P, _P, _I, _I, _D, _P, _P],
    "mb_matvec_c64": [_P, _P, _I64, _P, _P],
    "mb_residual_c128": [_P, _P, _P, _I64, _P, _P],
    "mb_spai_workspace_bytes": [_I64],
    "mb_spai_build_c64": [_P, _P, _P, _P, _I, _I64, _I64, _P, _I64, _P, _P, _P, _P, ctypes.c_size_t, _P],
    "mb_spai_status": [_P, _I64, _P, _P],
    "mb_spai_apply_c64": [_P, _P, _I64, _P, _P, _P],
    "mb_pgmres_workspace_bytes": [_I64, _I],
    "mb_pgmres_c64": [_P, _I64, _P, _P, _D, _P, _P, _P, _P, _I, _I, _D, _I, _P, ctypes.c_size_t, _P, _P],
    "mb_half_copy_c64": [_P, _I64, _P, _P, _P],
    "mb_mom_sym_zmat_batched_rows_c64": [_P, _P, _P, _P, _P, _I, _P, _P, _I64, _I, _P, _I64, _P, _P],
    "mb_gmres_blockdiag_pc_c64": [_P, _P, _P, _I, _I64, _I, _I, _I64, _P, _P, _P, _P, _P, _I, _I, _D, _I, _P,
                                  ctypes.c_size_t, _P, _P],
    "mb_pgmres_c128": [_P, _I64, _P, _P, _P, _P, _I, _I, _D, _I, _P, ctypes.c_size_t, _P, _P],
}

_RESTYPES = {"mb_gmres_workspace_bytes": ctypes.c_size_t, "mb_ray_bvh_bytes": ctypes.c_size_t,
             "mb_gmres_real_workspace_bytes": ctypes.c_size_t, "mb_cgemm_workspace_bytes": ctypes.c_size_t,
             "mb_gmres_multi_workspace_bytes": ctypes.c_size_t,
             "mb_gmres_blockdiag_workspace_bytes": ctypes.c_size_t,
             "mb_shared_vertex_pairs_workspace_bytes": ctypes.c_int64,
             "mb_spai_workspace_bytes": ctypes.c_size_t, "mb_pgmres_workspace_bytes": ctypes.c_size_t}


class GmresInfo(ctypes.Structure):
    """mb_gmres_info (include/mesh_bem_gb300.h)."""

    _fields_ = [("iterations", ctypes.c_int64), ("restarts", ctypes.c_int64),
                ("rel_residual", ctypes.c_double), ("status", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]

ABI_VERSION = 1

_lock = threading.Lock()
_lib = None


class MeshBEMError(RuntimeError):
    """Raised when a libmeshbem_gb300 entry point returns an error code."""


def lib_path() -> str:
    return _build.LIB


def load():
    """Load (never build) the library; raises if it is absent or incompatible."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            raise ImportError(
                f"libmeshbem_gb300.so not found at {path}: build it first with "
                "`python -c \"import __graft_entry__ as g; g.build()\"`")
        lib = ctypes.CDLL(path)
        lib.mb_last_error.restype = ctypes.c_char_p
        lib.mb_last_error.argtypes = []
        for name, args in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        v = lib.mb_abi_version()
        if v != ABI_VERSION:
            raise ImportError(f"libmeshbem_gb300 ABI {v} != expected {ABI_VERSION}; rebuild it")
        _lib = lib
    return _lib


# number of C-ABI calls made so far (each launches one or more of the library's kernels)
call_count = 0


def call(name: str, *args) -> None:
    global call_count
    lib = load()
    call_count += 1
    rc = getattr(lib, name)(*args)
    if rc != 0:
        msg = lib.mb_last_error().decode(errors="replace")
        raise MeshBEMError(f"{name} failed (code {rc}): {msg}")


def exported_symbols() -> list[str]:
    return ["mb_last_error", *_SIGS.keys()]


# ---------------------------------------------------------------------------------------
# tensor argument helpers
# ---------------------------------------------------------------------------------------

def stream_of(t: torch.Tensor) -> int:
    return torch.cuda.current_stream(t.device).cuda_stream


def ptr(t: torch.Tensor | None):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def check_tensor(t: torch.Tensor, name: str, dtype=None, device=None, ndim=None, shape=None):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if t.device.type != "cuda":
        raise ValueError(f"{name} must be a CUDA tensor (got {t.device}); this path has no CPU "
                         "implementation")
    if device is not None and t.device != device:
        raise ValueError(f"{name} is on {t.device}, expected {device}")
    if dtype is not None and t.dtype not in (dtype if isinstance(dtype, tuple) else (dtype,)):
        raise TypeError(f"{name} must have dtype {dtype} (got {t.dtype})")
    if ndim is not None and t.dim() != ndim:
        raise ValueError(f"{name} must have {ndim} dims (got shape {tuple(t.shape)})")
    if shape is not None:
        for i, s in enumerate(shape):
            if s is not None and t.shape[i] != s:
                raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {shape}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    return t


def sfx(dtype: torch.dtype) -> str:
    if dtype == torch.float32:
        return "f32"
    if dtype == torch.float64:
        return "f64"
    raise TypeError(f"unsupported float dtype {dtype} (float32 or float64)")


def csfx(dtype: torch.dtype) -> str:
    return "c64" if dtype in (torch.float32, torch.complex64) else "c128"
