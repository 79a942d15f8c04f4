"""Forward-only autograd wrappers of the MoM operators (src/mesh_BEM/kernel_functions.py:26-171).

Same classes, same ``apply`` signatures and return values as the reference: each allocates
zeroed outputs, calls the ``mesh_MOM_3d`` op and returns the complex result.  The op
module here is the sm_103a drop-in (``mesh_MOM_3d.py``), not a JIT build.
"""
from __future__ import annotations

from typing import Any

import torch

from . import mesh_MOM_3d


class MeshMOMZmatKernel(torch.autograd.Function):
    """Face-edge impedance matrix [1, 3F, 3F] complex (kernel_functions.py:26-74)."""

    @staticmethod
    def forward(ctx, verts, faces, face_areas, face_normals, gaussian_points_1d_x,
                gaussian_weights_1d_x, gaussian_points_1d_y, gaussian_weights_1d_y,
                wavenumber: float) -> Any:
        n_faces, dim = faces.shape
        zr = torch.zeros((1, n_faces * dim, n_faces * dim), dtype=verts.dtype, device=verts.device)
        zi = torch.zeros_like(zr)
        mesh_MOM_3d.create_MOM_Zmat_3d_forward(
            verts, faces, face_areas, face_normals, gaussian_points_1d_x, gaussian_weights_1d_x,
            gaussian_points_1d_y, gaussian_weights_1d_y, zr, zi, wavenumber)
        return torch.complex(zr, zi)


class MeshMOMRhsKernel(torch.autograd.Function):
    """Face-edge excitation [1, F, 3, 1] complex (kernel_functions.py:77-121)."""

    @staticmethod
    def forward(ctx, verts, faces, face_areas, face_normals, gaussian_points_1d,
                gaussian_weights_1d, wavenumber: float) -> Any:
        n_faces, dim = faces.shape
        rr = torch.zeros((1, n_faces, dim, 1), dtype=verts.dtype, device=verts.device)
        ri = torch.zeros_like(rr)
        mesh_MOM_3d.create_MOM_rhs_3d_forward(verts, faces, face_areas, face_normals,
                                              gaussian_points_1d, gaussian_weights_1d, rr, ri,
                                              wavenumber)
        return torch.complex(rr, ri)


class MeshMOMInterpolateJsKernel(torch.autograd.Function):
    """Per-face vertex currents [B, 3F, 3] complex (kernel_functions.py:124-171)."""

    @staticmethod
    def forward(ctx, verts, faces, face_edge_indices, face_areas, edge_I_coeff) -> Any:
        n_faces, dim = faces.shape
        batch = edge_I_coeff.shape[0]
        jr = torch.zeros((batch, n_faces * dim, dim), dtype=verts.dtype, device=verts.device)
        ji = torch.zeros_like(jr)
        ir = edge_I_coeff.real.to(verts.dtype).contiguous()
        ii = edge_I_coeff.imag.to(verts.dtype).contiguous()
        mesh_MOM_3d.interpolate_Icoeff_to_Js_3d_forward(verts, faces, face_edge_indices, face_areas,
                                                        ir, ii, jr, ji)
        return torch.complex(jr, ji)
