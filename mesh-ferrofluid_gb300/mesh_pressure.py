"""``MeshPressure``: the ferrofluid pressure projection, the caller of the Laplace solver's
mixed boundary-value path (src/mesh_ferrofluid/mesh_pressure.py:19-163).

Per step: Neumann data dp/dn = (rho/dt) (v - v_solid).n on Neumann vertices; Dirichlet
data p = -rho g.x - P_mag + sigma kappa on Dirichlet vertices, with the signed mean
curvature from the cotangent Laplacian as the reference computes it (:112-127); the mixed
Laplace problem solved by ``MeshBEMSolver3d.solve``; grad p = (dp/dn) n + the surface
gradient of p; v_new = v - (dt/rho) grad p.

The reference cannot run this path (its hypersingular layer is None); here the solve uses
``HyperSingularLayer3d`` with ``rule="dunavant7"`` by default (the reference rule is
available through ``rule="reference"`` but its hypersingular operator is indefinite on
coarse meshes).  ``solver`` is passed to ``MeshBEMSolver3d`` ("lu" as the reference, or
"schur").  Diagnostics go to the logger instead of stdout.
"""
from __future__ import annotations

import torch

from .mesh_BEM_solver_3d import MeshBEMSolver3d
from .utils import (
    BEMType,
    BoundaryType,
    VertexType,
    compute_face_normals,
    compute_mesh_vert_tangent_gradient,
    compute_vert_normals,
    cot_laplacian,
)


class MeshPressure:
    def __init__(self, density_fluid: float, gravity_strength: float, surface_tension, contact_angle,
                 gaussQR: int, order_type: int, logger, device: torch.device = torch.device("cpu"),
                 dtype: torch.dtype = torch.float32, rule: str = "dunavant7", solver: str = "lu"):
        self.gaussQR = gaussQR
        self.order_type = order_type
        self.logger = logger
        self.device = device
        self.dtype = dtype
        self.density_fluid = density_fluid
        self.gravity = torch.tensor([0.0, -gravity_strength, 0.0], device=device, dtype=dtype)
        self.surface_tension = surface_tension
        self.contact_angle = contact_angle
        self.BEM_solver = MeshBEMSolver3d(gaussQR=gaussQR, order_type=order_type, BEM_type=int(BEMType.LAPLACE),
                                          wavenumber=1.0, logger=logger, device=device, dtype=dtype, rule=rule,
                                          solver=solver)

    def signed_mean_curvature(self, verts: torch.Tensor, faces: torch.Tensor,
                              vert_normals: torch.Tensor) -> torch.Tensor:
        """kappa [V, 1] = 0.5 |L x| sign((L x).n) with L x = 1/2 inv_area sum_j w_ij (x_j - x_i)."""
        L, inv_areas = cot_laplacian(verts, faces)
        i, j = L.indices()
        w = L.values()[:, None]
        lap = torch.zeros_like(verts)
        lap.index_add_(0, j, w * (verts[i] - verts[j]))  # sum over i of L[i, j] (x_i - x_j)
        lap = 0.5 * inv_areas * lap
        H = 0.5 * lap.norm(dim=-1)
        return (H * torch.sign((lap * vert_normals).sum(-1))).reshape(-1, 1)

    def solve(self, verts: torch.Tensor, faces: torch.Tensor, dt: float, vel: torch.Tensor,
              vert_bc_flags: torch.Tensor, P_mag: torch.Tensor = None) -> torch.Tensor:
        """New vertex velocities [B, V, 3] after the pressure projection."""
        batch, n_verts, _ = vel.shape
        rho = self.density_fluid
        vert_normals = compute_vert_normals(verts, faces)
        face_normals = compute_face_normals(verts, faces)
        dpdn = (rho / dt) * (vel * vert_normals).sum(-1, keepdim=True)  # solid velocity 0
        dpdn = torch.where(vert_bc_flags == int(BoundaryType.DIRICHLET), torch.zeros_like(dpdn), dpdn)
        p = -rho * (self.gravity * verts).sum(-1, keepdim=True)
        if P_mag is not None:
            p = p - P_mag.reshape(n_verts, 1)
        p = p + self.surface_tension * self.signed_mean_curvature(verts, faces, vert_normals)
        p = p.reshape(1, n_verts, 1).repeat(batch, 1, 1)
        p = torch.where(vert_bc_flags == int(BoundaryType.NEUMANN), torch.zeros_like(p), p)
        vert_dpdn, vert_p = self.BEM_solver.solve(verts=verts, faces=faces, vert_bc_Dirichlet=p,
                                                  vert_bc_Neumann=dpdn, vert_bc_flags=vert_bc_flags,
                                                  Amat_scaler=1.0)
        grad_n = vert_dpdn.to(vel.dtype) * vert_normals
        grad_t = compute_mesh_vert_tangent_gradient(vert_p.to(vel.dtype), verts, faces, face_normals)
        grad = grad_n + grad_t
        if self.logger is not None:
            self.logger.InfoLog(f"dpdn = {grad_n.norm(dim=-1).max()}")
            self.logger.InfoLog(f"dpdt = {grad_t.norm(dim=-1).max()}")
            if int((vert_bc_flags == int(VertexType.TRIPLE_JUNCTION)).sum()) > 0:
                self.logger.ErrorLog("Not implemented for triple-junction points")
        return vel - (dt / rho) * grad
