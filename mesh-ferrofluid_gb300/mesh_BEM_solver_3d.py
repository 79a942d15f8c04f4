"""``MeshBEMSolver3d``: the reference's solver facade on the sm_103a kernels.

Same constructor and public methods as ``src/mesh_BEM/mesh_BEM_solver_3d.py:31-373``:

* ``MeshBEMSolver3d(gaussQR, order_type, BEM_type, wavenumber, logger, dtype, device)``
  builds the test rule (gaussQR) and source rule (gaussQR - 1) (:85-94) and the single,
  double and rhs layers (:54-83).
* ``solve_MOM(verts, faces, edges, face_edge_indices) -> vert_Js [1, V, 3] complex``
  (:96-195).  The face-edge matrix, its scatter onto RWG edges and the excitation scatter
  are fused into two kernels (``assemble_Z_rwg``, ``assemble_rhs_rwg``); the dense solve is
  ``torch.linalg.solve`` as in the reference (:174); the interpolation and vertex scatter
  are one kernel (``interpolate_vert_js``).
* ``solve(verts, faces, vert_bc_Dirichlet, vert_bc_Neumann, vert_bc_flags, Amat_scaler=None)
  -> (Neumann [B, V, 1], Dirichlet [B, V, 1])`` (:197-373) for Dirichlet, Neumann and mixed
  vertex data.  The reference runs only the all-Dirichlet case (its hypersingular layer is
  None); here the Neumann and mixed cases use ``HyperSingularLayer3d`` and the block
  system of the reference's layout [[V, -K], [K^T, D]] (:306-341) with the masks taken
  from ``vert_bc_flags`` (the reference builds them from the data values) and the rows of
  the right-hand side matched to the unknowns.  The pure Neumann matrix D is singular
  (constants); it is solved as D + a a^T with a_i = int phi_i (solution of zero mean for
  compatible data).  For these cases use ``rule="dunavant7"``.

Extra keyword ``solver`` selects "lu" (reference behaviour, ``torch.linalg.solve``) or
"gmres" (``mb_gmres_c64`` for the MoM system, ``mb_gmres_f32`` for the Laplace systems:
FP32 matrix-vector products, FP64 Arnoldi and refinement residual; float32 meshes only,
float64 meshes keep LU) or "schur" (Laplace only: Cholesky factors of V on the
Dirichlet vertices and of the Schur complement D + K V^-1 K^T on the Neumann ones, from
the symmetric parts of V and D; other BEM types keep LU).  Extra
keyword ``rule`` selects "reference" (the reference's EFIE + MFIE operator and collapsed
Gauss rule, parity path) or "dunavant7" (EFIE with the 7-point rule on both triangles and
closed-form singular integrals for pairs sharing a vertex, in FP64; excitation = the
incident E field only).  All tensors must live on a
CUDA device: there is no CPU implementation.
"""
from __future__ import annotations

from typing import List

import torch

from .layers import (
    DoubleLayer3d,
    HyperSingularLayer3d,
    RhsLayer3d,
    SingleLayer3d,
    laplace_sym_tight,
)
from .mesh_MOM_3d import (
    assemble_rhs_rwg,
    assemble_rhs_rwg_sym,
    assemble_Z_rwg,
    assemble_Z_rwg_sym,
    gmres,
    gmres_real,
    interpolate_vert_js,
    reference_plane_wave,
)
from .utils import (
    BEMType,
    BoundaryType,
    OrderType,
    compute_face_areas,
    compute_face_normals,
    compute_panel_relation,
    compute_vert_areas,
    get_gaussion_integration_points_and_weights,
    shared_vertex_pairs,
)


def _sym_part(A: torch.Tensor) -> torch.Tensor:
    return 0.5 * (A + A.transpose(0, 1))


def _check_cholesky(*infos: torch.Tensor) -> None:
    """One host synchronisation for all factorisations of a solve."""
    bad = [int(i) for i in torch.stack([i.reshape(()) for i in infos]).cpu()]
    if any(bad):
        raise RuntimeError(f"a symmetric part is not positive definite (cholesky info {bad})")


def _spd_solve(A: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """A x = b through the Cholesky factor of A's symmetric part (V, or D + a a^T)."""
    L, info = torch.linalg.cholesky_ex(_sym_part(A))
    x = torch.cholesky_solve(b.reshape(-1, 1), L).reshape(-1)
    _check_cholesky(info)
    return x


def _schur_solve(Vdd, B, Dnn, r1, r2):
    """The mixed block system [[Vdd, -B], [B^T, Dnn]] [x1; x2] = [r1; r2] by Cholesky factors:
    Vdd = L L^T, W = L^-1 B, S = Dnn + W^T W (symmetric positive definite),
    x2 = S^-1 (r2 - W^T L^-1 r1), x1 = L^-T (L^-1 r1 + W x2).  Vdd and Dnn enter through
    their symmetric parts (the Galerkin operators are symmetric; the assembled ones differ
    at the quadrature error)."""
    L, info_v = torch.linalg.cholesky_ex(_sym_part(Vdd))
    W = torch.linalg.solve_triangular(L, B, upper=False)
    y = torch.linalg.solve_triangular(L, r1.reshape(-1, 1), upper=False)
    Ls, info_s = torch.linalg.cholesky_ex(_sym_part(Dnn + W.transpose(0, 1) @ W))
    x2 = torch.cholesky_solve(r2.reshape(-1, 1) - W.transpose(0, 1) @ y, Ls)
    x1 = torch.linalg.solve_triangular(L.transpose(0, 1), y + W @ x2, upper=True)
    _check_cholesky(info_v, info_s)
    return torch.cat((x1, x2)).reshape(-1)


class MeshBEMSolver3d:
    rank = 3

    def __init__(self, gaussQR: int, order_type: int, BEM_type: int, wavenumber: float, logger=None,
                 dtype: torch.dtype = torch.float32, device: torch.device = torch.device("cpu"),
                 solver: str = "lu", gmres_restart: int = 50, gmres_tol: float = 1e-6,
                 gmres_max_iters: int = 2000, rule: str = "reference"):
        self._gaussQR = gaussQR
        self._order_type = order_type
        self._BEM_type = BEM_type
        self._wavenumber = wavenumber
        self.logger = logger
        self.device = torch.device(device)
        self.dtype = dtype
        if solver not in ("lu", "gmres", "schur"):
            raise ValueError(f"unknown solver {solver!r}")
        self.solver = solver
        self.gmres_restart = gmres_restart
        self.gmres_tol = gmres_tol
        self.gmres_max_iters = gmres_max_iters
        self.last_solve_info = None
        if rule not in ("reference", "dunavant7"):
            raise ValueError(f"unknown rule {rule!r}")
        self.rule = rule
        kw = dict(gaussQR=gaussQR, order_type=order_type, BEM_type=BEM_type, wavenumber=wavenumber,
                  logger=logger, dtype=dtype, device=self.device, rule=rule)
        self.single_layer = SingleLayer3d(**kw)
        self.double_layer = DoubleLayer3d(**kw)
        self.hypersingular_layer = HyperSingularLayer3d(**kw)
        self.rhs_layer = RhsLayer3d(parent=self, **kw)
        self.gaussian_points_1d_x, self.gaussian_weights_1d_x = \
            get_gaussion_integration_points_and_weights(gaussQR, device=self.device, dtype=dtype)
        self.gaussian_points_1d_y, self.gaussian_weights_1d_y = \
            get_gaussion_integration_points_and_weights(gaussQR - 1, device=self.device, dtype=dtype)

    gaussQR = property(lambda self: self._gaussQR)
    order_type = property(lambda self: self._order_type)
    BEM_type = property(lambda self: self._BEM_type)
    wavenumber = property(lambda self: self._wavenumber)

    def InfoLog(self, *a, **k):
        return self.logger.InfoLog(*a, **k) if self.logger is not None else None

    # ------------------------------------------------------------------ MoM
    def _rules_on(self, dev, dt):
        return [t.to(device=dev, dtype=dt).contiguous() for t in (
            self.gaussian_points_1d_x, self.gaussian_weights_1d_x,
            self.gaussian_points_1d_y, self.gaussian_weights_1d_y,
            self.rhs_layer.gaussian_points_1d, self.rhs_layer.gaussian_weights_1d)]

    def assemble_MOM(self, verts: torch.Tensor, faces: torch.Tensor, n_edges: int,
                     face_edge_indices: torch.Tensor, waves: torch.Tensor | None = None):
        """RWG matrix Z [E, E] and excitation [E, n_rhs] (reference wave when ``waves`` is None)."""
        verts = verts.contiguous()
        faces = faces.to(torch.int32).contiguous()
        fei = face_edge_indices.to(torch.int32).reshape(-1).contiguous()
        dev, dt = verts.device, verts.dtype
        areas = compute_face_areas(vertices=verts, faces=faces, keepdim=True).contiguous()
        if waves is None:
            waves = reference_plane_wave(self.wavenumber, device=dev)
        if self.rule == "dunavant7":
            Z = assemble_Z_rwg_sym(verts, faces, fei, n_edges, self.wavenumber)
            rhs = assemble_rhs_rwg_sym(verts, faces, fei, n_edges, waves)
            return Z, rhs, areas
        gpx, gwx, gpy, gwy, gp, gw = self._rules_on(dev, dt)
        normals = compute_face_normals(vertices=verts, faces=faces).contiguous()
        Z = assemble_Z_rwg(verts, faces, areas, normals, fei, n_edges, gpx, gwx, gpy, gwy,
                           self.wavenumber)
        rhs = assemble_rhs_rwg(verts, faces, areas, normals, fei, n_edges, gp, gw, waves)
        return Z, rhs, areas

    def solve_MOM(self, verts: torch.Tensor, faces: torch.Tensor, edges: torch.Tensor,
                  face_edge_indices: torch.Tensor) -> torch.Tensor:
        """Mesh-based MoM solve; returns [1, N_verts, 3] complex vertex currents."""
        assert self._BEM_type == int(BEMType.HELMHOLTZ_MOM)
        n_edges = edges.shape[0]
        Z, rhs, areas = self.assemble_MOM(verts, faces, n_edges, face_edge_indices)
        if self.solver == "gmres" and Z.dtype == torch.complex64:
            I_coeff, self.last_solve_info = gmres(Z, rhs, restart=self.gmres_restart,
                                                  tol=self.gmres_tol, max_iters=self.gmres_max_iters)
            I_coeff = I_coeff.to(Z.dtype)
        else:
            I_coeff = torch.linalg.solve(Z, rhs)  # [E, 1], as the reference (:174)
        fei = face_edge_indices.to(torch.int32).reshape(-1).contiguous()
        return interpolate_vert_js(verts.contiguous(), faces.to(torch.int32).contiguous(), fei,
                                   areas, I_coeff.reshape(1, n_edges))

    # ------------------------------------------------------------------ Laplace / BEM
    def solve(self, verts: torch.Tensor, faces: torch.Tensor, vert_bc_Dirichlet: torch.Tensor,
              vert_bc_Neumann: torch.Tensor, vert_bc_flags: torch.Tensor,
              Amat_scaler: float = None) -> List[torch.Tensor]:
        n_verts = verts.shape[-2]
        batch = vert_bc_flags.shape[0]
        faces = faces.to(torch.int32).contiguous()
        verts = verts.contiguous()
        sym = self.rule == "dunavant7" and not BEMType.belong_Helmholtz(self.BEM_type)
        areas = normals = None
        if not sym:  # the reference rule's layers take them
            areas = compute_face_areas(vertices=verts, faces=faces, keepdim=True).contiguous()
            normals = compute_face_normals(vertices=verts, faces=faces).contiguous()
        # the symmetric rule needs only the face pairs sharing a vertex (O(F)), not the
        # dense [F, F] relation of the reference rule
        near = shared_vertex_pairs(faces, n_verts) if sym else None
        panel_relations = None if sym else compute_panel_relation(faces)
        neu_list, dir_list = [], []
        mats = {}
        layers = {"V": self.single_layer, "K": self.double_layer, "D": self.hypersingular_layer}
        schur = self.solver == "schur" and self.BEM_type == int(BEMType.LAPLACE)

        def tight(name):
            if name not in mats and sym and self.order_type == int(OrderType.LINEAR):
                # packed straight from the face pairs; the [F, F, 3, 3] panels are not kept
                # faces were validated by shared_vertex_pairs (its count phase checks the ids)
                mats[name] = laplace_sym_tight(verts, faces, {"V": 1, "K": 2, "D": 3}[name], near,
                                               check_indices=not faces.is_cuda)
            if name not in mats and sym:
                layers[name].compute_sym(verts, faces, near)
                mats[name] = layers[name]._tight(verts, faces)
            if name not in mats:
                if name == "V":
                    self.single_layer.compute_Vmat(verts, faces, areas, normals, panel_relations)
                    mats[name] = self.single_layer.get_Vmat_tight(verts=verts, faces=faces)
                elif name == "K":
                    self.double_layer.compute_Kmat(verts, faces, areas, normals, panel_relations)
                    mats[name] = self.double_layer.get_Kmat_tight(verts=verts, faces=faces)
                else:
                    self.hypersingular_layer.compute_Dmat(verts, faces, areas, normals, panel_relations)
                    mats[name] = self.hypersingular_layer.get_Dmat_tight(verts=verts, faces=faces)
            return mats[name]

        for b in range(batch):
            is_d = (vert_bc_flags[b] == int(BoundaryType.DIRICHLET)).reshape(-1)
            is_n = (vert_bc_flags[b] == int(BoundaryType.NEUMANN)).reshape(-1)
            n_d, n_n = int(is_d.sum()), int(is_n.sum())
            self.InfoLog(f"Batch [{b}]: (Vertex attached) number of Dirichlet B.C. = {n_d}, "
                         f"number of Neumann B.C. = {n_n}, number of whole zone = "
                         f"{vert_bc_flags[b].numel()}")
            if n_d + n_n == 0:
                raise ValueError("no boundary data")
            K = tight("K")
            V = tight("V") if n_d else None
            D = tight("D") if n_n and self.BEM_type != int(BEMType.HELMHOLTZ_MOM) else None
            self.rhs_layer.compute_rhs(verts, faces, vert_bc_Dirichlet[b:b + 1], vert_bc_Neumann[b:b + 1],
                                       vert_bc_flags[b:b + 1], K_tight=K, V_tight=V, D_tight=D)
            rhs = self.rhs_layer.get_rhs_vec().reshape(-1)
            neu = vert_bc_Neumann[b].reshape(n_verts, 1).clone()
            dirv = vert_bc_Dirichlet[b].reshape(n_verts, 1).clone()
            if n_n == 0:
                A = V
            elif n_d == 0:
                if self.BEM_type == int(BEMType.HELMHOLTZ_MOM):
                    A = K.clone()
                    va = compute_vert_areas(vertices=verts, faces=faces).reshape(-1).to(K.dtype)
                    A[torch.arange(n_verts), torch.arange(n_verts)] = -0.5 * va
                else:
                    a = compute_vert_areas(vertices=verts, faces=faces).reshape(-1, 1).to(D.dtype)
                    A = D + a @ a.T
            else:
                ks = K.transpose(0, 1)  # Galerkin <phi_i, K phi_j>
                rhs = torch.cat((rhs[is_d], rhs[is_n]))
                A = None if schur else torch.cat(
                    (torch.cat((V[is_d][:, is_d], -ks[is_d][:, is_n]), 1),
                     torch.cat((ks.transpose(0, 1)[is_n][:, is_d], D[is_n][:, is_n]), 1)), 0)
            if Amat_scaler is not None and A is not None:
                A = Amat_scaler * A
            if schur:
                if n_n and n_d:
                    # one index list per mask (each boolean index would synchronise again)
                    i_d, i_n = torch.nonzero(is_d).reshape(-1), torch.nonzero(is_n).reshape(-1)
                    sol = _schur_solve(V.index_select(0, i_d).index_select(1, i_d),
                                       ks.index_select(0, i_d).index_select(1, i_n),
                                       D.index_select(0, i_n).index_select(1, i_n),
                                       rhs[:n_d].to(K.dtype), rhs[n_d:].to(K.dtype))
                    if Amat_scaler is not None:  # (s A) x = rhs
                        sol = sol / Amat_scaler
                else:
                    sol = _spd_solve(A, rhs.to(A.dtype))
                sol = sol.to(neu.dtype)
            elif self.solver == "gmres" and A.dtype == torch.float32:
                x, info = gmres_real(A.contiguous(), rhs, restart=self.gmres_restart, tol=self.gmres_tol,
                                     max_iters=self.gmres_max_iters)
                self.last_solve_info = info
                sol = x.to(neu.dtype)
            else:
                sol = torch.linalg.solve(A, rhs.to(A.dtype)).to(neu.dtype)
            if n_n == 0:
                neu = sol.reshape(n_verts, 1)
            elif n_d == 0:
                dirv = sol.reshape(n_verts, 1)
            else:
                neu[is_d] = sol[:n_d, None]
                dirv[is_n] = sol[n_d:, None]
            neu_list.append(neu)
            dir_list.append(dirv)
        return torch.stack(neu_list, 0), torch.stack(dir_list, 0)
