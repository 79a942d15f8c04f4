"""Galerkin layer operators of the 3D Laplace / Helmholtz BEM path.

Mirrors the reference's layer classes and the integration routine they share:

* ``double_integration_on_panels_3d`` (src/mesh_BEM/utils/integrations_3d.py:252-452) --
  same signature and result ([F_y, F_x, nphi, nphi]); the O(F^2 * rule) work runs in the
  sm_103a panel kernel (``mb_laplace_panels_*``);
* ``SingleLayer3d`` / ``DoubleLayer3d`` (single_layer/single_layer_3d.py:43-68,
  double_layer/double_layer_3d.py:43-68, abstract layers :17-98) with ``compute_Vmat`` /
  ``compute_Kmat``, ``get_*mat_unpacked`` and ``get_*mat_tight``;
* ``RhsLayer3d.compute_rhs`` (rhs_layer/rhs_layer_3d.py:74-203), Dirichlet branch
  gk = 1/2 f |A_v| + K^T f.  Mixed/Neumann data need the hypersingular operator, which the
  reference never implemented (integrations_3d.py:440-442); they raise
  NotImplementedError here instead of crashing on an attribute of ``None``.
"""
from __future__ import annotations

import torch

from . import _lib
from .mesh_MOM_3d import check_face_range
from .utils import (
    BEMType,
    BoundaryType,
    LayerType,
    OrderType,
    collapsed_rule_2d,
    compute_vert_areas,
    get_gaussion_integration_points_and_weights,
    pack_matrix_tight,
    panel_rule_table,
)


def double_integration_on_panels_3d(BEM_type: int, order_type: int, verts: torch.Tensor,
                                    faces: torch.Tensor, face_areas: torch.Tensor,
                                    face_normals: torch.Tensor, gauss_weightsx: torch.Tensor,
                                    gauss_weightsy: torch.Tensor, rands_x: torch.Tensor,
                                    rands_y: torch.Tensor, panel_relations: torch.Tensor,
                                    wavenumber: float = 1.0,
                                    layer_type: int = int(LayerType.SINGLE_LAYER)) -> torch.Tensor:
    """[F_y, F_x, nphi, nphi] panel integrals; ``panel_relations`` may be None (derived)."""
    if layer_type == int(LayerType.HYPERSINGULAR_LAYER):
        raise NotImplementedError("Not implemented for hypersingular")
    if layer_type not in (int(LayerType.SINGLE_LAYER), int(LayerType.DOUBLE_LAYER)):
        raise ValueError(f"unknown layer_type {layer_type}")
    _lib.check_tensor(verts, "verts", dtype=(torch.float32, torch.float64), ndim=2)
    dt, dev = verts.dtype, verts.device
    faces = faces.to(torch.int32).contiguous()
    _lib.check_tensor(faces, "faces", device=dev, ndim=2)
    nf = faces.shape[0]
    check_face_range(faces, verts.shape[0])
    areas = face_areas.to(dt).contiguous()
    if areas.numel() != nf or face_normals.numel() != 3 * nf:
        raise ValueError("face_areas / face_normals must have F / 3F entries")
    normals = face_normals.to(dt).contiguous()
    table, seg = panel_rule_table(rands_x.to(dt), rands_y.to(dt), gauss_weightsx.to(dt),
                                  gauss_weightsy.to(dt))
    table = table.to(dev).contiguous()
    seg_c = (torch.tensor(seg, dtype=torch.int32)).numpy()
    rel = None
    if panel_relations is not None:
        rel = panel_relations.to(device=dev, dtype=torch.uint8).contiguous()
        if rel.shape != (nf, nf):
            raise ValueError("panel_relations must be [F, F]")
    nphi = 3 if order_type == int(OrderType.LINEAR) else 1
    kind = 1 if BEMType.belong_Helmholtz(BEM_type) else 0
    out_r = torch.empty((nf, nf, nphi, nphi), dtype=dt, device=dev)
    out_i = torch.empty_like(out_r) if kind == 1 else None
    _lib.call(f"mb_laplace_panels_{_lib.sfx(dt)}", _lib.ptr(verts), verts.shape[0], _lib.ptr(faces),
              nf, _lib.ptr(areas), _lib.ptr(normals), _lib.ptr(table),
              seg_c.ctypes.data_as(__import__("ctypes").c_void_p), _lib.ptr(rel), int(layer_type),
              1 if nphi == 3 else 0, kind, float(wavenumber), 0, nf, _lib.ptr(out_r), _lib.ptr(out_i),
              _lib.stream_of(verts))
    return torch.complex(out_r, out_i) if kind == 1 else out_r


class _AbstractLayer:
    rank = 3
    layer_type = int(LayerType.SINGLE_LAYER)

    def __init__(self, gaussQR: int, order_type: int, BEM_type: int, wavenumber: float, logger,
                 dtype: torch.dtype = torch.float32, device: torch.device = torch.device("cpu")):
        self._gaussQR = gaussQR
        self._order_type = order_type
        self._BEM_type = BEM_type
        self._wavenumber = wavenumber
        self.logger = logger
        self.device = device
        self.dtype = dtype
        self.gaussian_points_1d, self.gaussian_weights_1d = \
            get_gaussion_integration_points_and_weights(gaussQR, device=device, dtype=dtype)
        rands, w = collapsed_rule_2d(self.gaussian_points_1d, self.gaussian_weights_1d)
        self.r1, self.r2 = rands[:, 0:1], rands[:, 1:2]
        self.gauss_weights = w
        self._unpacked = None
        self.initialized = False

    gaussQR = property(lambda self: self._gaussQR)
    order_type = property(lambda self: self._order_type)
    BEM_type = property(lambda self: self._BEM_type)
    wavenumber = property(lambda self: self._wavenumber)

    def _compute(self, verts, faces, face_areas, face_normals, panel_relations):
        rands = torch.cat((self.r1, self.r2), dim=-1)
        self._unpacked = double_integration_on_panels_3d(
            BEM_type=self.BEM_type, order_type=self.order_type, verts=verts, faces=faces,
            face_areas=face_areas, face_normals=face_normals, gauss_weightsx=self.gauss_weights,
            gauss_weightsy=self.gauss_weights, rands_x=rands, rands_y=rands,
            panel_relations=panel_relations, wavenumber=self.wavenumber, layer_type=self.layer_type)
        self.initialized = True

    def _tight(self, verts, faces):
        return pack_matrix_tight(self.order_type, self._unpacked, verts, faces)

    def InfoLog(self, *a, **k):
        return self.logger.InfoLog(*a, **k) if self.logger else None


class SingleLayer3d(_AbstractLayer):
    layer_type = int(LayerType.SINGLE_LAYER)

    def compute_Vmat(self, verts, faces, face_areas, face_normals, panel_relations=None):
        self._compute(verts, faces, face_areas, face_normals, panel_relations)

    def get_Vmat_unpacked(self):
        return self._unpacked

    def get_Vmat_tight(self, verts, faces):
        return self._tight(verts, faces)


class DoubleLayer3d(_AbstractLayer):
    layer_type = int(LayerType.DOUBLE_LAYER)

    def compute_Kmat(self, verts, faces, face_areas, face_normals, panel_relations=None):
        self._compute(verts, faces, face_areas, face_normals, panel_relations)

    def get_Kmat_unpacked(self):
        return self._unpacked

    def get_Kmat_tight(self, verts, faces):
        return self._tight(verts, faces)


class RhsLayer3d:
    rank = 3

    def __init__(self, parent, gaussQR: int, order_type: int, BEM_type: int, wavenumber: float,
                 logger, dtype=torch.float32, device=torch.device("cpu")):
        self.parent = parent
        self._gaussQR = gaussQR
        self._order_type = order_type
        self._BEM_type = BEM_type
        self._wavenumber = wavenumber
        self.logger = logger
        self.device = device
        self.dtype = dtype
        self.gaussian_points_1d, self.gaussian_weights_1d = \
            get_gaussion_integration_points_and_weights(gaussQR, device=device, dtype=dtype)
        rands, w = collapsed_rule_2d(self.gaussian_points_1d, self.gaussian_weights_1d)
        self.r1, self.r2 = rands[:, 0:1], rands[:, 1:2]
        self.gauss_weights = w
        self.rhs_vec = None
        self.initialized = False

    gaussQR = property(lambda self: self._gaussQR)
    order_type = property(lambda self: self._order_type)
    BEM_type = property(lambda self: self._BEM_type)
    wavenumber = property(lambda self: self._wavenumber)

    def compute_rhs(self, verts, faces, vert_bc_Dirichlet, vert_bc_Neumann, vert_bc_flags,
                    K_tight=None):
        """rhs [B, V, 1]: Dirichlet data f -> 1/2 f |A_v| + K^T f (rhs_layer_3d.py:122-160).

        K^T f equals the reference's unpacked contraction
        ``(K[fy, fx, a, b] * f[faces[fy, a]]).sum(fy, a)`` scattered to faces[fx, b], taken on
        the packed K.  ``K_tight`` defaults to the parent's packed double layer.
        """
        batch = vert_bc_Dirichlet.shape[0]
        vert_areas = compute_vert_areas(vertices=verts, faces=faces, keepdim=True)  # [V, 1]
        if K_tight is None:
            K_tight = self.parent.double_layer.get_Kmat_tight(verts=verts, faces=faces)
        out = []
        for b in range(batch):
            is_d = vert_bc_flags[b] == int(BoundaryType.DIRICHLET)
            is_n = vert_bc_flags[b] == int(BoundaryType.NEUMANN)
            if int(is_n.sum()) > 0:
                raise NotImplementedError(
                    "Neumann / mixed boundary data need the hypersingular operator, which the "
                    "reference does not implement (integrations_3d.py:440-442)")
            if int(is_d.sum()) == 0:
                raise ValueError("no boundary data")
            f = vert_bc_Dirichlet[b].to(K_tight.dtype)  # [V, 1]
            gk1 = 0.5 * vert_bc_Dirichlet[b] * vert_areas
            gk2 = K_tight.transpose(0, 1) @ f
            gk = gk1 + gk2
            if self.BEM_type == int(BEMType.HELMHOLTZ_MOM):
                gk = gk1 * 2
            out.append(gk)
        self.rhs_vec = torch.stack(out, dim=0)
        self.initialized = True

    def get_rhs_vec(self):
        return self.rhs_vec
