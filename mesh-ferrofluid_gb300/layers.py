"""Galerkin layer operators of the 3D Laplace / Helmholtz BEM path.

Mirrors the reference's layer classes and the integration routine they share:

* ``double_integration_on_panels_3d`` (src/mesh_BEM/utils/integrations_3d.py:252-452) --
  same signature and result ([F_y, F_x, nphi, nphi]); the O(F^2 * rule) work runs in the
  sm_103a panel kernel (``mb_laplace_panels_*``).  ``layer_type`` HYPERSINGULAR, which
  the reference leaves unimplemented (:440-442), returns the P1 hypersingular operator by
  Maue's formula from the P0 single layer of the same rule (``mb_laplace_hypersingular_*``);
* ``SingleLayer3d`` / ``DoubleLayer3d`` / ``HyperSingularLayer3d`` (single_layer_3d.py:43-68,
  double_layer_3d.py:43-68, hypersingular_layer_3d.py, abstract layers :17-98) with
  ``compute_*mat``, ``get_*mat_unpacked`` and ``get_*mat_tight``;
* ``RhsLayer3d.compute_rhs`` (rhs_layer/rhs_layer_3d.py:74-203) for Dirichlet, Neumann and
  mixed data.

Every layer takes ``rule``: ``"reference"`` (the reference's collapsed Gauss rule, results
equal to the reference's) or ``"dunavant7"`` (7-point rule, singular and near-singular
pairs in closed form, ``mb_laplace_sym_*``), which is accurate enough for the Neumann and
mixed problems (the reference rule's P0 single layer makes the hypersingular operator
indefinite on coarse meshes).
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
    compute_panel_relation,
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
        if BEMType.belong_Helmholtz(BEM_type):
            raise NotImplementedError("hypersingular operator: Laplace only")
        if int(order_type) != int(OrderType.LINEAR):
            raise ValueError("the hypersingular operator needs P1 (OrderType.LINEAR) functions")
        v0 = double_integration_on_panels_3d(BEM_type, int(OrderType.PLANAR), verts, faces, face_areas,
                                             face_normals, gauss_weightsx, gauss_weightsy, rands_x, rands_y,
                                             panel_relations, wavenumber, int(LayerType.SINGLE_LAYER))
        return hypersingular_from_v0(verts, faces.to(torch.int32).contiguous(), v0)
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
    table, seg = _cached_rule_table(rands_x, rands_y, gauss_weightsx, gauss_weightsy, dt, dev)
    seg_c = (torch.tensor(seg, dtype=torch.int32)).numpy()
    if panel_relations is None:  # the tiled kernels take the relation matrix (F^2 bytes)
        rel = compute_panel_relation(faces)
    else:
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


# Flattened sub-domain rule tables of recent calls.  Building a table takes ~150 small torch
# operations and a solver passes the same rule tensors on every call, so an entry is found
# first by the identity and version counter of the four rule tensors (the entry holds them,
# so their storage cannot be reused while it lives) -- no device synchronisation -- and
# otherwise by their values (a few dozen numbers, one small copy to the host).
_RULE_TABLES: list = []
_RULE_TABLES_MAX = 8


def _cached_rule_table(rx, ry, wx, wy, dt, dev):
    ins = (rx, ry, wx, wy)
    vers = tuple(t._version for t in ins)
    for held, held_vers, key, val in _RULE_TABLES:
        if (key[2], key[3]) == (dt, str(dev)) and held_vers == vers and all(a is b for a, b in zip(held, ins)):
            return val
    vals = torch.cat([t.reshape(-1).to(torch.float64) for t in ins]).cpu().tolist()
    key = (tuple(tuple(t.shape) for t in ins), tuple(vals), dt, str(dev))
    val = None
    for _, _, k, v in _RULE_TABLES:
        if k == key:
            val = v
            break
    if val is None:
        table, seg = panel_rule_table(rx.to(dt), ry.to(dt), wx.to(dt), wy.to(dt))
        val = (table.to(dev).contiguous(), seg)
    _RULE_TABLES.append((ins, vers, key, val))
    del _RULE_TABLES[:-_RULE_TABLES_MAX]
    return val


def hypersingular_from_v0(verts: torch.Tensor, faces: torch.Tensor, v0: torch.Tensor) -> torch.Tensor:
    """P1 hypersingular panels [F, F, 3, 3] from P0 single-layer panels v0 [F, F(, 1, 1)]."""
    _lib.check_tensor(verts, "verts", dtype=(torch.float32, torch.float64), ndim=2)
    nf = faces.shape[0]
    v0 = v0.reshape(nf, nf).to(verts.dtype).contiguous()
    _lib.check_tensor(faces, "faces", dtype=torch.int32, device=verts.device, ndim=2)
    out = torch.empty((nf, nf, 3, 3), dtype=verts.dtype, device=verts.device)
    _lib.call(f"mb_laplace_hypersingular_{_lib.sfx(verts.dtype)}", _lib.ptr(verts), verts.shape[0],
              _lib.ptr(faces), nf, _lib.ptr(v0), _lib.ptr(out), _lib.stream_of(verts))
    return out


# shared memory the row packing may use (3 x V values): mb_pack_tight_* and
# mb_laplace_hypersingular_tight_* take the row-accumulating path up to this size
PACK_ROWS_SMEM_MAX = 160 * 1024


def hypersingular_tight(verts: torch.Tensor, faces: torch.Tensor, v0: torch.Tensor) -> torch.Tensor:
    """Packed P1 hypersingular matrix [V, V] from P0 single-layer panels v0 [F, F(, 1, 1)]
    (``mb_laplace_hypersingular_tight_*``; equal to packing ``hypersingular_from_v0``).
    Meshes whose 3 V row values exceed the shared-memory budget take that two-step path."""
    _lib.check_tensor(verts, "verts", dtype=(torch.float32, torch.float64), ndim=2)
    faces = faces.to(torch.int32).contiguous()
    _lib.check_tensor(faces, "faces", device=verts.device, ndim=2)
    nf, nv = faces.shape[0], verts.shape[0]
    if 3 * nv * verts.element_size() > PACK_ROWS_SMEM_MAX:
        from .utils import pack_matrix_tight

        return pack_matrix_tight(int(OrderType.LINEAR), hypersingular_from_v0(verts, faces, v0), verts, faces)
    check_face_range(faces, nv)
    v0 = v0.reshape(nf, nf).to(verts.dtype).contiguous()
    out = torch.zeros((nv, nv), dtype=verts.dtype, device=verts.device)
    _lib.call(f"mb_laplace_hypersingular_tight_{_lib.sfx(verts.dtype)}", _lib.ptr(verts), nv, _lib.ptr(faces), nf,
              _lib.ptr(v0), _lib.ptr(out), _lib.stream_of(verts))
    return out


def laplace_sym_tight(verts: torch.Tensor, faces: torch.Tensor, op: int, near: torch.Tensor | None = None,
                      rows=None, out: torch.Tensor | None = None, check_indices: bool = True) -> torch.Tensor:
    """Packed symmetric-rule operator [V, V] (``mb_laplace_sym_tight_*``) without the
    [F, F, 3, 3] panels: op 1 single layer, 2 double layer (both P1, equal to packing
    ``laplace_sym_panels``), 3 hypersingular (equal to ``hypersingular_tight`` of the P0
    single layer).  Accumulates into ``out`` when given.  Meshes whose 3 V row values
    exceed the shared-memory budget take the panels-then-pack path.  ``check_indices=False``
    skips the vertex-id range check (one reduction and a host synchronisation) for faces
    already validated, e.g. by ``shared_vertex_pairs``."""
    _lib.check_tensor(verts, "verts", dtype=(torch.float32, torch.float64), ndim=2)
    faces = faces.to(torch.int32).contiguous()
    _lib.check_tensor(faces, "faces", device=verts.device, ndim=2)
    if int(op) not in (1, 2, 3):
        raise ValueError("op must be 1 (single layer), 2 (double layer) or 3 (hypersingular)")
    nf, nv = faces.shape[0], verts.shape[0]
    if check_indices:
        check_face_range(faces, nv)
    if near is None:
        near = laplace_near_pairs(faces, verts.shape[0])
    _lib.check_tensor(near, "near", dtype=torch.int32, device=verts.device)
    if out is None:
        out = torch.zeros((nv, nv), dtype=verts.dtype, device=verts.device)
    else:
        _lib.check_tensor(out, "out", dtype=verts.dtype, device=verts.device, shape=(nv, nv))
    r0, r1 = (0, nf) if rows is None else rows
    if 3 * nv * verts.element_size() > PACK_ROWS_SMEM_MAX:
        from .utils import pack_matrix_tight

        if int(op) == 3:
            v0 = laplace_sym_panels(verts, faces, 1, int(OrderType.PLANAR), near)
            part = hypersingular_from_v0(verts, faces, v0)
        else:
            part = laplace_sym_panels(verts, faces, int(op), int(OrderType.LINEAR), near)
        if rows is not None:
            part[:r0].zero_()
            part[r1:].zero_()
        out += pack_matrix_tight(int(OrderType.LINEAR), part, verts, faces)
        return out
    _lib.call(f"mb_laplace_sym_tight_{_lib.sfx(verts.dtype)}", _lib.ptr(verts), nv, _lib.ptr(faces), nf, int(op),
              _lib.ptr(near), near.shape[0], r0, r1, _lib.ptr(out), _lib.stream_of(verts))
    return out


def laplace_near_pairs(faces: torch.Tensor, n_verts: int | None = None) -> torch.Tensor:
    """Ordered face pairs sharing a vertex (incl. self), [n, 2] int32, sorted by first face."""
    from .utils import shared_vertex_pairs

    return shared_vertex_pairs(faces, n_verts)


def laplace_sym_panels(verts: torch.Tensor, faces: torch.Tensor, layer: int, order: int,
                       near: torch.Tensor | None = None, rows=None, out=None) -> torch.Tensor:
    """Symmetric-rule Galerkin panels [F_y, F_x, nphi, nphi] (``mb_laplace_sym_*``).

    layer 1: single layer 1/(4 pi R); 2: double layer n_y.(x - y)/(4 pi R^3) with the
    normal of the first ("y") face, as ``double_integration_on_panels_3d``.
    """
    _lib.check_tensor(verts, "verts", dtype=(torch.float32, torch.float64), ndim=2)
    faces = faces.to(torch.int32).contiguous()
    _lib.check_tensor(faces, "faces", device=verts.device, ndim=2)
    nf = faces.shape[0]
    check_face_range(faces, verts.shape[0])
    if near is None:
        near = laplace_near_pairs(faces, verts.shape[0])
    _lib.check_tensor(near, "near", dtype=torch.int32, device=verts.device)
    r0, r1 = (0, nf) if rows is None else rows
    nphi = 3 if int(order) == int(OrderType.LINEAR) else 1
    shape = (r1 - r0, nf, nphi, nphi)
    if out is None:
        out = torch.empty(shape, dtype=verts.dtype, device=verts.device)
    else:
        _lib.check_tensor(out, "out", dtype=verts.dtype, device=verts.device, shape=shape)
    _lib.call(f"mb_laplace_sym_{_lib.sfx(verts.dtype)}", _lib.ptr(verts), verts.shape[0], _lib.ptr(faces), nf,
              int(layer), 1 if nphi == 3 else 0, _lib.ptr(near), near.shape[0], r0, r1, _lib.ptr(out),
              _lib.stream_of(verts))
    return out


def laplace_colloc_sl(verts: torch.Tensor, faces: torch.Tensor, rows=None, out=None,
                      near: torch.Tensor | None = None, check_indices: bool = True) -> torch.Tensor:
    """Single-layer collocation matrix [F, F] at face centroids (``mb_laplace_colloc_sl_*``).

    ``near``: the pairs sharing a vertex (``laplace_near_pairs(faces)``), computed when None.
    """
    _lib.check_tensor(verts, "verts", dtype=(torch.float32, torch.float64), ndim=2)
    faces = faces.to(torch.int32).contiguous()
    _lib.check_tensor(faces, "faces", device=verts.device, ndim=2)
    nf = faces.shape[0]
    if check_indices:
        check_face_range(faces, verts.shape[0])
    if near is None:
        near = laplace_near_pairs(faces, verts.shape[0])
    _lib.check_tensor(near, "near", dtype=torch.int32, device=verts.device)
    r0, r1 = (0, nf) if rows is None else rows
    if out is None:
        out = torch.empty((r1 - r0, nf), dtype=verts.dtype, device=verts.device)
    else:
        _lib.check_tensor(out, "out", dtype=verts.dtype, device=verts.device, shape=(r1 - r0, nf))
    _lib.call(f"mb_laplace_colloc_sl_{_lib.sfx(verts.dtype)}", _lib.ptr(verts), verts.shape[0], _lib.ptr(faces),
              nf, _lib.ptr(near), near.shape[0], r0, r1, _lib.ptr(out), _lib.stream_of(verts))
    return out


def p1_mass_apply(verts: torch.Tensor, faces: torch.Tensor, g: torch.Tensor) -> torch.Tensor:
    """(M g) with the consistent P1 mass matrix M_ij = int phi_i phi_j; g [V, k] -> [V, k]."""
    from .utils import compute_face_areas

    f = faces.to(torch.int64)
    a = compute_face_areas(vertices=verts, faces=faces, keepdim=True).to(g.dtype)  # [F, 1]
    gv = g[f]  # [F, 3, k]
    s = gv.sum(1, keepdim=True)  # [F, 1, k]
    loc = (gv + s) * (a[:, :, None] / 12.0)  # A/12 (2 g_i + g_j + g_k)
    out = torch.zeros_like(g)
    out.index_add_(0, f.reshape(-1), loc.reshape(-1, g.shape[1]))
    return out


class _AbstractLayer:
    rank = 3
    layer_type = int(LayerType.SINGLE_LAYER)

    def __init__(self, gaussQR: int, order_type: int, BEM_type: int, wavenumber: float, logger,
                 dtype: torch.dtype = torch.float32, device: torch.device = torch.device("cpu"),
                 rule: str = "reference"):
        if rule not in ("reference", "dunavant7"):
            raise ValueError(f"unknown rule {rule!r} (reference or dunavant7)")
        self.rule = rule
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
        if self.rule == "dunavant7":
            if BEMType.belong_Helmholtz(self.BEM_type):
                raise NotImplementedError("rule dunavant7: Laplace kernels only")
            near = None
            if panel_relations is not None:
                near = torch.nonzero(panel_relations > 0).to(torch.int32).contiguous()
            self.compute_sym(verts, faces, near)
            return
        # one [n, 2] rule tensor per (r1, r2): the same object on every call finds the rule
        # table without a device synchronisation
        key = (self.r1, self.r2, self.r1._version, self.r2._version)
        held = getattr(self, "_rands_key", None)
        if held is None or held[0] is not key[0] or held[1] is not key[1] or held[2:] != key[2:]:
            self._rands_key, self._rands = key, torch.cat((self.r1, self.r2), dim=-1)
        rands = self._rands
        self._unpacked = double_integration_on_panels_3d(
            BEM_type=self.BEM_type, order_type=self.order_type, verts=verts, faces=faces,
            face_areas=face_areas, face_normals=face_normals, gauss_weightsx=self.gauss_weights,
            gauss_weightsy=self.gauss_weights, rands_x=rands, rands_y=rands,
            panel_relations=panel_relations, wavenumber=self.wavenumber, layer_type=self.layer_type)
        self.initialized = True

    def compute_sym(self, verts, faces, near=None):
        """Symmetric-rule panels from a near-pair list ([n, 2] int32 face pairs sharing a
        vertex, ``shared_vertex_pairs``; built here when None) instead of the dense relation."""
        if self.rule != "dunavant7" or BEMType.belong_Helmholtz(self.BEM_type):
            raise ValueError("compute_sym: Laplace layers with rule dunavant7 only")
        self._unpacked = self._sym(verts, faces, near)
        self.initialized = True

    def _tight(self, verts, faces):
        return pack_matrix_tight(self.order_type, self._unpacked, verts, faces)

    def InfoLog(self, *a, **k):
        return self.logger.InfoLog(*a, **k) if self.logger else None


class SingleLayer3d(_AbstractLayer):
    layer_type = int(LayerType.SINGLE_LAYER)

    def _sym(self, verts, faces, near):
        return laplace_sym_panels(verts, faces, 1, self.order_type, near)

    def compute_Vmat(self, verts, faces, face_areas, face_normals, panel_relations=None):
        self._compute(verts, faces, face_areas, face_normals, panel_relations)

    def get_Vmat_unpacked(self):
        return self._unpacked

    def get_Vmat_tight(self, verts, faces):
        return self._tight(verts, faces)


class DoubleLayer3d(_AbstractLayer):
    layer_type = int(LayerType.DOUBLE_LAYER)

    def _sym(self, verts, faces, near):
        return laplace_sym_panels(verts, faces, 2, self.order_type, near)

    def compute_Kmat(self, verts, faces, face_areas, face_normals, panel_relations=None):
        self._compute(verts, faces, face_areas, face_normals, panel_relations)

    def get_Kmat_unpacked(self):
        return self._unpacked

    def get_Kmat_tight(self, verts, faces):
        return self._tight(verts, faces)


class HyperSingularLayer3d(_AbstractLayer):
    """P1 hypersingular operator (the reference declares the class but never computes it)."""

    layer_type = int(LayerType.HYPERSINGULAR_LAYER)

    def _sym(self, verts, faces, near):
        if int(self.order_type) != int(OrderType.LINEAR):
            raise ValueError("the hypersingular operator needs P1 (OrderType.LINEAR) functions")
        v0 = laplace_sym_panels(verts, faces, 1, int(OrderType.PLANAR), near)
        return hypersingular_from_v0(verts, faces.to(torch.int32).contiguous(), v0)

    def compute_Dmat(self, verts, faces, face_areas, face_normals, panel_relations=None):
        self._compute(verts, faces, face_areas, face_normals, panel_relations)

    def get_Dmat_unpacked(self):
        return self._unpacked

    def get_Dmat_tight(self, verts, faces):
        return self._tight(verts, faces)


class RhsLayer3d:
    rank = 3

    def __init__(self, parent, gaussQR: int, order_type: int, BEM_type: int, wavenumber: float,
                 logger, dtype=torch.float32, device=torch.device("cpu"), rule: str = "reference"):
        self.parent = parent
        self.rule = rule
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

    def _mass(self, verts, faces, g):
        if self.rule == "dunavant7":
            return p1_mass_apply(verts, faces, g)
        return g * compute_vert_areas(vertices=verts, faces=faces, keepdim=True).to(g.dtype)

    def compute_rhs(self, verts, faces, vert_bc_Dirichlet, vert_bc_Neumann, vert_bc_flags,
                    K_tight=None, V_tight=None, D_tight=None):
        """rhs [B, V, 1] of the direct formulation (rhs_layer_3d.py:74-203).

        With g the Dirichlet data (zero off Gamma_D), f the Neumann data (zero off Gamma_N),
        M the mass matrix (lumped vertex areas for the reference rule, as the reference;
        the consistent P1 mass matrix for rule dunavant7) and K = K_tight^T the Galerkin
        double layer <phi_i, K phi_j>:
            Dirichlet rows:  1/2 M g + K g - V f
            Neumann rows:    1/2 M f - K^T f - D g
        (O. Steinbach, Numerical Approximation Methods for Elliptic Boundary Value Problems,
        2008, sec. 7.4).  Each vertex carries the row of its own boundary type.  The
        reference's Neumann rows use K f instead of K^T f and never run (its hypersingular
        layer is None).  The matrices default to the parent's layers.
        """
        batch = vert_bc_Dirichlet.shape[0]
        P = self.parent
        if K_tight is None:
            K_tight = P.double_layer.get_Kmat_tight(verts=verts, faces=faces)
        out = []
        for b in range(batch):
            is_d = (vert_bc_flags[b] == int(BoundaryType.DIRICHLET)).reshape(-1)
            is_n = (vert_bc_flags[b] == int(BoundaryType.NEUMANN)).reshape(-1)
            n_d, n_n = int(is_d.sum()), int(is_n.sum())
            if n_d + n_n == 0:
                raise ValueError("no boundary data")
            g = torch.where(is_d[:, None], vert_bc_Dirichlet[b].reshape(-1, 1), 0).to(K_tight.dtype)
            f = torch.where(is_n[:, None], vert_bc_Neumann[b].reshape(-1, 1), 0).to(K_tight.dtype)
            rhs = torch.zeros_like(g)
            if n_d:
                gk1 = 0.5 * self._mass(verts, faces, g)
                gk = gk1 + K_tight.transpose(0, 1) @ g
                if n_n:
                    Vt = V_tight if V_tight is not None else P.single_layer.get_Vmat_tight(verts=verts,
                                                                                            faces=faces)
                    gk = gk - Vt @ f
                if self.BEM_type == int(BEMType.HELMHOLTZ_MOM):
                    gk = gk1 * 2
                rhs = torch.where(is_d[:, None], gk, rhs)
            if n_n:
                fi1 = 0.5 * self._mass(verts, faces, f)
                fi = fi1 - K_tight @ f
                if n_d:
                    Dt = D_tight if D_tight is not None else P.hypersingular_layer.get_Dmat_tight(
                        verts=verts, faces=faces)
                    fi = fi - Dt @ g
                if self.BEM_type == int(BEMType.HELMHOLTZ_MOM):
                    fi = fi1 * 2
                rhs = torch.where(is_n[:, None], fi, rhs)
            out.append(rhs)
        self.rhs_vec = torch.stack(out, dim=0)
        self.initialized = True

    def get_rhs_vec(self):
        return self.rhs_vec
