"""Enums, quadrature tables and mesh helpers of the BEM hot path.

Mirrors the subset of the reference's ``src/utils`` that ``MeshBEMSolver3d`` uses:

* enums ``BoundaryType``, ``LayerType``, ``BEMType``, ``OrderType``, ``PanelRelationType``
  (``src/utils/types.py:81-154``) with the same values;
* ``get_gaussion_integration_points_and_weights`` (``src/utils/BEM_utils.py:360-588``);
* mesh geometry ``compute_face_areas/normals``, ``compute_vert_areas/normals``
  (``src/utils/mesh_utils.py:158-310``), ``get_edge_unique`` (``:921-977``),
  ``compute_panel_relation`` (``:700-725``);
* ``shape_function``, ``pack_matrix_tight`` (``BEM_utils.py:175-207``, ``:314-357``);
* ``get_rands_and_jacobian_3d`` (``src/mesh_BEM/utils/integrations_3d.py:18-249``) and its
  flattening into the rule table the panel kernel walks;
* ``Logger`` with the reference's ``InfoLog``/``WarnLog``/``ErrorLog`` surface
  (``src/utils/logger.py:7-98``).

Geometry helpers are plain tensor arithmetic (negligible work, any device); the
O(F^2) helpers (panel relations, tight packing) run as CUDA kernels and require CUDA
tensors.
"""
from __future__ import annotations

import ctypes
import math
import sys
from enum import Enum
from typing import List, Tuple

import numpy as np
import torch
import torch.nn.functional as F

from . import _lib

c0 = 1.0 / math.sqrt(8.8541878128e-12 * 1.25663706212e-6)  # speed of light (global_variables.py)


# ---------------------------------------------------------------------------------------
# enums (src/utils/types.py)
# ---------------------------------------------------------------------------------------
class _IntEnum(Enum):
    def __int__(self):
        return self.value


class BoundaryType(_IntEnum):
    DIRICHLET = 0
    NEUMANN = 1


class LayerType(_IntEnum):
    RHS = 0
    SINGLE_LAYER = 1
    DOUBLE_LAYER = 2
    HYPERSINGULAR_LAYER = 3


class BEMType(_IntEnum):
    LAPLACE = 0
    HELMHOLTZ_BEM = 1
    HELMHOLTZ_MOM = 2

    @staticmethod
    def use_complex(BEM_type: int) -> bool:
        return BEM_type in (int(BEMType.HELMHOLTZ_BEM), int(BEMType.HELMHOLTZ_MOM))

    @staticmethod
    def belong_Helmholtz(BEM_type: int) -> bool:
        return BEM_type in (int(BEMType.HELMHOLTZ_BEM), int(BEMType.HELMHOLTZ_MOM))


class OrderType(_IntEnum):
    PLANAR = 0
    LINEAR = 1


class VertexType(_IntEnum):
    AIR = 0
    FLUID = 1
    OBSTACLE = 2
    AIR_FLUID = 3
    FLUID_OBSTACLE = 4
    OBSTACLE_AIR = 5
    TRIPLE_JUNCTION = 6


class PanelRelationType(_IntEnum):
    SEPARATE = 0
    SAME_VERTEX = 1
    SAME_EDGE = 2
    SAME_FACE = 3


# ---------------------------------------------------------------------------------------
# logger (src/utils/logger.py:7-98): same method names; ErrorLog raises like the reference
# ---------------------------------------------------------------------------------------
class Logger:
    def __init__(self, root_path: str = "", log_to_disk: bool = False, verbose: bool = True):
        self.verbose = verbose
        self._fh = open(root_path + "log.txt", "a") if log_to_disk else None

    def _emit(self, tag: str, msg: str):
        line = f"[{tag}] {msg}"
        if self.verbose:
            print(line, file=sys.stdout)
        if self._fh is not None:
            self._fh.write(line + "\n")
            self._fh.flush()

    def InfoLog(self, *args, **kwargs):
        self._emit("Info", " ".join(str(a) for a in args))

    def WarnLog(self, *args, **kwargs):
        self._emit("Warn", " ".join(str(a) for a in args))

    def ErrorLog(self, *args, **kwargs):
        msg = " ".join(str(a) for a in args)
        self._emit("Error", msg)
        raise RuntimeError(msg)


# ---------------------------------------------------------------------------------------
# Gauss-Legendre tables (BEM_utils.py:360-588)
# ---------------------------------------------------------------------------------------
_SUPPORTED_GL = (1, 2, 3, 4, 5, 6, 7, 8, 12)


def get_gaussion_integration_points_and_weights(
    N: int, device: torch.device = torch.device("cpu"), dtype: torch.dtype = torch.float32
) -> List[torch.Tensor]:
    """N-point Gauss-Legendre nodes mapped to [0, 1] and weights summing to 1.

    Like the reference, the tables pass through torch's default dtype before conversion to
    ``dtype`` (its literal tables are built with ``torch.Tensor``, so with the usual float32
    default the nodes are float32-rounded even for a float64 solver), and the map to
    [0, 1] is done in ``dtype``.  Orders outside {1..8, 12} raise NotImplementedError.
    """
    if N not in _SUPPORTED_GL:
        raise NotImplementedError("Please refer N as 2~8 for gaussion interation")
    x, w = np.polynomial.legendre.leggauss(N)
    base = torch.get_default_dtype()
    p = torch.tensor(x, dtype=base).to(dtype).to(device)
    wt = torch.tensor(w, dtype=base).to(dtype).to(device)
    return [(p + 1.0) / 2.0, wt / 2.0]


def collapsed_rule_2d(points_1d: torch.Tensor, weights_1d: torch.Tensor):
    """(r1, r2) and weights of the collapsed 2-D rule, index b*n + a -> r1 = p_a, r2 = p_b p_a.

    Same layout as ``AbstractSingleLayer.__init__`` (single_layer/abstract_single_layer.py:49-63).
    """
    n = points_1d.numel()
    r1 = points_1d[None, :].repeat(n, 1)
    r2 = points_1d[:, None] * points_1d[None, :]
    w = weights_1d * weights_1d[:, None]
    return torch.stack((r1.reshape(-1), r2.reshape(-1)), dim=-1), w.reshape(-1, 1)


# ---------------------------------------------------------------------------------------
# mesh geometry (mesh_utils.py:158-310)
# ---------------------------------------------------------------------------------------
def _face_edge_vectors(vertices: torch.Tensor, faces: torch.Tensor):
    f = faces.long()
    v0, v1, v2 = vertices[..., f[:, 0], :], vertices[..., f[:, 1], :], vertices[..., f[:, 2], :]
    return v1 - v0, v2 - v1


def compute_face_areas(vertices: torch.Tensor, faces: torch.Tensor, keepdim: bool = True):
    e0, e1 = _face_edge_vectors(vertices, faces)
    return 0.5 * torch.cross(e0, e1, dim=-1).norm(dim=-1, keepdim=keepdim)


def compute_face_normals(vertices: torch.Tensor, faces: torch.Tensor):
    e0, e1 = _face_edge_vectors(vertices, faces)
    return F.normalize(torch.cross(e0, e1, dim=-1), dim=-1)


def compute_vert_areas(vertices: torch.Tensor, faces: torch.Tensor, keepdim: bool = True):
    areas = compute_face_areas(vertices, faces, keepdim=True)  # [F, 1]
    out = torch.zeros_like(vertices[..., 0:1])
    idx = faces.reshape(-1, 1).long()
    out.scatter_add_(-2, idx, (areas / 3).repeat_interleave(3, dim=-2))
    return out if keepdim else out.squeeze(-1)


def compute_vert_normals(vertices: torch.Tensor, faces: torch.Tensor):
    areas = compute_face_areas(vertices, faces, keepdim=True)
    normals = compute_face_normals(vertices, faces)
    out = torch.zeros_like(vertices)
    idx = faces.reshape(-1, 1).long().repeat(1, 3)
    out.scatter_add_(-2, idx, (areas * normals).repeat_interleave(3, dim=-2))
    return F.normalize(out, dim=-1)


def cot_laplacian(vertices: torch.Tensor, faces: torch.Tensor, eps: float = 1e-12):
    """Cotangent weights and inverse vertex areas of a triangle mesh.

    Returns (L, inv_areas): L is a sparse symmetric [V, V] matrix whose (i, j) entry is
    cot(alpha_ij) + cot(beta_ij), the cotangents of the angles opposite edge (i, j) in its
    two faces (U. Pinkall and K. Polthier, Experiment. Math. 2(1), 1993; M. Meyer et al.,
    Visualization and Mathematics III, 2003); inv_areas [V, 1] is 1 / (sum of the areas of
    the faces around each vertex), 0 for isolated vertices.  Same convention as the
    ``cot_laplacian`` the reference's pressure solver imports (mesh_pressure.py:112-115).
    """
    f = faces.long()
    p = [vertices[f[:, k]] for k in range(3)]
    rows, cols, vals = [], [], []
    for k in range(3):
        i, j = (k + 1) % 3, (k + 2) % 3  # edge (i, j) opposite corner k
        a, b = p[i] - p[k], p[j] - p[k]
        cr = torch.cross(a, b, dim=-1).norm(dim=-1).clamp_min(eps)
        cot = (a * b).sum(-1) / cr
        rows += [f[:, i], f[:, j]]
        cols += [f[:, j], f[:, i]]
        vals += [cot, cot]
    n = vertices.shape[0]
    L = torch.sparse_coo_tensor(torch.stack((torch.cat(rows), torch.cat(cols))), torch.cat(vals), (n, n),
                                check_invariants=False)
    L = L.coalesce()
    area = compute_face_areas(vertices, faces, keepdim=False)
    tot = torch.zeros(n, dtype=vertices.dtype, device=vertices.device)
    tot.index_add_(0, f.reshape(-1), area.repeat_interleave(3))
    inv = torch.where(tot > 0, 1.0 / tot.clamp_min(1e-300), torch.zeros_like(tot))
    return L, inv.reshape(n, 1)


def compute_mesh_face_tangent_gradient(vert_p: torch.Tensor, verts: torch.Tensor, faces: torch.Tensor,
                                       face_normals: torch.Tensor = None) -> torch.Tensor:
    """Surface gradient of the P1 interpolant of vert_p [B, V, 1] on each face -> [B, F, 3].

    grad p = sum_a p_a n x (P_{a+2} - P_{a+1}) / (2 A) (src/utils/mesh_utils.py:501-548).
    """
    if face_normals is None:
        face_normals = compute_face_normals(verts, faces)
    f = faces.long()
    area = compute_face_areas(verts, faces, keepdim=True)  # [F, 1]
    P = [verts[f[:, k]] for k in range(3)]
    g = 0
    for a in range(3):
        edge = P[(a + 2) % 3] - P[(a + 1) % 3]
        g = g + vert_p[:, f[:, a], :] * torch.cross(face_normals, edge, dim=-1)
    return g / 2.0 / area


def compute_mesh_vert_tangent_gradient(vert_p: torch.Tensor, verts: torch.Tensor, faces: torch.Tensor,
                                       face_normals: torch.Tensor = None) -> torch.Tensor:
    """Face gradients spread to vertices with weight 1/3 each -> [B, V, 3] (mesh_utils.py:574-615)."""
    fg = compute_mesh_face_tangent_gradient(vert_p, verts, faces, face_normals)  # [B, F, 3]
    out = torch.zeros((vert_p.shape[0], verts.shape[0], 3), dtype=fg.dtype, device=fg.device)
    idx = faces.long().reshape(-1)
    out.index_add_(1, idx, (fg / 3.0).repeat_interleave(3, dim=1))
    return out


def get_vertices_from_index(vertices: torch.Tensor, index: torch.Tensor):
    return torch.index_select(vertices, -2, index.long())


def get_edge_unique(verts: torch.Tensor, faces: torch.Tensor):
    """Unique undirected edges, the face-edge -> edge map and the two faces of each edge.

    Local edge e of face f joins faces[f, (e+1)%3] and faces[f, (e+2)%3] (the RWG edge
    opposite vertex e), as in ``get_edge_unique`` (mesh_utils.py:921-977).  Edges are
    numbered in increasing order of the key max*V + min, so the numbering is identical on
    every device (the reference's ``torch.unique(sorted=False)`` order is device-dependent).
    Returns (edges [E, 2] = (max, min), face_edge_indices [3F] in faces.dtype,
    edge_adjacent_faces [E, 2]).
    """
    n_verts = verts.shape[-2]
    n_faces = faces.shape[0]
    fe = torch.stack((faces[:, 1], faces[:, 2], faces[:, 2], faces[:, 0], faces[:, 0], faces[:, 1]),
                     dim=-1).reshape(n_faces * 3, 2).long()
    key = fe.max(dim=-1)[0] * n_verts + fe.min(dim=-1)[0]
    uniq, inv = torch.unique(key, sorted=True, return_inverse=True)
    edges = torch.stack((uniq // n_verts, uniq % n_verts), dim=-1).to(faces.dtype)
    face_idx = torch.arange(n_faces, device=faces.device, dtype=torch.long).repeat_interleave(3)
    n_edges = uniq.numel()
    adj = torch.zeros((n_edges, 2), dtype=torch.long, device=faces.device)
    adj[:, 0].scatter_add_(0, inv, face_idx)
    adj[:, 1].scatter_(0, inv, face_idx)
    adj[:, 0] = adj[:, 0] - adj[:, 1]
    return edges, inv.to(faces.dtype), adj.to(faces.dtype)


def shared_vertex_pairs(faces: torch.Tensor, n_verts: int | None = None) -> torch.Tensor:
    """All ordered face pairs sharing at least one vertex (each face with itself included),
    [n, 2] int32 sorted by first face, then second: the nonzeros of
    ``compute_panel_relation`` (mesh_utils.py:700-725) in row-major order, built in O(F) memory
    instead of from the dense [F, F] relation.  CUDA faces: ``mb_shared_vertex_pairs_*``
    (vertex-face incidences, per-face merge of the three sorted vertex lists; one host
    synchronisation for the length; ``n_verts`` defaults to max id + 1).  Host faces (the
    CPU baseline and host tests): the same list from torch -- every ordered pair of faces
    around each vertex, one sorted unique of the pair keys."""
    faces = faces.reshape(-1, 3)
    nf = faces.shape[0]
    dev = faces.device
    if nf == 0:
        return torch.zeros((0, 2), dtype=torch.int32, device=dev)
    if faces.is_cuda:
        faces = faces.to(torch.int32).contiguous()
        nv = int(faces.max()) + 1 if n_verts is None else int(n_verts)
        lib = _lib.load()
        ws = torch.empty(int(lib.mb_shared_vertex_pairs_workspace_bytes(nf, nv)), dtype=torch.uint8, device=dev)
        n = ctypes.c_int64(0)
        _lib.call("mb_shared_vertex_pairs_count", _lib.ptr(faces), nf, nv, _lib.ptr(ws), ws.numel(),
                  ctypes.byref(n), _lib.stream_of(faces))
        pairs = torch.empty((int(n.value), 2), dtype=torch.int32, device=dev)
        _lib.call("mb_shared_vertex_pairs_fill", _lib.ptr(faces), nf, nv, _lib.ptr(ws), _lib.ptr(pairs),
                  _lib.stream_of(faces))
        return pairs
    v = faces.reshape(-1).long()
    f = torch.arange(nf, device=dev, dtype=torch.long).repeat_interleave(3)
    order = torch.argsort(v, stable=True)
    vs, fs = v[order], f[order]
    _, counts = torch.unique_consecutive(vs, return_counts=True)
    starts = torch.cumsum(counts, 0) - counts
    c2 = counts * counts
    pstart = torch.cumsum(c2, 0) - c2
    gid = torch.repeat_interleave(torch.arange(counts.numel(), device=dev), c2)
    local = torch.arange(int(c2.sum()), device=dev) - pstart[gid]
    cg = counts[gid]
    fa = fs[starts[gid] + local // cg]
    fb = fs[starts[gid] + local % cg]
    key = torch.unique(fa * nf + fb)
    return torch.stack((key // nf, key % nf), dim=-1).to(torch.int32).contiguous()


def compute_panel_relation(faces: torch.Tensor) -> torch.Tensor:
    """[F, F] uint8 shared-vertex relation (0 separate .. 3 same face), CUDA kernel."""
    faces = _lib.check_tensor(faces.contiguous(), "faces", dtype=torch.int32, ndim=2)
    nf = faces.shape[0]
    rel = torch.empty((nf, nf), dtype=torch.uint8, device=faces.device)
    _lib.call("mb_panel_relation", _lib.ptr(faces), nf, _lib.ptr(rel), _lib.stream_of(faces))
    return rel


# ---------------------------------------------------------------------------------------
# shape functions / packing (BEM_utils.py:175-207, :314-357)
# ---------------------------------------------------------------------------------------
def shape_function(dim: int, order_type: int, r1: torch.Tensor, r2: torch.Tensor = None):
    if dim == 3:
        if order_type == int(OrderType.PLANAR):
            return (torch.ones_like(r1),)
        return 1 - r1, r1 - r2, r2
    if dim == 2:
        if order_type == int(OrderType.PLANAR):
            return (torch.ones_like(r1),)
        return 1 - r1, r1
    raise RuntimeError("We only accept 2D/3D for calculating shape function")


def pack_matrix_tight(order_type: int, unpacked_matrix: torch.Tensor, verts: torch.Tensor,
                      faces: torch.Tensor) -> torch.Tensor:
    """[F, F, nphi, nphi] -> [V, V]: packed[faces[fy,a], faces[fx,b]] += M[fy, fx, a, b]."""
    n_verts = verts.shape[-2]
    faces = _lib.check_tensor(faces.contiguous(), "faces", dtype=torch.int32, ndim=2)
    nf = faces.shape[0]
    if nf and (int(faces.min()) < 0 or int(faces.max()) >= n_verts):
        raise ValueError(f"faces reference vertex ids outside [0, {n_verts})")
    m = unpacked_matrix.contiguous()
    if m.shape[:2] != (nf, nf) or m.shape[2] != m.shape[3] or m.shape[2] not in (1, 3):
        raise ValueError("unpacked_matrix must be [F, F, nphi, nphi] with nphi 1 or 3")
    if (m.shape[2] == 3) != (int(order_type) == int(OrderType.LINEAR)):
        raise ValueError("unpacked_matrix shape does not match order_type")
    _lib.check_tensor(m, "unpacked_matrix", device=faces.device)
    if m.is_complex():
        base = m.real.dtype
        mr, mi = m.real.contiguous(), m.imag.contiguous()
        out = torch.zeros((n_verts, n_verts, 2), dtype=base, device=m.device)
    else:
        base = m.dtype
        mr, mi = m, None
        out = torch.zeros((n_verts, n_verts), dtype=base, device=m.device)
    _lib.call(f"mb_pack_tight_{_lib.sfx(base)}", _lib.ptr(mr), _lib.ptr(mi), _lib.ptr(faces), nf,
              n_verts, int(order_type), _lib.ptr(out), _lib.stream_of(m))
    return torch.view_as_complex(out) if mi is not None else out


# ---------------------------------------------------------------------------------------
# Sauter-Schwab style sub-domain maps (integrations_3d.py:18-249)
# ---------------------------------------------------------------------------------------
def get_rands_and_jacobian_3d(xsi, eta1, eta2, eta3):
    """Per relation r: (r1_x, r2_x, r1_y, r2_y, jacobian), each [Ng, ND_r]; ND = 1, 2, 5, 3."""
    xsi, eta1, eta2, eta3 = (t.reshape(-1, 1) for t in (xsi, eta1, eta2, eta3))
    r1x, r2x, r1y, r2y, jac = [None] * 4, [None] * 4, [None] * 4, [None] * 4, [None] * 4
    # separate
    r1x[0], r2x[0], r1y[0], r2y[0] = xsi, eta1 * xsi, eta2, eta2 * eta3
    jac[0] = xsi * eta2
    # shared vertex: two sub-domains
    d1 = torch.cat((xsi, xsi * eta1, xsi * eta2, xsi * eta2 * eta3), -1)
    d2 = torch.cat((xsi * eta2, xsi * eta2 * eta3, xsi, xsi * eta1), -1)
    sv = torch.stack((d1, d2), -2)
    jv = xsi * xsi * xsi * eta2
    r1x[1], r2x[1], r1y[1], r2y[1] = sv[..., 0], sv[..., 1], sv[..., 2], sv[..., 3]
    jac[1] = torch.cat((jv, jv), -1)
    # shared edge: five sub-domains, each w -> (w0, w3, w0 + w1, w2)
    ws = [
        (xsi, -xsi * eta1 * eta2, xsi * eta1 * (1.0 - eta2), xsi * eta1 * eta3),
        (xsi, -xsi * eta1 * eta2 * eta3, xsi * eta1 * eta2 * (1.0 - eta3), xsi * eta1),
        (xsi * (1.0 - eta1 * eta2), xsi * eta1 * eta2, xsi * eta1 * eta2 * eta3,
         xsi * eta1 * (1.0 - eta2)),
        (xsi * (1.0 - eta1 * eta2 * eta3), xsi * eta1 * eta2 * eta3, xsi * eta1,
         xsi * eta1 * eta2 * (1.0 - eta3)),
        (xsi * (1.0 - eta1 * eta2 * eta3), xsi * eta1 * eta2 * eta3, xsi * eta1 * eta2,
         xsi * eta1 * (1.0 - eta2 * eta3)),
    ]
    se = torch.stack([torch.cat((w[0], w[3], w[0] + w[1], w[2]), -1) for w in ws], -2)
    je0 = xsi * xsi * xsi * eta1 * eta1
    je1 = xsi * xsi * xsi * eta1 * eta1 * eta2
    r1x[2], r2x[2], r1y[2], r2y[2] = se[..., 0], se[..., 1], se[..., 2], se[..., 3]
    jac[2] = torch.cat((je0, je1, je1, je1, je1), -1)
    # same face: three sub-domains from linear maps of w = (xsi, xsi e1, xsi e1 e2, xsi e1 e2 e3)
    w0, w1, w2, w3 = xsi, xsi * eta1, xsi * eta1 * eta2, xsi * eta1 * eta2 * eta3
    xz = [
        (w0, w0 - w1 + w2, w3, w2),
        (w0, w1 - w2 + w3, w2, w3),
        (w0 - w3, w1 - w3, -w3, w2 - w3),
    ]
    sf = torch.stack([torch.cat((z[0], z[1], z[0] - z[2], z[1] - z[3]), -1) for z in xz], -2)
    jf = xsi * xsi * xsi * eta1 * eta1 * eta2
    r1x[3], r2x[3], r1y[3], r2y[3] = sf[..., 0], sf[..., 1], sf[..., 2], sf[..., 3]
    jac[3] = torch.cat((jf, jf, jf), -1)
    return r1x, r2x, r1y, r2y, jac


def panel_rule_table(rands_x: torch.Tensor, rands_y: torch.Tensor, weights_x: torch.Tensor,
                     weights_y: torch.Tensor) -> Tuple[torch.Tensor, List[int]]:
    """Flatten the 4-D rules of double_integration_on_panels_3d (integrations_3d.py:349-372).

    The 4-D point g = s*Q + t (Q = rule size) has xsi = r1[t], eta1 = r2[t], eta2 = r1[s],
    eta3 = r2[s] and weight wy[s] wx[t].  Returns a [rows, 5] table of
    (r1x, r2x, r1y, r2y, weight * jacobian) grouped by relation, and the 5 segment offsets.
    Computed in the dtype of the inputs, like the reference.
    """
    q = weights_x.numel()
    ng = q * q
    xsi = rands_x[..., 0:1].reshape(1, q).repeat(q, 1).reshape(ng, 1)
    eta1 = rands_x[..., 1:2].reshape(1, q).repeat(q, 1).reshape(ng, 1)
    eta2 = rands_y[..., 0:1].reshape(q, 1).repeat(1, q).reshape(ng, 1)
    eta3 = rands_y[..., 1:2].reshape(q, 1).repeat(1, q).reshape(ng, 1)
    wx = weights_x.reshape(1, q).repeat(q, 1).reshape(ng, 1)
    wy = weights_y.reshape(q, 1).repeat(1, q).reshape(ng, 1)
    wyx = (wy * wx).reshape(ng, 1)
    r1x, r2x, r1y, r2y, jac = get_rands_and_jacobian_3d(xsi, eta1, eta2, eta3)
    rows, seg = [], [0]
    for r in range(4):
        t = torch.stack((r1x[r], r2x[r], r1y[r], r2y[r], wyx * jac[r]), -1)  # [ng, nd, 5]
        rows.append(t.reshape(-1, 5))
        seg.append(seg[-1] + t.shape[0] * t.shape[1])
    return torch.cat(rows, 0).contiguous(), seg
