"""Drop-in for the reference's JIT extension ``mesh_MOM_3d`` plus the RWG-space operators.

The reference builds ``mesh_MOM_3d`` with ``torch.utils.cpp_extension.load``
(``src/mesh_BEM/kernel_functions.py:14-23``) and exports three in-place forward ops
(``src/mesh_BEM/cuda/mesh_MOM_3d.cpp:111-121``).  This module exports the same three
functions with the same argument order, meaning and in-place outputs, backed by
libmeshbem_gb300 (sm_103a).  Differences from the reference, all in the safe direction:
inputs are checked (device, dtype, shape, contiguity) and errors raise ``MeshBEMError`` /
``ValueError`` instead of failing silently; launches go to the caller's current stream
instead of the legacy default stream; indexing is 64-bit.

``register_torch_ops()`` also exposes them as ``torch.ops.mesh_MOM_3d.*`` (the reference
registers ``TORCH_LIBRARY(mesh_MOM_3d, m)``).

The RWG-space operators fuse the reference's scatter steps:
``assemble_Z_rwg`` (face-edge matrix straight into the [E, E] RWG matrix),
``assemble_rhs_rwg`` (many plane waves at once into [E, n_rhs]),
``interpolate_vert_js`` (edge coefficients straight to [B, V, 3] vertex currents).
"""
from __future__ import annotations

import math

import torch

from . import _lib

_FLOATS = (torch.float32, torch.float64)


def _mesh_args(verts, faces, face_areas, face_normals):
    _lib.check_tensor(verts, "verts", dtype=_FLOATS, ndim=2)
    dt, dev = verts.dtype, verts.device
    if verts.shape[1] != 3:
        raise ValueError("verts must be [N_verts, 3]")
    _lib.check_tensor(faces, "faces", dtype=torch.int32, device=dev, ndim=2)
    if faces.shape[1] != 3:
        raise ValueError("faces must be [N_faces, 3]")
    nf = faces.shape[0]
    _lib.check_tensor(face_areas, "face_areas", dtype=dt, device=dev)
    if face_areas.numel() != nf:
        raise ValueError("face_areas must have N_faces entries")
    _lib.check_tensor(face_normals, "face_normals", dtype=dt, device=dev)
    if face_normals.numel() != 3 * nf:
        raise ValueError("face_normals must be [N_faces, 3]")
    check_face_range(faces, verts.shape[0])
    return dt, dev, verts.shape[0], nf


# face tensors already checked: (tensor, version counter, vertex count); an entry holds its
# tensor, so the identity cannot be taken by another tensor while the entry lives
_CHECKED_FACES: list = []
_CHECKED_FACES_MAX = 8


def check_face_range(faces, n_verts):
    """Vertex ids must index ``verts``; the kernels trust them (one reduction, one sync -- once
    per face tensor and vertex count while the tensor is not modified in place)."""
    if faces.numel():
        for held, ver, nv in _CHECKED_FACES:
            if held is faces and ver == faces._version and nv == n_verts:
                return
        lo, hi = torch.aminmax(faces)
        if int(lo) < 0 or int(hi) >= n_verts:
            raise ValueError(f"faces reference vertex ids outside [0, {n_verts})")
        _CHECKED_FACES.append((faces, faces._version, int(n_verts)))
        del _CHECKED_FACES[:-_CHECKED_FACES_MAX]


def _rule(p, w, name, dt, dev):
    _lib.check_tensor(p, f"{name} points", dtype=dt, device=dev)
    _lib.check_tensor(w, f"{name} weights", dtype=dt, device=dev)
    if p.numel() != w.numel():
        raise ValueError(f"{name}: points and weights differ in length")
    if not 1 <= p.numel() <= 16:
        raise ValueError(f"{name}: 1..16 Gauss nodes supported (got {p.numel()})")
    return p.numel()


# ---------------------------------------------------------------------------------------
# reference-op drop-ins
# ---------------------------------------------------------------------------------------
def create_MOM_Zmat_3d_forward(verts, faces, face_areas, face_normals, gaussian_points_1d_x,
                               gaussian_weights_1d_x, gaussian_points_1d_y, gaussian_weights_1d_y,
                               face_edge_Zmat_real, face_edge_Zmat_imag, wavenumber):
    """Face-edge CFIE matrix into [B, 3F, 3F] real/imag outputs (mesh_MOM_3d.cu:332-496)."""
    dt, dev, nv, nf = _mesh_args(verts, faces, face_areas, face_normals)
    nx = _rule(gaussian_points_1d_x, gaussian_weights_1d_x, "test rule", dt, dev)
    ny = _rule(gaussian_points_1d_y, gaussian_weights_1d_y, "source rule", dt, dev)
    for t, n in ((face_edge_Zmat_real, "face_edge_Zmat_real"), (face_edge_Zmat_imag, "face_edge_Zmat_imag")):
        _lib.check_tensor(t, n, dtype=dt, device=dev)
        if t.numel() != t.shape[0] * 9 * nf * nf:
            raise ValueError(f"{n} must hold [B, 3F, 3F] entries")
    batch = face_edge_Zmat_real.shape[0]
    _lib.call(f"mb_mom_zmat_fe_{_lib.sfx(dt)}", _lib.ptr(verts), nv, _lib.ptr(faces), nf,
              _lib.ptr(face_areas), _lib.ptr(face_normals), _lib.ptr(gaussian_points_1d_x),
              _lib.ptr(gaussian_weights_1d_x), nx, _lib.ptr(gaussian_points_1d_y),
              _lib.ptr(gaussian_weights_1d_y), ny, float(wavenumber), batch,
              _lib.ptr(face_edge_Zmat_real), _lib.ptr(face_edge_Zmat_imag), _lib.stream_of(verts))


def create_MOM_rhs_3d_forward(verts, faces, face_areas, face_normals, gaussian_points_1d,
                              gaussian_weights_1d, face_edge_rhs_real, face_edge_rhs_imag, wavenumber):
    """Face-edge excitation of the reference's plane wave into [B, F, 3, 1] (mesh_MOM_3d.cu:244-330)."""
    dt, dev, nv, nf = _mesh_args(verts, faces, face_areas, face_normals)
    n = _rule(gaussian_points_1d, gaussian_weights_1d, "rule", dt, dev)
    for t, nm in ((face_edge_rhs_real, "face_edge_rhs_real"), (face_edge_rhs_imag, "face_edge_rhs_imag")):
        _lib.check_tensor(t, nm, dtype=dt, device=dev)
        if t.numel() != t.shape[0] * 3 * nf:
            raise ValueError(f"{nm} must hold [B, F, 3, 1] entries")
    batch = face_edge_rhs_real.shape[0]
    _lib.call(f"mb_mom_rhs_fe_{_lib.sfx(dt)}", _lib.ptr(verts), nv, _lib.ptr(faces), nf,
              _lib.ptr(face_areas), _lib.ptr(face_normals), _lib.ptr(gaussian_points_1d),
              _lib.ptr(gaussian_weights_1d), n, float(wavenumber), batch,
              _lib.ptr(face_edge_rhs_real), _lib.ptr(face_edge_rhs_imag), _lib.stream_of(verts))


def interpolate_Icoeff_to_Js_3d_forward(verts, faces, face_edge_indices, face_areas, edge_I_coeff_real,
                                        edge_I_coeff_imag, face_vert_Js_real, face_vert_Js_imag):
    """Edge coefficients [B, E] -> per-face vertex currents [B, 3F, 3] (+=) (mesh_MOM_3d.cu:498-565)."""
    _lib.check_tensor(verts, "verts", dtype=_FLOATS, ndim=2)
    dt, dev = verts.dtype, verts.device
    _lib.check_tensor(faces, "faces", dtype=torch.int32, device=dev, ndim=2)
    nf = faces.shape[0]
    check_face_range(faces, verts.shape[0])
    _lib.check_tensor(face_edge_indices, "face_edge_indices", dtype=torch.int32, device=dev)
    if face_edge_indices.numel() != 3 * nf:
        raise ValueError("face_edge_indices must have 3F entries")
    _lib.check_tensor(face_areas, "face_areas", dtype=dt, device=dev)
    _lib.check_tensor(edge_I_coeff_real, "edge_I_coeff_real", dtype=dt, device=dev)
    _lib.check_tensor(edge_I_coeff_imag, "edge_I_coeff_imag", dtype=dt, device=dev)
    batch = face_vert_Js_real.shape[0]
    n_edges = edge_I_coeff_imag.shape[1]
    if edge_I_coeff_real.numel() < batch * n_edges:
        raise ValueError("edge coefficients must be [B, E]")
    for t, nm in ((face_vert_Js_real, "face_vert_Js_real"), (face_vert_Js_imag, "face_vert_Js_imag")):
        _lib.check_tensor(t, nm, dtype=dt, device=dev)
        if t.numel() != batch * 9 * nf:
            raise ValueError(f"{nm} must be [B, 3F, 3]")
    if nf:
        fei_max = int(face_edge_indices.max().item())
        if fei_max >= n_edges or int(face_edge_indices.min().item()) < 0:
            raise ValueError("face_edge_indices out of range of the edge coefficients")
    _lib.call(f"mb_mom_interp_js_{_lib.sfx(dt)}", _lib.ptr(verts), verts.shape[0], _lib.ptr(faces), nf,
              _lib.ptr(face_edge_indices), _lib.ptr(face_areas), _lib.ptr(edge_I_coeff_real),
              _lib.ptr(edge_I_coeff_imag), n_edges, batch, _lib.ptr(face_vert_Js_real),
              _lib.ptr(face_vert_Js_imag), _lib.stream_of(verts))


# ---------------------------------------------------------------------------------------
# RWG-space operators
# ---------------------------------------------------------------------------------------
def _check_fei(face_edge_indices, nf, n_edges, dev):
    _lib.check_tensor(face_edge_indices, "face_edge_indices", dtype=torch.int32, device=dev)
    if face_edge_indices.numel() != 3 * nf:
        raise ValueError("face_edge_indices must have 3F entries")
    if nf and (int(face_edge_indices.max().item()) >= n_edges or int(face_edge_indices.min().item()) < 0):
        raise ValueError("face_edge_indices out of range [0, n_edges)")


def assemble_Z_rwg(verts, faces, face_areas, face_normals, face_edge_indices, n_edges,
                   gaussian_points_1d_x, gaussian_weights_1d_x, gaussian_points_1d_y,
                   gaussian_weights_1d_y, wavenumber, out=None, rows=None, check_indices=True,
                   order="auto", edge_rows_map=None, out_host=None, chunks=16):
    """RWG impedance matrix Z [E, E] complex (complex64 for float32 meshes).

    Same entries as ``create_MOM_Zmat_3d_forward`` followed by the reference's
    ``scatter_add_`` onto face_edge_indices (mesh_BEM_solver_3d.py:128-147), in one pass.
    ``out`` (complex [E, E]) is accumulated into if given, else a zeroed matrix is made.
    ``rows`` = (begin, end) restricts the test rows (for chunked assembly): face-edge rows
    with ``order="faces"``, Z rows (edges) with ``order="edges"`` (float32, gaussQR 2-5: each
    Z row built by one block row, its two face contributions summed before one atomic).
    ``order="gather"``: Z rows (edges) in gather form -- each entry's (up to 2 x 2) face-edge
    contributions summed by one thread and stored once, no atomics and no zeroing; rows of
    ``out`` are OVERWRITTEN, not accumulated into (half the DRAM traffic of the edge order, but
    ~3 % slower at 20480 faces: neighbouring threads read scattered source faces).
    ``order="auto"`` (default) takes the edge order when it applies (float32, a fast rule, no
    ``rows``, every edge on at most two faces) and the face order otherwise.
    ``edge_rows_map``: ``edge_rows(face_edge_indices, F, E)`` computed once by the caller.
    ``out_host`` (complex64 [E, E] CPU tensor, pinned for overlap): Z goes to host memory,
    assembled in ``chunks`` Z-row ranges with each range's copy overlapping the next range's
    assembly; ``out`` is then the device scratch (overwritten).  Returns ``out_host`` then.
    """
    dt, dev, nv, nf = _mesh_args(verts, faces, face_areas, face_normals)
    nx = _rule(gaussian_points_1d_x, gaussian_weights_1d_x, "test rule", dt, dev)
    ny = _rule(gaussian_points_1d_y, gaussian_weights_1d_y, "source rule", dt, dev)
    if check_indices:
        _check_fei(face_edge_indices, nf, n_edges, dev)
    cdt = torch.complex64 if dt == torch.float32 else torch.complex128
    if out is None:
        out = torch.zeros((n_edges, n_edges), dtype=cdt, device=dev)
    else:
        _lib.check_tensor(out, "out", dtype=cdt, device=dev, shape=(n_edges, n_edges))
    rules = (_lib.ptr(gaussian_points_1d_x), _lib.ptr(gaussian_weights_1d_x), nx,
             _lib.ptr(gaussian_points_1d_y), _lib.ptr(gaussian_weights_1d_y), ny, float(wavenumber))
    if out_host is not None:
        if dt != torch.float32:
            raise ValueError("out_host needs a float32 mesh")
        if (out_host.device.type != "cpu" or out_host.dtype != torch.complex64 or not out_host.is_contiguous()
                or tuple(out_host.shape) != (n_edges, n_edges)):
            raise ValueError("out_host must be a contiguous complex64 CPU tensor [E, E]")
        er = torch.empty(2 * n_edges + 1, dtype=torch.int32, device=dev)
        _lib.call("mb_mom_zmat_rwg_to_host_c64", _lib.ptr(verts), nv, _lib.ptr(faces), nf,
                  _lib.ptr(face_areas), _lib.ptr(face_normals), _lib.ptr(face_edge_indices), n_edges, *rules,
                  _lib.ptr(er), _lib.ptr(out), out_host.data_ptr(), int(chunks), _lib.stream_of(verts))
        return out_host
    if order == "auto":
        order = "faces"
        if dt == torch.float32 and rows is None and (nx, ny) in _EDGE_RULES:
            try:
                edge_rows_map = edge_rows(face_edge_indices, nf, n_edges) if edge_rows_map is None else edge_rows_map
                order = "edges"
            except ValueError:
                pass
    if order == "gather":
        if dt != torch.float32:
            raise ValueError("order='gather' needs a float32 mesh")
        er = edge_rows(face_edge_indices, nf, n_edges) if edge_rows_map is None else edge_rows_map
        m0, m1 = (0, n_edges) if rows is None else rows
        _lib.call("mb_mom_zmat_rwg_gather_c64", _lib.ptr(verts), nv, _lib.ptr(faces), nf, _lib.ptr(face_areas),
                  _lib.ptr(face_normals), _lib.ptr(er), n_edges, *rules, int(m0), int(m1), _lib.ptr(out),
                  _lib.stream_of(verts))
        return out
    if order == "edges":
        if dt != torch.float32:
            raise ValueError("order='edges' needs a float32 mesh")
        er = edge_rows(face_edge_indices, nf, n_edges) if edge_rows_map is None else edge_rows_map
        m0, m1 = (0, n_edges) if rows is None else rows
        _lib.call("mb_mom_zmat_rwg_edges_c64", _lib.ptr(verts), nv, _lib.ptr(faces), nf, _lib.ptr(face_areas),
                  _lib.ptr(face_normals), _lib.ptr(face_edge_indices), _lib.ptr(er), n_edges, *rules, int(m0),
                  int(m1), _lib.ptr(out), _lib.stream_of(verts))
        return out
    if order != "faces":
        raise ValueError("order must be 'auto', 'faces', 'edges' or 'gather'")
    r0, r1 = (0, 3 * nf) if rows is None else rows
    _lib.call(f"mb_mom_zmat_rwg_{_lib.csfx(dt)}", _lib.ptr(verts), nv, _lib.ptr(faces), nf,
              _lib.ptr(face_areas), _lib.ptr(face_normals), _lib.ptr(face_edge_indices), n_edges, *rules,
              int(r0), int(r1), _lib.ptr(out), _lib.stream_of(verts))
    return out


_EDGE_RULES = {(4, 3), (3, 2), (2, 1), (5, 4)}  # (n_x, n_y) with an edge-row kernel


def edge_rows(face_edge_indices, n_faces: int, n_edges: int) -> torch.Tensor:
    """Z row -> face-edge rows map for ``order='edges'``: int32 [2 E + 1] (see
    ``mb_mom_edge_rows``); raises if some edge has more than two faces."""
    dev = face_edge_indices.device
    er = torch.empty(2 * n_edges + 1, dtype=torch.int32, device=dev)
    _lib.call("mb_mom_edge_rows", _lib.ptr(face_edge_indices), int(n_faces), int(n_edges), _lib.ptr(er),
              _lib.stream_of(face_edge_indices))
    if int(er[-1].item()):
        raise ValueError("an edge has more than two faces: use order='faces'")
    return er


def plane_waves(wavenumber: float, directions, polarizations, eta: float = 1.0,
                device=None) -> torch.Tensor:
    """Pack plane waves for ``assemble_rhs_rwg``: [n, 9] float64 (k*khat, E, khat x E / eta)."""
    d = torch.as_tensor(directions, dtype=torch.float64).reshape(-1, 3)
    e = torch.as_tensor(polarizations, dtype=torch.float64).reshape(-1, 3)
    d = d / d.norm(dim=-1, keepdim=True)
    h = torch.cross(d, e, dim=-1) / eta
    return torch.cat((wavenumber * d, e, h), dim=-1).contiguous().to(device)


def reference_plane_wave(wavenumber: float, device=None) -> torch.Tensor:
    """The reference's hard-coded incidence (mesh_MOM_3d.cu:24-70) in ``plane_waves`` form."""
    az = 30 / 180.0 * math.pi
    hdir = az - 0.5 * math.pi
    w = torch.tensor([[wavenumber * math.cos(az), wavenumber * math.sin(az), 0.0, 0.0, 0.0, 1.0,
                       math.cos(hdir), math.sin(hdir), 0.0]], dtype=torch.float64)
    return w.to(device)


def assemble_rhs_rwg(verts, faces, face_areas, face_normals, face_edge_indices, n_edges,
                     gaussian_points_1d, gaussian_weights_1d, waves, out=None):
    """Excitation vectors [E, n_rhs] complex for the plane waves ``waves`` ([n_rhs, 9] float64)."""
    dt, dev, nv, nf = _mesh_args(verts, faces, face_areas, face_normals)
    n = _rule(gaussian_points_1d, gaussian_weights_1d, "rule", dt, dev)
    _check_fei(face_edge_indices, nf, n_edges, dev)
    waves = waves.to(device=dev, dtype=torch.float64).contiguous()
    _lib.check_tensor(waves, "waves", dtype=torch.float64, device=dev, ndim=2)
    if waves.shape[1] != 9:
        raise ValueError("waves must be [n_rhs, 9]")
    n_rhs = waves.shape[0]
    cdt = torch.complex64 if dt == torch.float32 else torch.complex128
    if out is None:
        out = torch.zeros((n_edges, n_rhs), dtype=cdt, device=dev)
    else:
        _lib.check_tensor(out, "out", dtype=cdt, device=dev, shape=(n_edges, n_rhs))
    _lib.call(f"mb_mom_rhs_rwg_{_lib.csfx(dt)}", _lib.ptr(verts), nv, _lib.ptr(faces), nf,
              _lib.ptr(face_areas), _lib.ptr(face_normals), _lib.ptr(face_edge_indices), n_edges,
              _lib.ptr(gaussian_points_1d), _lib.ptr(gaussian_weights_1d), n, _lib.ptr(waves), n_rhs,
              _lib.ptr(out), _lib.stream_of(verts))
    return out


def interpolate_vert_js(verts, faces, face_edge_indices, face_areas, i_coeff, out=None):
    """Edge coefficients [B, E] complex -> vertex currents [B, V, 3] complex."""
    _lib.check_tensor(verts, "verts", dtype=_FLOATS, ndim=2)
    dt, dev = verts.dtype, verts.device
    _lib.check_tensor(faces, "faces", dtype=torch.int32, device=dev, ndim=2)
    nf, nv = faces.shape[0], verts.shape[0]
    check_face_range(faces, nv)
    cdt = torch.complex64 if dt == torch.float32 else torch.complex128
    i_coeff = i_coeff.reshape(i_coeff.shape[0] if i_coeff.dim() > 1 else 1, -1).to(cdt).contiguous()
    batch, n_edges = i_coeff.shape
    _check_fei(face_edge_indices, nf, n_edges, dev)
    _lib.check_tensor(face_areas, "face_areas", dtype=dt, device=dev)
    if out is None:
        out = torch.zeros((batch, nv, 3), dtype=cdt, device=dev)
    else:
        _lib.check_tensor(out, "out", dtype=cdt, device=dev, shape=(batch, nv, 3))
    _lib.call(f"mb_mom_interp_vert_{_lib.csfx(dt)}", _lib.ptr(verts), nv, _lib.ptr(faces), nf,
              _lib.ptr(face_edge_indices), _lib.ptr(face_areas), _lib.ptr(i_coeff), n_edges, batch,
              _lib.ptr(out), _lib.stream_of(verts))
    return out


# ---------------------------------------------------------------------------------------
# EFIE with the symmetric 7-point rule and singularity extraction (new capability)
# ---------------------------------------------------------------------------------------
def near_pairs(faces) -> torch.Tensor:
    """All ordered face pairs sharing at least one vertex (incl. self), [n, 2] int32, sorted by
    test face (``utils.shared_vertex_pairs``: O(F) memory)."""
    from .utils import shared_vertex_pairs

    return shared_vertex_pairs(faces)


def assemble_Z_rwg_sym(verts, faces, face_edge_indices, n_edges, wavenumber, out=None, pairs=None,
                       faces_range=None, check_indices=True, out_host=None, chunks=16):
    """EFIE RWG matrix [E, E] with the 7-point rule on both triangles.

    Separated pairs run in the mesh dtype; pairs sharing a vertex (``pairs``, default
    ``near_pairs(faces)``, sorted by test face) have the 1/R part integrated in closed form in
    FP64.  ``faces_range`` restricts the separated pairs to test faces [begin, end) (the near
    pairs are then left to the caller).  ``out_host`` (pinned complex64 CPU tensor [E, E],
    float32 meshes): Z goes to host memory with the copy overlapped with the assembly
    (``chunks`` test-face ranges); ``out`` is then the device scratch.  Returns ``out_host``.
    """
    _lib.check_tensor(verts, "verts", dtype=_FLOATS, ndim=2)
    dt, dev = verts.dtype, verts.device
    _lib.check_tensor(faces, "faces", dtype=torch.int32, device=dev, ndim=2)
    nf = faces.shape[0]
    check_face_range(faces, verts.shape[0])
    if check_indices:
        _check_fei(face_edge_indices, nf, n_edges, dev)
    cdt = torch.complex64 if dt == torch.float32 else torch.complex128
    if out is None:
        out = torch.zeros((n_edges, n_edges), dtype=cdt, device=dev)
    else:
        _lib.check_tensor(out, "out", dtype=cdt, device=dev, shape=(n_edges, n_edges))
    st = _lib.stream_of(verts)
    if out_host is not None:
        if dt != torch.float32 or faces_range is not None:
            raise ValueError("out_host needs a float32 mesh and no faces_range")
        if (out_host.device.type != "cpu" or out_host.dtype != torch.complex64 or not out_host.is_contiguous()
                or tuple(out_host.shape) != (n_edges, n_edges) or not out_host.is_pinned()):
            raise ValueError("out_host must be a pinned contiguous complex64 CPU tensor [E, E]")
        if pairs is None:
            pairs = near_pairs(faces)
        _lib.check_tensor(pairs, "pairs", dtype=torch.int32, device=dev, ndim=2)
        _lib.call("mb_mom_sym_zmat_rwg_to_host_c64", _lib.ptr(verts), verts.shape[0], _lib.ptr(faces), nf,
                  _lib.ptr(face_edge_indices), n_edges, float(wavenumber), _lib.ptr(pairs), pairs.shape[0],
                  _lib.ptr(out), out_host.data_ptr(), int(chunks), st)
        return out_host
    f0, f1 = (0, nf) if faces_range is None else faces_range
    _lib.call(f"mb_mom_sym_zmat_rwg_{_lib.csfx(dt)}", _lib.ptr(verts), verts.shape[0], _lib.ptr(faces), nf,
              _lib.ptr(face_edge_indices), n_edges, float(wavenumber), int(f0), int(f1), _lib.ptr(out), st)
    if faces_range is None:
        if pairs is None:
            pairs = near_pairs(faces)
        _lib.check_tensor(pairs, "pairs", dtype=torch.int32, device=dev, ndim=2)
        _lib.call(f"mb_mom_sym_near_{_lib.csfx(dt)}", _lib.ptr(verts), verts.shape[0], _lib.ptr(faces), nf,
                  _lib.ptr(face_edge_indices), n_edges, _lib.ptr(pairs), pairs.shape[0], float(wavenumber),
                  _lib.ptr(out), st)
    return out


def assemble_rhs_rwg_sym(verts, faces, face_edge_indices, n_edges, waves, out=None):
    """EFIE excitation [E, n_rhs] with the 7-point rule for plane waves [n_rhs, 9] float64."""
    _lib.check_tensor(verts, "verts", dtype=_FLOATS, ndim=2)
    dt, dev = verts.dtype, verts.device
    _lib.check_tensor(faces, "faces", dtype=torch.int32, device=dev, ndim=2)
    nf = faces.shape[0]
    check_face_range(faces, verts.shape[0])
    _check_fei(face_edge_indices, nf, n_edges, dev)
    waves = waves.to(device=dev, dtype=torch.float64).contiguous()
    if waves.dim() != 2 or waves.shape[1] != 9:
        raise ValueError("waves must be [n_rhs, 9]")
    cdt = torch.complex64 if dt == torch.float32 else torch.complex128
    if out is None:
        out = torch.zeros((n_edges, waves.shape[0]), dtype=cdt, device=dev)
    else:
        _lib.check_tensor(out, "out", dtype=cdt, device=dev, shape=(n_edges, waves.shape[0]))
    _lib.call(f"mb_mom_sym_rhs_rwg_{_lib.csfx(dt)}", _lib.ptr(verts), verts.shape[0], _lib.ptr(faces), nf,
              _lib.ptr(face_edge_indices), n_edges, _lib.ptr(waves), waves.shape[0], _lib.ptr(out),
              _lib.stream_of(verts))
    return out


# ---------------------------------------------------------------------------------------
# radiated field after the solve (demo/demo_Helmholtz_MOM_3d.py:246-257)
# ---------------------------------------------------------------------------------------
def radiate_H(points, verts, vert_areas, vert_Js, wavenumber, out=None):
    """Scattered H [P, 3] complex at ``points`` [P, 3] from vertex currents ``vert_Js`` [V, 3].

    Equals the reference's ``-(vert_areas * cross(Js, -gradG_y(k, p1=points, p2=verts))).sum(-2)``
    (its helpers' e^{+jkR} phase and 1e-6 singularity mask included), as one fused kernel.
    """
    _lib.check_tensor(verts, "verts", dtype=_FLOATS, ndim=2)
    dt, dev = verts.dtype, verts.device
    cdt = torch.complex64 if dt == torch.float32 else torch.complex128
    pts = points.to(device=dev, dtype=dt).reshape(-1, 3).contiguous()
    va = vert_areas.to(device=dev, dtype=dt).reshape(-1).contiguous()
    js = vert_Js.to(device=dev, dtype=cdt).reshape(-1, 3).contiguous()
    nv = verts.shape[0]
    if va.numel() != nv or js.shape[0] != nv:
        raise ValueError("vert_areas / vert_Js must have one entry per vertex")
    n_pts = pts.shape[0]
    if out is None:
        out = torch.empty((n_pts, 3), dtype=cdt, device=dev)
    else:
        _lib.check_tensor(out, "out", dtype=cdt, device=dev, shape=(n_pts, 3))
    _lib.call(f"mb_radiate_h_{_lib.csfx(dt)}", _lib.ptr(pts), n_pts, _lib.ptr(verts), _lib.ptr(va),
              _lib.ptr(js), nv, float(wavenumber), _lib.ptr(out), _lib.stream_of(verts))
    return out


# ---------------------------------------------------------------------------------------
# dense iterative solve (replaces torch.linalg.solve at mesh_BEM_solver_3d.py:174)
# ---------------------------------------------------------------------------------------
def gmres_workspace_bytes(n: int, restart: int = 50) -> int:
    return int(_lib.load().mb_gmres_workspace_bytes(int(n), int(restart)))


def gmres(Z, b, x0=None, restart: int = 50, max_iters: int = 2000, tol: float = 1e-6,
          workspace=None):
    """Solve Z x = b by GMRES(restart) with FP64 refinement residuals (``mb_gmres_c64``).

    Z: complex64 [n, n] CUDA tensor.  b: [n] or [n, k] (any complex/real dtype; solved in
    complex128).  Returns (x complex128 with b's shape, list of per-column info dicts with
    ``iterations``, ``restarts``, ``rel_residual`` and ``converged``).  ``workspace`` is an
    optional uint8 CUDA tensor of at least ``gmres_workspace_bytes(n, restart)`` bytes.
    """
    _lib.check_tensor(Z, "Z", dtype=torch.complex64, ndim=2)
    n = Z.shape[0]
    if Z.shape[1] != n:
        raise ValueError("Z must be square")
    dev = Z.device
    bb = b.to(device=dev, dtype=torch.complex128)
    single = bb.dim() == 1
    bb = bb.reshape(n, -1)
    if x0 is None:
        xx = torch.zeros_like(bb)
    else:
        xx = x0.to(device=dev, dtype=torch.complex128).reshape(n, -1).clone()
    need = gmres_workspace_bytes(n, restart)
    if workspace is None:
        workspace = torch.empty(need, dtype=torch.uint8, device=dev)
    else:
        _lib.check_tensor(workspace, "workspace", dtype=torch.uint8, device=dev)
        if workspace.numel() < need:
            raise ValueError(f"workspace needs {need} bytes")
    infos = []
    for c in range(bb.shape[1]):
        bc_ = bb[:, c].contiguous()
        xc = xx[:, c].contiguous()
        info = _lib.GmresInfo()
        _lib.call("mb_gmres_c64", _lib.ptr(Z), n, _lib.ptr(bc_), _lib.ptr(xc), int(restart),
                  int(max_iters), float(tol), _lib.ptr(workspace), workspace.numel(),
                  __import__("ctypes").byref(info), _lib.stream_of(Z))
        xx[:, c] = xc
        infos.append({"iterations": info.iterations, "restarts": info.restarts,
                      "rel_residual": info.rel_residual, "converged": info.status == 0})
    return (xx[:, 0] if single else xx), infos


SPAI_WIDTH = 48  # MB_SPAI_WIDTH: columns per row of the near-field preconditioner


class SpaiPreconditioner:
    """Sparse approximate inverse M of an RWG matrix on the mesh's near field (right
    preconditioner of ``pgmres``): ``cols`` int32 [E, SPAI_WIDTH] local column ids (a row
    ends at its first -1), ``vals`` complex64 [E, SPAI_WIDTH], ``status`` the build's status
    word (bit 0: a pattern cut to its cap; bit 1: a rank-deficient least-squares block)."""

    def __init__(self, cols, vals, status):
        self.cols, self.vals, self.status = cols, vals, status

    def apply(self, v):
        """y = M v (complex64 [E])."""
        n = self.cols.shape[0]
        vv = v.to(device=self.cols.device, dtype=torch.complex64).reshape(n).contiguous()
        y = torch.empty_like(vv)
        _lib.call("mb_spai_apply_c64", _lib.ptr(self.cols), _lib.ptr(self.vals), n, _lib.ptr(vv), _lib.ptr(y),
                  _lib.stream_of(vv))
        return y


def spai_preconditioner(Z, verts, faces, face_edge_indices, n_edges, pairs=None, workspace=None):
    """Near-field sparse approximate inverse of the complex64 RWG matrix Z [E, E] of one mesh
    (``mb_spai_build_c64``): column j minimises ||Z[I_j, J_j] m - e_j|| over the edges J_j of
    the faces sharing a vertex with edge j's faces (rows I_j: one ring further).  ``pairs``:
    the mesh's near-pair list (``near_pairs(faces)`` when None)."""
    _lib.check_tensor(Z, "Z", dtype=torch.complex64, ndim=2, shape=(n_edges, n_edges))
    dev = Z.device
    _lib.check_tensor(verts, "verts", dtype=torch.float32, device=dev, ndim=2)
    _lib.check_tensor(faces, "faces", dtype=torch.int32, device=dev, ndim=2)
    _lib.check_tensor(face_edge_indices, "face_edge_indices", dtype=torch.int32, device=dev)
    nf = faces.shape[0]
    if pairs is None:
        pairs = near_pairs(faces)
    _lib.check_tensor(pairs, "pairs", dtype=torch.int32, device=dev, ndim=2)
    desc = torch.tensor([[0, nf, 0, n_edges, 0, n_edges]], dtype=torch.int64, device=dev)
    need = int(_lib.load().mb_spai_workspace_bytes(int(n_edges)))
    if workspace is None:
        workspace = torch.empty(need, dtype=torch.uint8, device=dev)
    elif workspace.numel() < need:
        raise ValueError(f"workspace needs {need} bytes")
    cols = torch.empty((n_edges, SPAI_WIDTH), dtype=torch.int32, device=dev)
    vals = torch.empty((n_edges, SPAI_WIDTH), dtype=torch.complex64, device=dev)
    st = _lib.stream_of(Z)
    _lib.call("mb_spai_build_c64", _lib.ptr(verts), _lib.ptr(faces), _lib.ptr(face_edge_indices), _lib.ptr(desc), 1,
              nf, int(n_edges), _lib.ptr(pairs), pairs.shape[0], _lib.ptr(Z), _lib.ptr(cols), _lib.ptr(vals),
              _lib.ptr(workspace), workspace.numel(), st)
    status = __import__("ctypes").c_int32(0)
    _lib.call("mb_spai_status", _lib.ptr(workspace), int(n_edges), __import__("ctypes").byref(status), st)
    if status.value & 4:
        raise ValueError("face_edge_indices: an edge id out of range, or an edge without faces or with more "
                         "than two")
    return SpaiPreconditioner(cols, vals, int(status.value))


def pgmres_workspace_bytes(n: int, restart: int = 50) -> int:
    return int(_lib.load().mb_pgmres_workspace_bytes(int(n), int(restart)))


def half_copy(Z):
    """Half-precision copy of the complex64 matrix Z for ``pgmres(..., Z_half=...)``
    (``mb_half_copy_c64``): (Zh float16 [n, 2n] = Z / scale interleaved, scale float32 [1] on
    the device = max |Re|, |Im| of Z)."""
    _lib.check_tensor(Z, "Z", dtype=torch.complex64, ndim=2)
    n0, n1 = Z.shape
    Zh = torch.empty((n0, 2 * n1), dtype=torch.float16, device=Z.device)
    scale = torch.empty(1, dtype=torch.float32, device=Z.device)
    _lib.call("mb_half_copy_c64", _lib.ptr(Z), n0 * n1, _lib.ptr(Zh), _lib.ptr(scale), _lib.stream_of(Z))
    return Zh, scale


def pgmres(Z, b, M=None, x0=None, restart: int = 50, max_iters: int = 2000, tol: float = 1e-6,
           use_graph: bool = True, workspace=None, Z_half=None, inner_rtol: float = 3e-3):
    """Solve Z x = b by right-preconditioned GMRES(restart) with the whole restart cycle on the
    device (``mb_pgmres_c64`` / ``mb_pgmres_c128``): FP32 products and a complex64 basis for
    complex64 Z, FP64 for complex128 Z; refinement residual every cycle.  ``M``: a
    ``SpaiPreconditioner`` or None.  ``Z_half``: ``half_copy(Z)`` for complex64 Z -- the
    Arnoldi products then read the half-precision copy and each cycle ends once its residual
    estimate has dropped by ``inner_rtol``.  b: [n] or [n, k].  Returns (x complex128 with b's
    shape, per-column info dicts as ``gmres``)."""
    _lib.check_tensor(Z, "Z", dtype=(torch.complex64, torch.complex128), ndim=2)
    n = Z.shape[0]
    if Z.shape[1] != n:
        raise ValueError("Z must be square")
    dev = Z.device
    bb = b.to(device=dev, dtype=torch.complex128)
    single = bb.dim() == 1
    bb = bb.reshape(n, -1)
    xx = torch.zeros_like(bb) if x0 is None else x0.to(device=dev, dtype=torch.complex128).reshape(n, -1).clone()
    if M is not None and tuple(M.cols.shape) != (n, SPAI_WIDTH):
        raise ValueError("preconditioner size does not match Z")
    need = pgmres_workspace_bytes(n, restart)
    if workspace is None:
        workspace = torch.empty(need, dtype=torch.uint8, device=dev)
    else:
        _lib.check_tensor(workspace, "workspace", dtype=torch.uint8, device=dev)
        if workspace.numel() < need:
            raise ValueError(f"workspace needs {need} bytes")
    c64 = Z.dtype == torch.complex64
    if Z_half is not None:
        if not c64:
            raise ValueError("Z_half applies to a complex64 Z")
        zh, zscale = Z_half
        _lib.check_tensor(zh, "Z_half", dtype=torch.float16, device=dev, shape=(n, 2 * n))
        half_args = (_lib.ptr(zh), _lib.ptr(zscale), float(inner_rtol))
    else:
        half_args = (None, None, 0.0)
    infos = []
    for c in range(bb.shape[1]):
        bc_ = bb[:, c].contiguous()
        xc = xx[:, c].contiguous()
        info = _lib.GmresInfo()
        mp = (_lib.ptr(M.cols if M is not None else None), _lib.ptr(M.vals if M is not None else None))
        if c64:
            _lib.call("mb_pgmres_c64", _lib.ptr(Z), n, *half_args, *mp, _lib.ptr(bc_), _lib.ptr(xc), int(restart),
                      int(max_iters), float(tol), int(bool(use_graph)), _lib.ptr(workspace), workspace.numel(),
                      __import__("ctypes").byref(info), _lib.stream_of(Z))
        else:
            _lib.call("mb_pgmres_c128", _lib.ptr(Z), n, *mp, _lib.ptr(bc_), _lib.ptr(xc), int(restart),
                      int(max_iters), float(tol), int(bool(use_graph)), _lib.ptr(workspace), workspace.numel(),
                      __import__("ctypes").byref(info), _lib.stream_of(Z))
        xx[:, c] = xc
        infos.append({"iterations": info.iterations, "restarts": info.restarts,
                      "rel_residual": info.rel_residual, "converged": info.status == 0})
    return (xx[:, 0] if single else xx), infos


def gmres_real(A, b, x0=None, restart: int = 50, max_iters: int = 2000, tol: float = 1e-6,
               workspace=None):
    """Solve the real system A x = b by GMRES(restart) (``mb_gmres_f32`` / ``mb_gmres_f64``).

    A: float32 (FP32 products) or float64 (FP64 products) [n, n] CUDA tensor; b: [n] or
    [n, k].  Returns (x float64 with b's shape, list of per-column info dicts).  The
    refinement residual b - A x is FP64 in both cases.
    """
    _lib.check_tensor(A, "A", dtype=(torch.float32, torch.float64), ndim=2)
    n = A.shape[0]
    if A.shape[1] != n:
        raise ValueError("A must be square")
    dev = A.device
    bb = b.to(device=dev, dtype=torch.float64)
    single = bb.dim() == 1
    bb = bb.reshape(n, -1)
    xx = torch.zeros_like(bb) if x0 is None else x0.to(device=dev, dtype=torch.float64).reshape(n, -1).clone()
    need = int(_lib.load().mb_gmres_real_workspace_bytes(int(n), int(restart)))
    if workspace is None:
        workspace = torch.empty(need, dtype=torch.uint8, device=dev)
    else:
        _lib.check_tensor(workspace, "workspace", dtype=torch.uint8, device=dev)
        if workspace.numel() < need:
            raise ValueError(f"workspace needs {need} bytes")
    fn = "mb_gmres_f32" if A.dtype == torch.float32 else "mb_gmres_f64"
    infos = []
    for c in range(bb.shape[1]):
        bc_ = bb[:, c].contiguous()
        xc = xx[:, c].contiguous()
        info = _lib.GmresInfo()
        _lib.call(fn, _lib.ptr(A), n, _lib.ptr(bc_), _lib.ptr(xc), int(restart), int(max_iters), float(tol),
                  _lib.ptr(workspace), workspace.numel(), __import__("ctypes").byref(info), _lib.stream_of(A))
        xx[:, c] = xc
        infos.append({"iterations": info.iterations, "restarts": info.restarts,
                      "rel_residual": info.rel_residual, "converged": info.status == 0})
    return (xx[:, 0] if single else xx), infos


def split_tf32(Z):
    """(hi, lo) fp32 [n, 2n] TF32 split of a complex64 [n, n] matrix (``mb_split_tf32``)."""
    _lib.check_tensor(Z, "Z", dtype=torch.complex64, ndim=2)
    n = Z.shape[0]
    if Z.shape[1] != n:
        raise ValueError("Z must be square")
    real = torch.view_as_real(Z).reshape(n, 2 * n)
    hi = torch.empty_like(real)
    lo = torch.empty_like(real)
    _lib.call("mb_split_tf32", _lib.ptr(real), real.numel(), _lib.ptr(hi), _lib.ptr(lo), _lib.stream_of(real))
    return hi, lo


def cgemm_workspace_bytes(n: int, m: int) -> int:
    return int(_lib.load().mb_cgemm_workspace_bytes(int(n), int(m)))


def multi_rhs_matmul(z_split, X, out=None, workspace=None, check: bool = False):
    """Y = Z X for many right-hand sides on the tcgen05 tensor cores (``mb_cgemm_tf32x3``).

    z_split: (hi, lo) from ``split_tf32(Z)``; X: complex64 [n, m]; returns complex64 [n, m].
    Split-TF32 x 3 products with FP32 accumulation (FP32-class accuracy).  ``check`` reads
    the kernel's status word (a synchronisation) and raises if a pipeline wait ran out.
    """
    hi, lo = z_split
    n = hi.shape[0]
    _lib.check_tensor(hi, "z_hi", dtype=torch.float32, ndim=2, shape=(n, 2 * n))
    _lib.check_tensor(lo, "z_lo", dtype=torch.float32, device=hi.device, ndim=2, shape=(n, 2 * n))
    _lib.check_tensor(X, "X", dtype=torch.complex64, device=hi.device, ndim=2)
    if X.shape[0] != n:
        raise ValueError("X must have n rows")
    m = X.shape[1]
    if out is None:
        out = torch.empty((n, m), dtype=torch.complex64, device=hi.device)
    else:
        _lib.check_tensor(out, "out", dtype=torch.complex64, device=hi.device, shape=(n, m))
    need = cgemm_workspace_bytes(n, m)
    if workspace is None:
        workspace = torch.empty(need, dtype=torch.uint8, device=hi.device)
    elif workspace.numel() < need:
        raise ValueError(f"workspace needs {need} bytes")
    _lib.call("mb_cgemm_tf32x3", _lib.ptr(hi), _lib.ptr(lo), n, _lib.ptr(X), m, _lib.ptr(out), _lib.ptr(workspace),
              workspace.numel(), _lib.stream_of(hi))
    if check:
        st = __import__("ctypes").c_int32(0)
        _lib.call("mb_cgemm_status", _lib.ptr(workspace), n, m, __import__("ctypes").byref(st), _lib.stream_of(hi))
        if st.value:
            raise _lib.MeshBEMError(f"multi_rhs_matmul: pipeline wait timed out (status {st.value})")
    return out


def gmres_multi(z_split, B, X0=None, restart: int = 50, max_iters: int = 2000, tol: float = 1e-6,
                workspace=None):
    """Solve Z X = B for all columns of B in lockstep (``mb_gmres_multi_c64``).

    z_split: (hi, lo) from ``split_tf32(Z)``; B: [n, m] (cast to complex128).  Every Arnoldi
    step does one tensor-core product with all m basis vectors.  Returns (X complex128
    [n, m], info dict with ``iterations`` (Arnoldi steps, shared by all columns),
    ``restarts``, ``max_rel_residual`` and ``converged``).
    """
    hi, lo = z_split
    n = hi.shape[0]
    _lib.check_tensor(hi, "z_hi", dtype=torch.float32, ndim=2, shape=(n, 2 * n))
    _lib.check_tensor(lo, "z_lo", dtype=torch.float32, device=hi.device, ndim=2, shape=(n, 2 * n))
    dev = hi.device
    bb = B.to(device=dev, dtype=torch.complex128).reshape(n, -1).contiguous()
    m = bb.shape[1]
    xx = torch.zeros_like(bb) if X0 is None else X0.to(device=dev, dtype=torch.complex128).reshape(n, m).clone()
    need = int(_lib.load().mb_gmres_multi_workspace_bytes(int(n), int(m), int(restart)))
    if workspace is None:
        workspace = torch.empty(need, dtype=torch.uint8, device=dev)
    elif workspace.numel() < need:
        raise ValueError(f"workspace needs {need} bytes")
    info = _lib.GmresInfo()
    _lib.call("mb_gmres_multi_c64", _lib.ptr(hi), _lib.ptr(lo), n, _lib.ptr(bb), _lib.ptr(xx), m, int(restart),
              int(max_iters), float(tol), _lib.ptr(workspace), workspace.numel(), __import__("ctypes").byref(info),
              _lib.stream_of(hi))
    steps = torch.empty(m, dtype=torch.int32, device=bb.device)
    _lib.call("mb_gmres_multi_column_steps", _lib.ptr(workspace), n, m, int(restart), _lib.ptr(steps),
              _lib.stream_of(bb))
    return xx, {"iterations": info.iterations, "restarts": info.restarts, "max_rel_residual": info.rel_residual,
                "converged": info.status == 0, "column_iterations": steps}


def matvec(Z, v):
    """y = Z v (complex64 Z, v cast to complex64) with FP64 row sums -> complex128 [n]."""
    _lib.check_tensor(Z, "Z", dtype=torch.complex64, ndim=2)
    n = Z.shape[0]
    vv = v.to(device=Z.device, dtype=torch.complex64).reshape(n).contiguous()
    y = torch.empty(n, dtype=torch.complex128, device=Z.device)
    _lib.call("mb_matvec_c64", _lib.ptr(Z), _lib.ptr(vv), n, _lib.ptr(y), _lib.stream_of(Z))
    return y


def residual(Z, x, b):
    """r = b - Z x in FP64 (complex64 Z; x, b complex128 [n])."""
    _lib.check_tensor(Z, "Z", dtype=torch.complex64, ndim=2)
    n = Z.shape[0]
    xx = x.to(device=Z.device, dtype=torch.complex128).reshape(n).contiguous()
    bb = b.to(device=Z.device, dtype=torch.complex128).reshape(n).contiguous()
    r = torch.empty(n, dtype=torch.complex128, device=Z.device)
    _lib.call("mb_residual_c128", _lib.ptr(Z), _lib.ptr(xx), _lib.ptr(bb), n, _lib.ptr(r),
              _lib.stream_of(Z))
    return r


# ---------------------------------------------------------------------------------------
# torch.ops registration (TORCH_LIBRARY(mesh_MOM_3d), mesh_MOM_3d.cpp:117-121)
# ---------------------------------------------------------------------------------------
_registered = None


def register_torch_ops():
    """Expose the three reference ops as ``torch.ops.mesh_MOM_3d.*`` (CUDA dispatch key)."""
    global _registered
    if _registered is not None:
        return _registered
    lib = torch.library.Library("mesh_MOM_3d", "DEF")
    lib.define(
        "create_MOM_rhs_3d_forward(Tensor verts, Tensor faces, Tensor face_areas, Tensor face_normals, "
        "Tensor gaussian_points_1d, Tensor gaussian_weights_1d, Tensor(a!) face_edge_rhs_real, "
        "Tensor(b!) face_edge_rhs_imag, float wavenumber) -> ()")
    lib.define(
        "create_MOM_Zmat_3d_forward(Tensor verts, Tensor faces, Tensor face_areas, Tensor face_normals, "
        "Tensor gaussian_points_1d_x, Tensor gaussian_weights_1d_x, Tensor gaussian_points_1d_y, "
        "Tensor gaussian_weights_1d_y, Tensor(a!) face_edge_Zmat_real, Tensor(b!) face_edge_Zmat_imag, "
        "float wavenumber) -> ()")
    lib.define(
        "interpolate_Icoeff_to_Js_3d_forward(Tensor verts, Tensor faces, Tensor face_edge_indices, "
        "Tensor face_areas, Tensor edge_I_coeff_real, Tensor edge_I_coeff_imag, "
        "Tensor(a!) face_vert_Js_real, Tensor(b!) face_vert_Js_imag) -> ()")
    lib.impl("create_MOM_rhs_3d_forward", create_MOM_rhs_3d_forward, "CUDA")
    lib.impl("create_MOM_Zmat_3d_forward", create_MOM_Zmat_3d_forward, "CUDA")
    lib.impl("interpolate_Icoeff_to_Js_3d_forward", interpolate_Icoeff_to_Js_3d_forward, "CUDA")
    _registered = lib
    return lib
