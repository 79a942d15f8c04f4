"""numpy front end of the CPU oracle (test infrastructure only).

Wraps ``oracle/_build/libmeshbem_oracle.so`` (the C restatement) and, where it was built,
``oracle/_ref/libref_mom.so`` (the reference's own kernel bodies compiled for the host).
Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it.

Every function takes numpy arrays and returns new numpy arrays; ``dtype`` selects the
float64 or float32 build.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build_oracle as _bo

_lib = None
_ref = None

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I = ctypes.c_int
_D = ctypes.c_double


def _load():
    global _lib
    if _lib is None:
        path = _bo.build()
        lib = ctypes.CDLL(path)
        for sfx in ("f64", "f32"):
            getattr(lib, f"orc_mom_zmat_fe_{sfx}").argtypes = [
                _P, _P, _I64, _P, _P, _P, _P, _I, _P, _P, _I, _D, _I64, _I64, _P, _P]
            getattr(lib, f"orc_mom_rhs_fe_{sfx}").argtypes = [
                _P, _P, _I64, _P, _P, _P, _P, _I, _D, _I, _P, _P, _D, _P, _P]
            getattr(lib, f"orc_mom_interp_js_{sfx}").argtypes = [
                _P, _P, _P, _I64, _P, _P, _P, _I64, _I64, _P, _P]
            getattr(lib, f"orc_laplace_panels_{sfx}").argtypes = [
                _P, _P, _I64, _P, _P, _P, _P, _I, _P, _I, _I, _I, _D, _I64, _I64, _P, _P]
            getattr(lib, f"orc_panel_relation_{sfx}").argtypes = [_P, _I64, _P]
            getattr(lib, f"orc_radiate_h_{sfx}").argtypes = [_P, _I64, _P, _P, _P, _P, _I64, _D, _P, _P]
            getattr(lib, f"orc_mom_sym_zmat_rwg_{sfx}").argtypes = [_P, _P, _I64, _P, _I64, _D, _I64, _I64, _P, _P]
            getattr(lib, f"orc_mom_sym_rhs_rwg_{sfx}").argtypes = [_P, _P, _I64, _P, _I64, _P, _I, _P, _P]
            getattr(lib, f"orc_ray_query_{sfx}").argtypes = [_P, _P, _I64, _P, _P, _I64, _I64, _D, _D, _P]
        lib.orc_potential_integrals.argtypes = [_P, _P, _P, _P]
        lib.orc_laplace_sym_f64.argtypes = [_P, _P, _I64, _I, _I, _I64, _I64, _P]
        lib.orc_laplace_colloc_sl_f64.argtypes = [_P, _P, _I64, _P]
        _lib = lib
    return _lib


def ref_lib():
    """The host build of the reference kernels, or None where the checkout is absent."""
    global _ref
    if _ref is None:
        path = _bo.build_ref()
        if path is None:
            return None
        lib = ctypes.CDLL(path)
        lib.ref_zmat_f64.argtypes = [_P, _P, _P, _P, _P, _P, _I, _P, _P, _I, _P, _P, _I, _I, _D]
        lib.ref_zmat_f32.argtypes = [_P, _P, _P, _P, _P, _P, _I, _P, _P, _I, _P, _P, _I, _I, _D]
        lib.ref_rhs_f64.argtypes = [_P, _P, _P, _P, _P, _P, _I, _P, _P, _I, _I, _D]
        lib.ref_interp_f64.argtypes = [_P, _P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I]
        _ref = lib
    return _ref


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _sfx(dtype):
    return "f64" if np.dtype(dtype) == np.float64 else "f32"


def mom_zmat_fe(verts, faces, areas, normals, gpx, gwx, gpy, gwy, k, rows=None, dtype=np.float64):
    """Face-edge CFIE matrix [3F, 3F] complex (rows: optional (begin, end) slice)."""
    lib = _load()
    v, f = _c(verts, dtype), _c(faces, np.int32)
    a, n = _c(np.reshape(areas, -1), dtype), _c(normals, dtype)
    gpx, gwx, gpy, gwy = (_c(t, dtype) for t in (gpx, gwx, gpy, gwy))
    nf = f.shape[0]
    r0, r1 = (0, 3 * nf) if rows is None else rows
    zr = np.zeros((r1 - r0, 3 * nf), dtype)
    zi = np.zeros_like(zr)
    getattr(lib, f"orc_mom_zmat_fe_{_sfx(dtype)}")(
        _ptr(v), _ptr(f), nf, _ptr(a), _ptr(n), _ptr(gpx), _ptr(gwx), gpx.size,
        _ptr(gpy), _ptr(gwy), gpy.size, float(k), r0, r1, _ptr(zr), _ptr(zi))
    return zr + 1j * zi


def mom_rhs_fe(verts, faces, areas, normals, gp, gw, k, khat=None, e0=None, eta=1.0,
               dtype=np.float64):
    """Face-edge excitation [F, 3] complex.  khat/e0 None -> the reference's hard-coded wave."""
    lib = _load()
    v, f = _c(verts, dtype), _c(faces, np.int32)
    a, n = _c(np.reshape(areas, -1), dtype), _c(normals, dtype)
    gp, gw = _c(gp, dtype), _c(gw, dtype)
    nf = f.shape[0]
    rr = np.zeros(3 * nf, dtype)
    ri = np.zeros_like(rr)
    ref = khat is None
    kh = _c([1, 0, 0] if ref else khat, np.float64)
    ee = _c([0, 0, 1] if ref else e0, np.float64)
    getattr(lib, f"orc_mom_rhs_fe_{_sfx(dtype)}")(
        _ptr(v), _ptr(f), nf, _ptr(a), _ptr(n), _ptr(gp), _ptr(gw), gp.size, float(k),
        1 if ref else 0, _ptr(kh), _ptr(ee), float(eta), _ptr(rr), _ptr(ri))
    return (rr + 1j * ri).reshape(nf, 3)


def mom_interp_js(verts, faces, fei, areas, icoeff, dtype=np.float64):
    """Per-face vertex currents [B, 3F, 3] complex from edge coefficients icoeff [B, E]."""
    lib = _load()
    v, f, e = _c(verts, dtype), _c(faces, np.int32), _c(np.reshape(fei, -1), np.int32)
    a = _c(np.reshape(areas, -1), dtype)
    icoeff = np.atleast_2d(icoeff)
    b, ne = icoeff.shape
    ir, ii = _c(icoeff.real, dtype), _c(icoeff.imag, dtype)
    nf = f.shape[0]
    jr = np.zeros((b, 3 * nf, 3), dtype)
    ji = np.zeros_like(jr)
    getattr(lib, f"orc_mom_interp_js_{_sfx(dtype)}")(
        _ptr(v), _ptr(f), _ptr(e), nf, _ptr(a), _ptr(ir), _ptr(ii), ne, b, _ptr(jr), _ptr(ji))
    return jr + 1j * ji


def panel_relation(faces):
    lib = _load()
    f = _c(faces, np.int32)
    nf = f.shape[0]
    rel = np.zeros((nf, nf), np.uint8)
    lib.orc_panel_relation_f64(_ptr(f), nf, _ptr(rel))
    return rel


def laplace_panels(verts, faces, areas, normals, rands, weights, rel, layer, order, kind=0,
                   k=1.0, rows=None, dtype=np.float64):
    """double_integration_on_panels_3d: [F, F, nphi, nphi] (complex when kind=1)."""
    lib = _load()
    v, f = _c(verts, dtype), _c(faces, np.int32)
    a, n = _c(np.reshape(areas, -1), dtype), _c(normals, dtype)
    rd, w = _c(np.reshape(rands, (-1, 2)), dtype), _c(np.reshape(weights, -1), dtype)
    rel = _c(rel, np.uint8)
    nf = f.shape[0]
    r0, r1 = (0, nf) if rows is None else rows
    nphi = 3 if order == 1 else 1
    out_r = np.zeros((r1 - r0, nf, nphi, nphi), dtype)
    out_i = np.zeros_like(out_r) if kind == 1 else None
    getattr(lib, f"orc_laplace_panels_{_sfx(dtype)}")(
        _ptr(v), _ptr(f), nf, _ptr(a), _ptr(n), _ptr(rd), _ptr(w), w.size, _ptr(rel),
        int(layer), int(order), int(kind), float(k), r0, r1, _ptr(out_r), _ptr(out_i))
    return out_r if kind == 0 else out_r + 1j * out_i


def radiate_h(points, verts, vert_areas, vert_js, k, dtype=np.float64):
    """Scattered H [P, 3] complex at points from vertex currents vert_js [V, 3] complex."""
    lib = _load()
    p, v = _c(points, dtype), _c(verts, dtype)
    a = _c(np.reshape(vert_areas, -1), dtype)
    js = np.asarray(vert_js).reshape(-1, 3)
    jr, ji = _c(js.real, dtype), _c(js.imag, dtype)
    hr = np.zeros((p.shape[0], 3), dtype)
    hi = np.zeros_like(hr)
    getattr(lib, f"orc_radiate_h_{_sfx(dtype)}")(_ptr(p), p.shape[0], _ptr(v), _ptr(a), _ptr(jr), _ptr(ji),
                                                 v.shape[0], float(k), _ptr(hr), _ptr(hi))
    return hr + 1j * hi


def potential_integrals(x, tri):
    """Closed-form (int_T 1/R dS, int_T (y - x)/R dS) for point x and triangle tri [3, 3]."""
    lib = _load()
    xx, t = _c(x, np.float64), _c(tri, np.float64)
    i1 = np.zeros(1)
    iv = np.zeros(3)
    lib.orc_potential_integrals(_ptr(xx), _ptr(t), _ptr(i1), _ptr(iv))
    return float(i1[0]), iv


def ray_query(verts, faces, origins, dirs, tmin=0.001, tmax=10000.0):
    """Closest hits [H, W, 4] (face, 0, 0, distance) / (-1, 0, 0, -1) for rays dirs [H, W, 3]."""
    lib = _load()
    v, f = _c(verts, np.float64), _c(faces, np.int32)
    o = _c(np.reshape(origins, (-1, 3)), np.float64)
    h = o.shape[0]
    d = _c(np.reshape(dirs, (h, -1, 3)), np.float64)
    w = d.shape[1]
    out = np.zeros((h, w, 4))
    lib.orc_ray_query_f64(_ptr(v), _ptr(f), f.shape[0], _ptr(o), _ptr(d), h, w, float(tmin), float(tmax),
                          _ptr(out))
    return out


def laplace_sym(verts, faces, layer, order, rows=None):
    """Symmetric-rule Galerkin operator [F, F, nphi, nphi] (double; see orc_laplace_sym_f64)."""
    lib = _load()
    v, f = _c(verts, np.float64), _c(faces, np.int32)
    nf = f.shape[0]
    r0, r1 = (0, nf) if rows is None else rows
    nphi = 3 if order == 1 else 1
    out = np.zeros((r1 - r0, nf, nphi, nphi))
    lib.orc_laplace_sym_f64(_ptr(v), _ptr(f), nf, int(layer), int(order), r0, r1, _ptr(out))
    return out


def laplace_colloc_sl(verts, faces):
    """P0 single-layer collocation matrix [F, F] at face centroids (double)."""
    lib = _load()
    v, f = _c(verts, np.float64), _c(faces, np.int32)
    nf = f.shape[0]
    out = np.zeros((nf, nf))
    lib.orc_laplace_colloc_sl_f64(_ptr(v), _ptr(f), nf, _ptr(out))
    return out


def mom_sym_zmat(verts, faces, fei, n_edges, k, faces_range=None):
    """EFIE RWG matrix [E, E] complex128 with the symmetric 7-point rule + singular extraction."""
    lib = _load()
    v, f, e = _c(verts, np.float64), _c(faces, np.int32), _c(np.reshape(fei, -1), np.int32)
    nf = f.shape[0]
    f0, f1 = (0, nf) if faces_range is None else faces_range
    zr = np.zeros((n_edges, n_edges))
    zi = np.zeros_like(zr)
    lib.orc_mom_sym_zmat_rwg_f64(_ptr(v), _ptr(f), nf, _ptr(e), n_edges, float(k), f0, f1, _ptr(zr), _ptr(zi))
    return zr + 1j * zi


def mom_sym_rhs(verts, faces, fei, n_edges, waves):
    """EFIE excitation [E, n_rhs] complex128 with the symmetric rule; waves [n, 9] float64."""
    lib = _load()
    v, f, e = _c(verts, np.float64), _c(faces, np.int32), _c(np.reshape(fei, -1), np.int32)
    w = _c(np.reshape(waves, (-1, 9)), np.float64)
    nr = w.shape[0]
    rr = np.zeros((n_edges, nr))
    ri = np.zeros_like(rr)
    lib.orc_mom_sym_rhs_rwg_f64(_ptr(v), _ptr(f), f.shape[0], _ptr(e), n_edges, _ptr(w), nr, _ptr(rr), _ptr(ri))
    return rr + 1j * ri


# ---- reference kernels compiled for the host (pinning only) ----------------------------

def ref_zmat_fe(verts, faces, areas, normals, gpx, gwx, gpy, gwy, k, dtype=np.float64):
    lib = ref_lib()
    if lib is None:
        raise RuntimeError("reference checkout not available")
    v, f = _c(verts, dtype), _c(faces, np.int32)
    a, n = _c(np.reshape(areas, -1), dtype), _c(normals, dtype)
    gpx, gwx, gpy, gwy = (_c(t, dtype) for t in (gpx, gwx, gpy, gwy))
    nf = f.shape[0]
    zr = np.zeros((3 * nf, 3 * nf), dtype)
    zi = np.zeros_like(zr)
    fn = lib.ref_zmat_f64 if np.dtype(dtype) == np.float64 else lib.ref_zmat_f32
    fn(_ptr(v), _ptr(f), _ptr(a), _ptr(n), _ptr(gpx), _ptr(gwx), gpx.size, _ptr(gpy), _ptr(gwy),
       gpy.size, _ptr(zr), _ptr(zi), v.shape[0], nf, float(k))
    return zr + 1j * zi


def ref_rhs_fe(verts, faces, areas, normals, gp, gw, k):
    lib = ref_lib()
    v, f = _c(verts, np.float64), _c(faces, np.int32)
    a, n = _c(np.reshape(areas, -1), np.float64), _c(normals, np.float64)
    gp, gw = _c(gp, np.float64), _c(gw, np.float64)
    nf = f.shape[0]
    rr = np.zeros(3 * nf)
    ri = np.zeros(3 * nf)
    lib.ref_rhs_f64(_ptr(v), _ptr(f), _ptr(a), _ptr(n), _ptr(gp), _ptr(gw), gp.size, _ptr(rr),
                    _ptr(ri), v.shape[0], nf, float(k))
    return (rr + 1j * ri).reshape(nf, 3)


def ref_interp_js(verts, faces, fei, areas, icoeff):
    lib = ref_lib()
    v, f, e = _c(verts, np.float64), _c(faces, np.int32), _c(np.reshape(fei, -1), np.int32)
    a = _c(np.reshape(areas, -1), np.float64)
    icoeff = np.atleast_2d(icoeff)
    b, ne = icoeff.shape
    ir, ii = _c(icoeff.real, np.float64), _c(icoeff.imag, np.float64)
    nf = f.shape[0]
    jr = np.zeros((b, 3 * nf, 3))
    ji = np.zeros((b, 3 * nf, 3))
    lib.ref_interp_f64(_ptr(v), _ptr(f), _ptr(e), _ptr(a), _ptr(ir), _ptr(ii), _ptr(jr), _ptr(ji),
                       v.shape[0], nf, ne, b)
    return jr + 1j * ji
