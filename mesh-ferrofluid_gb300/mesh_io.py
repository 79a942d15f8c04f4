"""Triangle-mesh input/output with the reference's interface.

* ``LoadSingleMesh(obj_path, device, dtype) -> [verts [V,3] dtype, faces [F,3] int32]``
  (``src/utils/io.py:60-139``) for ``.obj``, ``.ply`` (ASCII and binary little/big endian)
  and ``.json`` ({"verts", "faces"}).  The reference delegates to pywavefront / open3d /
  trimesh; these are self-contained numpy parsers.  ``.dae`` (COLLADA scenes) is not read.
* ``save_beast_in(filename, verts, faces)`` writes the BEAST ``.in`` surface-mesh format
  (``demo/generate_in_file.py:12-40``): ``1``, ``V F``, vertex rows, 1-based face rows.
* ``save_obj``, ``save_ply`` (binary little endian) and ``save_json`` for round trips.

Polygons with more than three vertices are fan-triangulated; OBJ vertex references may
carry texture/normal indices (``v/vt/vn``) and may be negative (relative), as in the
format.
"""
from __future__ import annotations

import json
import os
from typing import List

import numpy as np
import torch

_PLY_TYPES = {
    "char": "i1", "int8": "i1", "uchar": "u1", "uint8": "u1", "short": "i2", "int16": "i2",
    "ushort": "u2", "uint16": "u2", "int": "i4", "int32": "i4", "uint": "u4", "uint32": "u4",
    "float": "f4", "float32": "f4", "double": "f8", "float64": "f8",
}


def _fan(poly):
    return [(poly[0], poly[i], poly[i + 1]) for i in range(1, len(poly) - 1)]


def _read_obj(path):
    verts, faces = [], []
    with open(path, "r", errors="replace") as fh:
        for line in fh:
            if line.startswith("v "):
                p = line.split()
                verts.append((float(p[1]), float(p[2]), float(p[3])))
            elif line.startswith("f "):
                idx = []
                for tok in line.split()[1:]:
                    i = int(tok.split("/")[0])
                    idx.append(i - 1 if i > 0 else len(verts) + i)
                faces.extend(_fan(idx))
    return np.asarray(verts, np.float64).reshape(-1, 3), np.asarray(faces, np.int64).reshape(-1, 3)


def _read_ply(path):
    with open(path, "rb") as fh:
        if fh.readline().strip() != b"ply":
            raise ValueError(f"{path}: not a PLY file")
        fmt, elements = None, []
        while True:
            line = fh.readline()
            if not line:
                raise ValueError(f"{path}: truncated PLY header")
            tok = line.decode("ascii", "replace").split()
            if not tok or tok[0] in ("comment", "obj_info"):
                continue
            if tok[0] == "format":
                fmt = tok[1]
            elif tok[0] == "element":
                elements.append([tok[1], int(tok[2]), []])
            elif tok[0] == "property":
                if tok[1] == "list":
                    elements[-1][2].append((tok[4], "list", tok[2], tok[3]))
                else:
                    elements[-1][2].append((tok[2], tok[1]))
            elif tok[0] == "end_header":
                break
        verts = faces = None
        if fmt == "ascii":
            rest = fh.read().decode("ascii", "replace").split("\n")
            pos = 0
            for name, count, props in elements:
                rows = [r.split() for r in rest[pos:pos + count]]
                pos += count
                if name == "vertex":
                    names = [p[0] for p in props]
                    ix = [names.index(c) for c in ("x", "y", "z")]
                    verts = np.asarray([[float(r[i]) for i in ix] for r in rows], np.float64)
                elif name == "face":
                    tri = []
                    for r in rows:
                        n = int(r[0])
                        tri.extend(_fan([int(v) for v in r[1:1 + n]]))
                    faces = np.asarray(tri, np.int64)
            return verts.reshape(-1, 3), faces.reshape(-1, 3)
        end = "<" if fmt == "binary_little_endian" else ">"
        if fmt not in ("binary_little_endian", "binary_big_endian"):
            raise ValueError(f"{path}: unsupported PLY format {fmt!r}")
        data = fh.read()
        off = 0
        for name, count, props in elements:
            if all(p[1] != "list" for p in props):
                dt = np.dtype([(p[0], end + _PLY_TYPES[p[1]]) for p in props])
                arr = np.frombuffer(data, dt, count, off)
                off += dt.itemsize * count
                if name == "vertex":
                    verts = np.stack([arr["x"], arr["y"], arr["z"]], -1).astype(np.float64)
            else:
                tri = []
                for _ in range(count):
                    for p in props:
                        if p[1] == "list":
                            ct = np.dtype(end + _PLY_TYPES[p[2]])
                            it = np.dtype(end + _PLY_TYPES[p[3]])
                            n = int(np.frombuffer(data, ct, 1, off)[0])
                            off += ct.itemsize
                            vals = np.frombuffer(data, it, n, off)
                            off += it.itemsize * n
                            if name == "face" and p[0] in ("vertex_indices", "vertex_index"):
                                tri.extend(_fan([int(v) for v in vals]))
                        else:
                            off += np.dtype(_PLY_TYPES[p[1]]).itemsize
                if name == "face":
                    faces = np.asarray(tri, np.int64)
        return verts.reshape(-1, 3), faces.reshape(-1, 3)


def LoadSingleMesh(obj_path: str, device: torch.device = torch.device("cpu"),
                   dtype=torch.float32) -> List[torch.Tensor]:
    """[verts [V, 3] dtype, faces [F, 3] int32] from an .obj / .ply / .json file."""
    if not os.path.exists(obj_path):
        raise RuntimeError(f"Mesh object path :{obj_path} not found, check your DataSet")
    p = str(obj_path)
    if ".obj" in p:
        v, f = _read_obj(p)
    elif ".json" in p:
        with open(p, "r") as fh:
            d = json.load(fh)
        v = np.asarray(d["verts"], np.float64).reshape(-1, 3)
        f = np.asarray(d["faces"], np.int64).reshape(-1, 3)
    elif ".ply" in p:
        v, f = _read_ply(p)
    else:
        raise NotImplementedError(f"unsupported mesh format: {p}")
    return [torch.from_numpy(v).to(device).to(dtype), torch.from_numpy(f).to(device).to(torch.int32)]


def save_beast_in(filename: str, verts, faces) -> None:
    """BEAST ``.in`` surface mesh: "1", "V F", V coordinate rows, F 1-based index rows."""
    verts = np.asarray(verts)
    faces = np.asarray(faces)
    if faces.size and np.min(faces) == 0:
        faces = faces + 1
    with open(filename, "w") as fh:
        fh.write("1\n")
        fh.write(f"{verts.shape[0]} {faces.shape[0]}\n")
        for v in verts:
            fh.write(f"{v[0]} {v[1]} {v[2]}\n")
        for f in faces:
            fh.write(f"{f[0]} {f[1]} {f[2]}\n")


def save_obj(filename: str, verts, faces) -> None:
    verts, faces = np.asarray(verts), np.asarray(faces)
    with open(filename, "w") as fh:
        for v in verts:
            fh.write(f"v {float(v[0])!r} {float(v[1])!r} {float(v[2])!r}\n")
        for f in faces:
            fh.write(f"f {f[0] + 1} {f[1] + 1} {f[2] + 1}\n")


def save_ply(filename: str, verts, faces) -> None:
    """Binary little-endian PLY with float64 vertices and uchar/int face lists."""
    verts = np.asarray(verts, "<f8")
    faces = np.asarray(faces, "<i4")
    hdr = ("ply\nformat binary_little_endian 1.0\n"
           f"element vertex {verts.shape[0]}\nproperty double x\nproperty double y\nproperty double z\n"
           f"element face {faces.shape[0]}\nproperty list uchar int vertex_indices\nend_header\n")
    rec = np.zeros(faces.shape[0], dtype=[("n", "u1"), ("i", "<i4", (3,))])
    rec["n"] = 3
    rec["i"] = faces
    with open(filename, "wb") as fh:
        fh.write(hdr.encode("ascii"))
        fh.write(verts.tobytes())
        fh.write(rec.tobytes())


def save_json(filename: str, verts, faces) -> None:
    with open(filename, "w") as fh:
        json.dump({"verts": np.asarray(verts).tolist(), "faces": np.asarray(faces).tolist()}, fh)
