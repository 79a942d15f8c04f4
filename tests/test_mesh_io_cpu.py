"""Mesh file round trips (LoadSingleMesh, src/utils/io.py:60-139) and the BEAST writer."""
import numpy as np
import pytest
import torch


@pytest.mark.parametrize("ext", ["obj", "ply", "json"])
def test_round_trip(pkg, tmp_path, ext):
    io = pkg.mesh_io
    v, f = pkg.meshes.ellipsoid(2, seed=2)
    path = str(tmp_path / f"m.{ext}")
    {"obj": io.save_obj, "ply": io.save_ply, "json": io.save_json}[ext](path, v, f)
    vv, ff = io.LoadSingleMesh(path, dtype=torch.float64)
    assert ff.dtype == torch.int32 and vv.dtype == torch.float64
    assert np.array_equal(ff.numpy(), f) and np.array_equal(vv.numpy(), v)


def test_ascii_ply_with_quads_and_obj_slashes(pkg, tmp_path):
    ply = tmp_path / "q.ply"
    ply.write_text("ply\nformat ascii 1.0\ncomment quad\nelement vertex 4\nproperty float x\n"
                   "property float y\nproperty float z\nelement face 1\n"
                   "property list uchar int vertex_indices\nend_header\n"
                   "0 0 0\n1 0 0\n1 1 0\n0 1 0\n4 0 1 2 3\n")
    v, f = pkg.mesh_io.LoadSingleMesh(str(ply))
    assert f.tolist() == [[0, 1, 2], [0, 2, 3]] and v.shape == (4, 3)
    obj = tmp_path / "s.obj"
    obj.write_text("# x\nv 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\nf -3/1/1 -2/1/1 -1/1/1\n")
    v, f = pkg.mesh_io.LoadSingleMesh(str(obj))
    assert f.tolist() == [[0, 1, 2], [0, 1, 2]]


def test_missing_file_raises(pkg):
    with pytest.raises(RuntimeError):
        pkg.mesh_io.LoadSingleMesh("/nonexistent/mesh.obj")


def test_beast_in_writer(pkg, tmp_path):
    v, f = pkg.meshes.icosphere(0)
    path = tmp_path / "m.in"
    pkg.mesh_io.save_beast_in(str(path), v, f)
    lines = path.read_text().strip().split("\n")
    assert lines[0] == "1" and lines[1] == f"{v.shape[0]} {f.shape[0]}"
    rows = np.array([list(map(int, r.split())) for r in lines[2 + v.shape[0]:]])
    assert np.array_equal(rows, f + 1)
