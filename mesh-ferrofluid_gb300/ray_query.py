"""Closest-hit ray queries: drop-in for the reference's ``VulkanRayTracing`` plugin.

The reference builds a Vulkan ray-tracing pipeline (``src/vulkan_ray_tracing/``:
``pybind.cpp:14-28`` exports ``RayQueryApp(vertices, indices, raygen, miss, chit)`` with
``QueryForLOS(txs, rxs)`` and ``QueryForNLOS(rxs, rayDirs)``, ``ray_query_App.hpp:881-1000``;
the shaders are ``raygen.rgen:23-64``, ``closesthit.rchit`` and ``miss.rmiss``) and the
Python helpers ``initialize_vulkan_ray_querier`` / ``GetRayQueryDepthMap`` /
``SampleSkydomRays`` (``src/utils/functions.py:235-268, 770-802, 871-886``).

Here the acceleration structure is a linear BVH built on the GPU and queried by a CUDA
kernel (``csrc/rayquery.cu``) through the C ABI (``mb_ray_bvh_build_f32``,
``mb_ray_query_f32``).  The semantics follow the shaders: rays start at ``origins[row]`` and
run along the normalised ``dirs[row, col]``; geometry is opaque with no culling; a hit needs
``t`` in [0.001, 10000]; each ray returns (face index, 0, 0, distance) or (-1, 0, 0, -1).
Where several faces are hit at the same distance the lower face index is returned (the
hardware traversal leaves that choice open).

The shader-path arguments of ``RayQueryApp`` are accepted and ignored.  Host inputs (lists,
numpy arrays) give a flat float32 numpy array of length ``H * W * 4`` as the plugin's
``std::vector<float>`` does; CUDA tensors stay on the device and give a CUDA tensor.
"""
from __future__ import annotations

import ctypes
import math
from typing import List

import numpy as np
import torch

from . import _lib

T_MIN = 0.001     # raygen.rgen: tMin
T_MAX = 10000.0   # raygen.rgen: tMax


def _as_points(x, device, name):
    """(tensor [N, 3] float32 on device, came_from_host)."""
    if isinstance(x, torch.Tensor):
        host = x.device.type != "cuda"
        t = x.detach().to(device=device, dtype=torch.float32)
    else:
        host = True
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.float32))).to(device)
    if t.numel() % 3:
        raise ValueError(f"{name} must hold 3 floats per point (got {t.numel()} values)")
    return t.reshape(-1, 3).contiguous(), host


class RayQueryApp:
    """GPU closest-hit ray querier over one triangle mesh (``RayQueryApp`` of the plugin)."""

    def __init__(self, vertices, indices, raygenShaderPath: str = "", missShaderPath: str = "",
                 chitShaderPath: str = "", device=None):
        if device is None:
            device = vertices.device if isinstance(vertices, torch.Tensor) and vertices.is_cuda else "cuda"
        self.device = torch.device(device)
        if self.device.type == "cuda" and self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.verts, _ = _as_points(vertices, self.device, "vertices")
        if isinstance(indices, torch.Tensor):
            f = indices.detach().to(device=self.device, dtype=torch.int64)
        else:
            f = torch.from_numpy(np.asarray(indices).astype(np.int64)).to(self.device)
        if f.numel() == 0 or f.numel() % 3:
            raise ValueError("indices must hold 3 vertex ids per triangle and at least one triangle")
        if int(f.min()) < 0 or int(f.max()) >= self.verts.shape[0]:
            raise ValueError(f"indices reference vertex ids outside [0, {self.verts.shape[0]})")
        self.faces = f.to(torch.int32).reshape(-1, 3).contiguous()
        self.n_faces = int(self.faces.shape[0])
        nbytes = int(_lib.load().mb_ray_bvh_bytes(self.n_faces))
        self._bvh = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        if self._bvh.data_ptr() % 256:
            raise _lib.MeshBEMError("BVH buffer is not 256-byte aligned")
        _lib.call("mb_ray_bvh_build_f32", _lib.ptr(self.verts), self.verts.shape[0], _lib.ptr(self.faces),
                  self.n_faces, _lib.ptr(self._bvh), nbytes, _lib.stream_of(self._bvh))

    # -- device API ----------------------------------------------------------------------

    def query(self, origins: torch.Tensor, dirs: torch.Tensor, tmin: float = T_MIN, tmax: float = T_MAX,
              out: torch.Tensor | None = None) -> torch.Tensor:
        """origins [H, 3], dirs [H, W, 3] (float32 CUDA) -> [H, W, 4] float32 on the device."""
        if self._bvh is None:
            raise RuntimeError("RayQueryApp was cleaned up")
        _lib.check_tensor(origins, "origins", dtype=torch.float32, device=self.device, ndim=2, shape=(None, 3))
        _lib.check_tensor(dirs, "dirs", dtype=torch.float32, device=self.device, ndim=3)
        h, w = dirs.shape[0], dirs.shape[1]
        if dirs.shape[2] != 3 or h != origins.shape[0]:
            raise ValueError("dirs must be [H, W, 3] with H = origins.shape[0]")
        if out is None:
            out = torch.empty(h, w, 4, dtype=torch.float32, device=self.device)
        else:
            _lib.check_tensor(out, "out", dtype=torch.float32, device=self.device, shape=(h, w, 4))
        if h and w:
            _lib.call("mb_ray_query_f32", _lib.ptr(self._bvh), self.n_faces, _lib.ptr(origins), _lib.ptr(dirs), h,
                      w, float(tmin), float(tmax), _lib.ptr(out), _lib.stream_of(out))
        return out

    def status(self) -> int:
        """Nonzero if any traversal since the build stopped early (see mb_ray_status)."""
        st = ctypes.c_int32(0)
        _lib.call("mb_ray_status", _lib.ptr(self._bvh), self.n_faces, ctypes.byref(st),
                  _lib.stream_of(self._bvh))
        return int(st.value)

    # -- plugin API ----------------------------------------------------------------------

    def _finish(self, res: torch.Tensor, host: bool):
        flat = res.reshape(-1)
        return flat.cpu().numpy() if host else flat

    def QueryForLOS(self, txs, rxs):
        """Rays from txs[j] towards rxs[j, i] (direction rx - tx, full [tMin, tMax] range)."""
        o, host_o = _as_points(txs, self.device, "txs")
        r, host_r = _as_points(rxs, self.device, "rxs")
        h = o.shape[0]
        if h == 0:
            return self._finish(torch.empty(0, device=self.device), host_o or host_r)
        w = r.shape[0] // h
        d = (r[: h * w].reshape(h, w, 3) - o[:, None, :]).contiguous()
        return self._finish(self.query(o, d), host_o or host_r)

    def QueryForNLOS(self, rxs, rayDirs):
        """Rays from rxs[j] along rayDirs[j, i]."""
        o, host_o = _as_points(rxs, self.device, "rxs")
        d, host_d = _as_points(rayDirs, self.device, "rayDirs")
        h = o.shape[0]
        if h == 0:
            return self._finish(torch.empty(0, device=self.device), host_o or host_d)
        w = d.shape[0] // h
        return self._finish(self.query(o, d[: h * w].reshape(h, w, 3).contiguous()), host_o or host_d)

    def cleanUp(self) -> None:
        self._bvh = None

    def __del__(self):
        self._bvh = None


def initialize_vulkan_ray_querier(verts: torch.Tensor, faces: torch.Tensor) -> RayQueryApp:
    """Builds the querier for one mesh (``src/utils/functions.py:871-886``)."""
    dev = verts.device if verts.is_cuda else None
    return RayQueryApp(verts.reshape(-1, 3).to(torch.float32), faces.reshape(-1, 3), device=dev)


def GetRayQueryDepthMap(vulkan_ray_tracer: RayQueryApp, ray_o: torch.Tensor, ray_d: torch.Tensor,
                        keepdim: bool = True) -> List[torch.Tensor]:
    """Depth and face index per ray (``src/utils/functions.py:770-802``).

    ray_o [B, 3], ray_d [(B), n_rays, 3] -> depth [B, n_rays, (1)] in ray_o's dtype and face
    index [B, n_rays, 1] int32 (-1 / -1 on a miss), on ray_o's device.
    """
    n_rays = ray_d.shape[-2]
    ray_d = ray_d + torch.zeros_like(ray_o).unsqueeze(-2)
    dev = vulkan_ray_tracer.device
    o = ray_o.reshape(-1, 3).to(device=dev, dtype=torch.float32).contiguous()
    d = ray_d.reshape(o.shape[0], n_rays, 3).to(device=dev, dtype=torch.float32).contiguous()
    res = vulkan_ray_tracer.query(o, d).reshape(*ray_o.shape[:-1], n_rays, 4)
    face_idx = res[..., 0:1].to(torch.int32).to(ray_o.device)
    depth = res[..., 3:4].to(ray_o.dtype).to(ray_o.device)
    if not keepdim:
        depth = depth.squeeze(-1)
    return [depth, face_idx]


def SampleSkydomRays(n_rays: int, device=torch.device("cpu"), dtype=torch.float32) -> List:
    """Equirectangular ray directions (``src/utils/functions.py:235-268``).

    n_rays = 2 n_theta^2; returns [dirs [n_rays, 3], thetas, phis, theta_interval,
    phi_interval] with cell-centred angles, theta in (0, pi) rows, phi in (0, 2 pi) columns.
    """
    n_theta = int(math.sqrt(n_rays / 2))
    if 2 * n_theta * n_theta != n_rays:
        raise ValueError("n_rays must be 2 * n_theta^2")
    n_phi = 2 * n_theta
    th = torch.linspace(0, math.pi, n_theta + 1, device=device, dtype=dtype)[:-1]
    th_step = float((th[1] - th[0]).item()) if n_theta > 1 else math.pi
    th = (th + th_step / 2.0)[:, None].repeat(1, n_phi).flatten()
    ph = torch.linspace(0, 2.0 * math.pi, n_phi + 1, device=device, dtype=dtype)[:-1]
    ph_step = float((ph[1] - ph[0]).item())
    ph = (ph + ph_step / 2.0)[None, :].repeat(n_theta, 1).flatten()
    d = torch.stack((torch.sin(th) * torch.cos(ph), torch.sin(th) * torch.sin(ph), torch.cos(th)), -1)
    d = torch.nn.functional.normalize(d, dim=-1)
    return [d, th, ph, th_step, ph_step]
