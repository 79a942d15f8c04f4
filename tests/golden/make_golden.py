"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run where the reference checkout is present (it is read, never written; the environment
variable MESH_FERROFLUID_REF names its root if it is not at the default place):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py

What it does
------------
* Imports the reference package ``src`` (GeCao/Mesh-Ferrofluid) on CPU.  Third-party
  modules the hot path never calls (pytorch3d, kaolin, open3d, soft_renderer, the Vulkan
  plugin, plotting ...) are replaced by inert stand-ins, and
  ``torch.utils.cpp_extension.load`` returns a host stand-in for the ``mesh_MOM_3d``
  extension whose three functions run the reference's own CUDA kernel bodies compiled
  for the host (``oracle/_ref/libref_mom.so``, see oracle/build_oracle.py).
* Runs, in float64:
    - ``get_gaussion_integration_points_and_weights`` for every supported order;
    - ``compute_face_areas/normals``, ``compute_vert_areas``, ``get_edge_unique``,
      ``compute_panel_relation`` on the fixture meshes;
    - ``MeshBEMSolver3d.solve_MOM`` (BEM_type HELMHOLTZ_MOM) -- face-edge Z, face-edge rhs,
      the solved edge coefficients and the vertex currents;
    - ``MeshBEMSolver3d.solve`` (BEM_type LAPLACE, all-Dirichlet, f = x^2 - y^2 as in
      ``demo/demo_Laplace_3d.py:39-55``) -- unpacked V and K, packed V, rhs and solution.
* Saves compressed ``.npz`` files next to this script.
"""
from __future__ import annotations

import importlib
import importlib.abc
import importlib.machinery
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
# the reference checkout (read-only); MESH_FERROFLUID_REF overrides where it lives
REF_ROOT = os.environ.get("MESH_FERROFLUID_REF", "/root/reference")

sys.dont_write_bytecode = True
sys.path.insert(0, REPO)

import torch  # noqa: E402

from oracle import oracle as O  # noqa: E402

meshes = importlib.import_module("mesh-ferrofluid_gb300.meshes")

STUB_ROOTS = {
    "pytorch3d", "kaolin", "open3d", "pymeshlab", "pywavefront", "trimesh", "cv2", "mesh2sdf",
    "tecplot", "matplotlib", "mpl_toolkits", "taichi", "imageio", "PIL", "cmap",
    "soft_renderer", "VulkanRayTracing", "skimage", "scipy_stub_never", "igl", "plyfile",
    "drjit", "mitsuba", "tensorboard", "torch_geometric", "pyvista", "meshio", "gpytoolbox",
    "tqdm_stub_never", "point_cloud_utils", "pyrender", "cebra", "bempp",
}


class _Inert:
    """Accepts any call / attribute access; stands in for unused third-party objects."""

    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Inert()

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Inert()

    def __mro_entries__(self, bases):
        return (object,)


class _StubModule(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Inert()


class _StubFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def find_spec(self, fullname, path, target=None):
        root = fullname.split(".")[0]
        if root in STUB_ROOTS or fullname.startswith("src.vulkan_ray_tracing"):
            return importlib.machinery.ModuleSpec(fullname, self, is_package=True)
        return None

    def create_module(self, spec):
        m = _StubModule(spec.name)
        m.__path__ = []
        return m

    def exec_module(self, module):
        pass


class _HostMOM:
    """Host stand-in for the JIT extension ``mesh_MOM_3d`` (kernel_functions.py:14-23)."""

    @staticmethod
    def create_MOM_Zmat_3d_forward(verts, faces, areas, normals, gpx, gwx, gpy, gwy, zr, zi, k):
        z = O.ref_zmat_fe(verts.numpy(), faces.numpy(), areas.numpy(), normals.numpy(),
                          gpx.numpy(), gwx.numpy(), gpy.numpy(), gwy.numpy(), k)
        zr[0].copy_(torch.from_numpy(z.real))
        zi[0].copy_(torch.from_numpy(z.imag))

    @staticmethod
    def create_MOM_rhs_3d_forward(verts, faces, areas, normals, gp, gw, rr, ri, k):
        r = O.ref_rhs_fe(verts.numpy(), faces.numpy(), areas.numpy(), normals.numpy(),
                         gp.numpy(), gw.numpy(), k)
        rr.view(-1).copy_(torch.from_numpy(r.real.reshape(-1)))
        ri.view(-1).copy_(torch.from_numpy(r.imag.reshape(-1)))

    @staticmethod
    def interpolate_Icoeff_to_Js_3d_forward(verts, faces, fei, areas, ir, ii, jr, ji):
        i = ir.numpy().reshape(ir.shape[0], -1) + 1j * ii.numpy().reshape(ii.shape[0], -1)
        j = O.ref_interp_js(verts.numpy(), faces.numpy(), fei.numpy(), areas.numpy(), i)
        jr.copy_(torch.from_numpy(j.real).reshape(jr.shape))
        ji.copy_(torch.from_numpy(j.imag).reshape(ji.shape))


def import_reference():
    sys.meta_path.insert(0, _StubFinder())
    import torch.utils.cpp_extension as cpp

    cpp.load = lambda *a, **k: _HostMOM()
    sys.path.insert(0, REF_ROOT)
    src = importlib.import_module("src")
    mesh_BEM = importlib.import_module("src.mesh_BEM")
    utils = importlib.import_module("src.utils")
    return src, mesh_BEM, utils


class _QuietLogger:
    def InfoLog(self, *a, **k):
        pass

    WarnLog = InfoLog

    def ErrorLog(self, *a, **k):
        raise RuntimeError(str(a))


def fixture_meshes():
    out = {}
    v, f = meshes.icosphere(0)
    out["ico0"] = (v, f)
    v, f = meshes.icosphere(1)
    out["ico1"] = (v, f)
    v, f = meshes.ellipsoid(1, axes=(1.0, 0.7, 0.5), jitter=0.05, seed=3)
    out["ell1"] = (v, f)
    return out


def main():
    assert os.path.isdir(REF_ROOT), "reference checkout not found"
    _, mesh_BEM, U = import_reference()
    torch.set_default_dtype(torch.float64)
    dt = torch.float64
    logger = _QuietLogger()

    # Gauss tables (BEM_utils.py:360-588)
    gauss = {}
    for n in (1, 2, 3, 4, 5, 6, 7, 8, 12):
        p, w = U.get_gaussion_integration_points_and_weights(n, dtype=dt)
        gauss[f"p{n}"] = p.numpy()
        gauss[f"w{n}"] = w.numpy()
    np.savez_compressed(os.path.join(HERE, "gauss_tables.npz"), **gauss)

    for name, (vn, fn) in fixture_meshes().items():
        verts = torch.from_numpy(vn).to(dt)
        faces = torch.from_numpy(fn.astype(np.int32))
        rec = {"verts": vn, "faces": fn.astype(np.int32)}
        rec["face_areas"] = U.compute_face_areas(vertices=verts, faces=faces, keepdim=True).numpy()
        rec["face_normals"] = U.compute_face_normals(vertices=verts, faces=faces).numpy()
        rec["vert_areas"] = U.compute_vert_areas(vertices=verts, faces=faces, keepdim=True).numpy()
        rec["panel_relations"] = U.compute_panel_relation(faces=faces).numpy()
        edges, fei, adj = U.get_edge_unique(verts=verts, faces=faces)
        rec["edges"], rec["face_edge_indices"], rec["edge_adjacent_faces"] = (
            edges.numpy(), fei.numpy(), adj.numpy())

        # ---- MoM (HELMHOLTZ_MOM), gaussQR = 4 as in the demo default ----
        for gq, k in ((4, 2.0), (3, 4.5)):
            solver = mesh_BEM.MeshBEMSolver3d(
                gaussQR=gq, order_type=1, BEM_type=int(U.BEMType.HELMHOLTZ_MOM), wavenumber=k,
                logger=logger, dtype=dt, device=torch.device("cpu"))
            captured = {}
            orig_z = mesh_BEM.MeshMOMZmatKernel.apply
            orig_r = mesh_BEM.MeshMOMRhsKernel.apply
            orig_j = mesh_BEM.MeshMOMInterpolateJsKernel.apply

            def cap(fn, key):
                def wrapped(*a):
                    out = fn(*a)
                    captured[key] = out.detach().clone()
                    if key == "interp":
                        captured["I_coeff"] = a[-1].detach().clone()
                    return out
                return wrapped

            mod = sys.modules["src.mesh_BEM.mesh_BEM_solver_3d"]
            mod.MeshMOMZmatKernel.apply = cap(orig_z, "zfe")
            mod.MeshMOMRhsKernel.apply = cap(orig_r, "rhsfe")
            mod.MeshMOMInterpolateJsKernel.apply = cap(orig_j, "interp")
            try:
                import contextlib
                import io
                with contextlib.redirect_stdout(io.StringIO()):
                    js = solver.solve_MOM(verts=verts, faces=faces, edges=edges,
                                          face_edge_indices=fei)
            finally:
                mod.MeshMOMZmatKernel.apply = orig_z
                mod.MeshMOMRhsKernel.apply = orig_r
                mod.MeshMOMInterpolateJsKernel.apply = orig_j
            tag = f"mom_gq{gq}"
            rec[f"{tag}_k"] = np.float64(k)
            zfe = captured["zfe"].numpy()[0]
            if name == "ico0":
                rec[f"{tag}_zfe"] = zfe
            else:
                rec[f"{tag}_zfe_rows"] = zfe[:36]
            rec[f"{tag}_zfe_fro"] = np.float64(np.linalg.norm(zfe))
            rec[f"{tag}_rhsfe"] = captured["rhsfe"].numpy()[0, :, :, 0]
            rec[f"{tag}_icoeff"] = captured["I_coeff"].numpy()
            rec[f"{tag}_face_vert_js"] = captured["interp"].numpy()
            rec[f"{tag}_vert_js"] = js.numpy()

        # ---- scattered H radiated from the solved vertex currents (demo_Helmholtz_MOM_3d.py:246-257)
        F = importlib.import_module("src.utils.functions")
        g1 = np.linspace(-2.0, 2.0, 9)
        gx, gz = np.meshgrid(g1, g1, indexing="ij")
        pts = np.stack([gx.ravel(), np.zeros(gx.size), gz.ravel()], -1)
        pts = np.concatenate([pts, vn[0:1], vn[1:2] + np.array([[4e-7, 0.0, 0.0]]),
                              1.5 * vn[2:3]], 0)
        pm = torch.from_numpy(pts).reshape(-1, 1, 3)
        ejs = torch.from_numpy(rec["mom_gq4_vert_js"][0])
        va = torch.from_numpy(rec["vert_areas"])
        kk = float(rec["mom_gq4_k"])
        nm = pm.shape[0]
        h_sc = -(va * torch.cross(ejs[None].repeat(nm, 1, 1),
                                  -F.gradG_y(wavenumber=kk, p1=pm, p2=verts), dim=-1))
        rec["field_points"] = pts
        rec["field_H"] = h_sc.sum(dim=-2).numpy()

        # ---- Laplace all-Dirichlet (demo_Laplace_3d.py), P1 and P0, gaussQR = 2 and 3 ----
        vb = verts.unsqueeze(0)
        f_val = (vb[..., 0] * vb[..., 0] - vb[..., 1] * vb[..., 1]).unsqueeze(-1)
        flags = torch.zeros_like(f_val).to(torch.uint8)
        for gq, order in ((2, 1), (3, 1), (2, 0)):
            solver = mesh_BEM.MeshBEMSolver3d(
                gaussQR=gq, order_type=order, BEM_type=int(U.BEMType.LAPLACE), wavenumber=1.0,
                logger=logger, dtype=dt, device=torch.device("cpu"))
            neu, dirv = solver.solve(verts=verts, faces=faces, vert_bc_Dirichlet=f_val.clone(),
                                     vert_bc_Neumann=torch.zeros_like(f_val),
                                     vert_bc_flags=flags)
            tag = f"lap_gq{gq}_o{order}"
            vun = solver.single_layer.get_Vmat_unpacked().numpy()
            kun = solver.double_layer.get_Kmat_unpacked().numpy()
            if name == "ico0":
                rec[f"{tag}_V_unpacked"] = vun
                rec[f"{tag}_K_unpacked"] = kun
            elif name == "ell1" and gq == 2:
                rec[f"{tag}_V_unpacked_rows"] = vun[:12]
                rec[f"{tag}_K_unpacked_rows"] = kun[:12]
            rec[f"{tag}_V_fro"] = np.float64(np.linalg.norm(vun))
            rec[f"{tag}_K_fro"] = np.float64(np.linalg.norm(kun))
            rec[f"{tag}_V_packed"] = solver.single_layer.get_Vmat_tight(verts=verts, faces=faces).numpy()
            rec[f"{tag}_K_packed"] = solver.double_layer.get_Kmat_tight(verts=verts, faces=faces).numpy()
            rec[f"{tag}_rhs"] = solver.rhs_layer.get_rhs_vec().numpy()
            rec[f"{tag}_neumann"] = neu.numpy()
            rec[f"{tag}_dirichlet"] = dirv.numpy()
            rec[f"{tag}_rands"] = torch.cat((solver.single_layer.r1, solver.single_layer.r2), -1).numpy()
            rec[f"{tag}_weights"] = solver.single_layer.gauss_weights.numpy()
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
        print(name, {k: v.shape for k, v in rec.items() if hasattr(v, "shape")})


if __name__ == "__main__":
    main()
