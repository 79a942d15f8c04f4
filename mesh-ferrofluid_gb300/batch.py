"""Many meshes at once: batched assembly and solve of the MoM systems.

The reference handles one mesh per ``MeshBEMSolver3d`` call.  ``MeshBatch`` packs any number
of meshes of uneven size (and wavenumber) into one vertex / face array and runs

* the assembly of every mesh's impedance matrix into one flat block-diagonal array: with
  ``formulation="efie_sym"`` (the 7-point-rule EFIE, pairs sharing a vertex in FP64) one
  launch of the separated-pair kernel and one of the near-pair kernel
  (``mb_mom_sym_zmat_batched_c64``); with ``formulation="cfie_ref"`` (the reference's EFIE +
  MFIE operator and collapsed Gauss rule, gaussQR 4) one launch
  (``mb_mom_ref_zmat_batched_c64``);
* the excitation of ``nc`` plane waves per mesh in one launch (``mb_mom_sym_rhs_batched_c64``)
  into a padded block [max E_i, n_mesh * nc];
* GMRES on every (mesh, wave) column in lockstep with the block-diagonal product
  (``mb_gmres_blockdiag_c64``), each restart cycle replayed from a captured CUDA graph; the
  product's tile shape (1, 2, 4 or 8 rows per warp reading Z directly, or 32 rows per block
  with Z streamed through shared memory by bulk copies) is picked by timing the candidates
  once (``autotune``).

Each Z_i is stored row-major with its row pitch rounded up to even, so every row starts on a
16-byte boundary.

All data live on one CUDA device; there is no CPU path.
"""
from __future__ import annotations

import ctypes
from typing import List, Sequence

import numpy as np
import torch

from . import _lib
from .utils import get_edge_unique, shared_vertex_pairs

_DESC = 6


class MeshBatch:
    """A batch of triangle meshes with their wavenumbers, packed for batched kernels."""

    def __init__(self, meshes: Sequence, wavenumbers: Sequence[float], device=None, formulation: str = "efie_sym",
                 gaussQR: int = 4):
        if len(meshes) != len(wavenumbers) or not meshes:
            raise ValueError("need one wavenumber per mesh and at least one mesh")
        if formulation not in ("efie_sym", "cfie_ref"):
            raise ValueError(f"unknown formulation {formulation!r} (efie_sym or cfie_ref)")
        self.formulation = formulation
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        verts, faces, fei, near = [], [], [], []
        desc = np.zeros((len(meshes), _DESC), np.int64)
        v_off = f_off = z_off = blk = 0
        self.n_edges: List[int] = []
        for i, (v, f) in enumerate(meshes):
            v = torch.as_tensor(np.asarray(v), dtype=torch.float32).to(dev)
            f = torch.as_tensor(np.asarray(f)).to(device=dev, dtype=torch.int32)
            edges, fe, _ = get_edge_unique(v, f)
            ne, nf = int(edges.shape[0]), int(f.shape[0])
            near.append(shared_vertex_pairs(f, v.shape[0]) + f_off)
            verts.append(v)
            faces.append(f + v_off)
            fei.append(fe.reshape(-1, 3).to(torch.int32))
            desc[i] = (f_off, nf, ne, z_off, blk, 0)
            self.n_edges.append(ne)
            v_off += v.shape[0]
            f_off += nf
            z_off += ne * (ne + (ne & 1))  # rows padded to an even pitch (16-byte aligned rows)
            blk += nf * ((nf + 127) // 128)
        self.n_mesh = len(meshes)
        self.verts = torch.cat(verts).contiguous()
        self.faces = torch.cat(faces).contiguous()
        self.fei = torch.cat(fei).contiguous()
        self.near = torch.cat(near).contiguous()
        self.total_faces = f_off
        self.total_blocks = blk
        self.z_size = z_off
        self.n_rows = max(self.n_edges)
        self._desc_np = desc
        if formulation == "cfie_ref":
            from .utils import compute_face_areas, compute_face_normals, \
                get_gaussion_integration_points_and_weights

            self.areas = compute_face_areas(self.verts, self.faces).reshape(-1).contiguous()
            self.normals = compute_face_normals(self.verts, self.faces).contiguous()
            self.gq = gaussQR
            self.gpx, self.gwx = get_gaussion_integration_points_and_weights(gaussQR, device=dev)
            self.gpy, self.gwy = get_gaussion_integration_points_and_weights(gaussQR - 1, device=dev)
            nfs = desc[:, 1]
            per = 3 * nfs * ((3 * nfs + 127) // 128)
            self.ref_boff = torch.tensor(np.concatenate([[0], np.cumsum(per)]).astype(np.int64), device=dev)
        self.ks = torch.tensor(np.asarray(wavenumbers, np.float64), device=dev)
        if not bool(torch.all(self.ks > 0)):
            raise ValueError("wavenumbers must be > 0")
        self.nc = None
        self.desc = None
        self.rows_per_warp = None
        self._goff = {}
        self._descs = {}

    # -- layout --------------------------------------------------------------------------
    def _desc_for(self, nc: int) -> torch.Tensor:
        if nc not in self._descs:
            d = self._desc_np.copy()
            d[:, 5] = np.arange(self.n_mesh) * nc
            self._descs[nc] = torch.tensor(d, device=self.device)
        return self._descs[nc]

    def _set_nc(self, nc: int):
        if self.nc == nc:
            return
        self.desc = self._desc_for(nc)
        self.nc = nc

    def _warp_offsets(self, rows: int):
        if rows not in self._goff:
            per = [(e + rows - 1) // rows for e in self.n_edges]
            off = np.concatenate([[0], np.cumsum(per)]).astype(np.int64)
            self._goff[rows] = torch.tensor(off, device=self.device)
        return self._goff[rows]

    def z_block(self, z_flat: torch.Tensor, i: int) -> torch.Tensor:
        """View of mesh i's impedance matrix [E_i, E_i] in the flat array (row pitch E_i
        rounded up to even)."""
        o, e = int(self._desc_np[i, 3]), self.n_edges[i]
        p = e + (e & 1)
        return z_flat[o:o + e * p].view(e, p)[:, :e]

    def column(self, X: torch.Tensor, i: int, r: int) -> torch.Tensor:
        """Mesh i, right-hand side r of a padded [n_rows, n_mesh * nc] block."""
        return X[: self.n_edges[i], i * self.nc + r]

    # -- kernels -------------------------------------------------------------------------
    def assemble(self, out: torch.Tensor | None = None) -> torch.Tensor:
        """All impedance matrices, flat complex64 [sum E_i^2] (one launch per kernel)."""
        if self.desc is None:
            self._set_nc(1)
        if out is None:
            out = torch.zeros(self.z_size, dtype=torch.complex64, device=self.device)
        else:
            _lib.check_tensor(out, "out", dtype=torch.complex64, device=self.device)
            out.zero_()
        if self.formulation == "cfie_ref":
            cfg = getattr(self, "asm_config", None)
            name = "mb_mom_ref_zmat_batched_persistent_c64" if cfg == ("persistent", None) else \
                "mb_mom_ref_zmat_batched_c64"
            _lib.call(name, _lib.ptr(self.verts), _lib.ptr(self.faces), _lib.ptr(self.areas),
                      _lib.ptr(self.normals), _lib.ptr(self.fei), _lib.ptr(self.desc), _lib.ptr(self.ref_boff),
                      int(self.ref_boff[-1]), _lib.ptr(self.ks), self.n_mesh, _lib.ptr(self.gpx), _lib.ptr(self.gwx),
                      self.gq, _lib.ptr(self.gpy), _lib.ptr(self.gwy), self.gq - 1, _lib.ptr(out),
                      _lib.stream_of(out))
            return out
        cfg = getattr(self, "asm_config", None)
        if cfg is not None and cfg[0] not in ("pair", "grid", "persistent"):
            sched, boff, total = self._asm_schedule(*cfg)
            _lib.call("mb_mom_sym_zmat_batched_rows_c64", _lib.ptr(self.verts), _lib.ptr(self.faces),
                      _lib.ptr(self.fei), _lib.ptr(self.desc), _lib.ptr(self.ks), self.n_mesh, _lib.ptr(sched),
                      _lib.ptr(boff), total, int(cfg[0]), _lib.ptr(self.near), self.near.shape[0], _lib.ptr(out),
                      _lib.stream_of(out))
            return out
        _lib.call("mb_mom_sym_zmat_batched_c64", _lib.ptr(self.verts), _lib.ptr(self.faces), _lib.ptr(self.fei),
                  _lib.ptr(self.desc), _lib.ptr(self.ks), self.n_mesh, self.total_blocks, _lib.ptr(self.near),
                  self.near.shape[0], _lib.ptr(out), _lib.stream_of(out))
        return out

    def _asm_schedule(self, rows: int, order: str):
        """(schedule int32 [n_mesh], block offsets int64 [n_mesh + 1], total blocks) of the rows
        layout: meshes in packing order ("packed") or largest first ("largest")."""
        key = (rows, order)
        if not hasattr(self, "_asm_sched"):
            self._asm_sched = {}
        if key not in self._asm_sched:
            nf = self._desc_np[:, 1]
            idx = np.arange(self.n_mesh) if order == "packed" else np.argsort(-nf, kind="stable")
            per = ((nf[idx] + rows - 1) // rows) * ((nf[idx] + 127) // 128)
            off = np.concatenate([[0], np.cumsum(per)]).astype(np.int64)
            self._asm_sched[key] = (torch.tensor(idx.astype(np.int32), device=self.device),
                                    torch.tensor(off, device=self.device), int(off[-1]))
        return self._asm_sched[key]

    def autotune_assembly(self, out: torch.Tensor | None = None, reps: int = 2):
        """Pick the assembly's tile and block schedule by timing each candidate.  EFIE: the one-
        pair-per-thread kernel, or the rows layout with 8, 16 or 32 test faces per block and the
        meshes' blocks in packing order or largest mesh first.  Reference CFIE: one block per
        (mesh, row, 128-column tile) ("grid", None) or a resident grid taking those tiles from a
        work counter ("persistent", None).  Returns the chosen configuration."""
        if self.desc is None:
            self._set_nc(1)
        if out is None:
            out = torch.zeros(self.z_size, dtype=torch.complex64, device=self.device)
        if self.formulation == "cfie_ref":
            cands = [("grid", None), ("persistent", None)]
        else:
            cands = [("pair", None)] + [(r, o) for r in (8, 16, 32) for o in ("packed", "largest")]
        best, best_t = None, None
        self.asm_times = {}
        for cfg in cands:
            self.asm_config = cfg
            self.assemble(out=out)  # warm-up
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                self.assemble(out=out)
            e1.record()
            torch.cuda.synchronize(self.device)
            t = e0.elapsed_time(e1) / reps
            self.asm_times[cfg] = t
            if best_t is None or t < best_t:
                best, best_t = cfg, t
        self.asm_config = best
        self.asm_ms = best_t
        return best

    def excitation(self, waves: torch.Tensor) -> torch.Tensor:
        """waves [n_mesh, nc, 9] (``mesh_MOM_3d.plane_waves`` records) -> B complex64
        [n_rows, n_mesh * nc], rows beyond E_i zero."""
        waves = waves.to(device=self.device, dtype=torch.float64).contiguous()
        if waves.dim() != 3 or waves.shape[0] != self.n_mesh or waves.shape[2] != 9:
            raise ValueError("waves must be [n_mesh, nc, 9]")
        nc = waves.shape[1]
        self._set_nc(nc)
        B = torch.zeros((self.n_rows, self.n_mesh * nc), dtype=torch.complex64, device=self.device)
        if self.formulation == "cfie_ref":
            _lib.call("mb_mom_ref_rhs_batched_c64", _lib.ptr(self.verts), _lib.ptr(self.faces), _lib.ptr(self.areas),
                      _lib.ptr(self.normals), _lib.ptr(self.fei), _lib.ptr(self.desc), self.n_mesh,
                      self.total_faces, _lib.ptr(self.gpx), _lib.ptr(self.gwx), self.gq, _lib.ptr(waves), nc,
                      self.n_mesh * nc, _lib.ptr(B), _lib.stream_of(B))
            return B
        _lib.call("mb_mom_sym_rhs_batched_c64", _lib.ptr(self.verts), _lib.ptr(self.faces), _lib.ptr(self.fei),
                  _lib.ptr(self.desc), self.n_mesh, self.total_faces, _lib.ptr(waves), nc, self.n_mesh * nc,
                  _lib.ptr(B), _lib.stream_of(B))
        return B

    def matvec(self, z_flat: torch.Tensor, X: torch.Tensor, rows_per_warp: int | None = None,
               out: torch.Tensor | None = None, nc: int | None = None) -> torch.Tensor:
        """Block-diagonal product Y = blockdiag(Z_i) X on the padded layout (complex64); ``nc``
        columns per mesh (default: the excitation's)."""
        rows = rows_per_warp or self.rows_per_warp or 2
        goff = self._warp_offsets(rows)
        nc = nc or self.nc
        if X.shape[1] != self.n_mesh * nc:
            raise ValueError(f"X must have n_mesh * nc = {self.n_mesh * nc} columns")
        if out is None:
            out = torch.zeros_like(X)
        _lib.call("mb_blockdiag_matvec_c64", _lib.ptr(z_flat), _lib.ptr(self._desc_for(nc)), _lib.ptr(goff),
                  self.n_mesh, int(goff[-1]), _lib.ptr(X), X.shape[1], nc, rows, _lib.ptr(out), _lib.stream_of(X))
        return out

    def autotune(self, z_flat: torch.Tensor, candidates=(1, 2, 4, 8, 32), reps: int = 3) -> int:
        """Pick the block-diagonal product's tile (rows per work unit) by timing each candidate."""
        X = torch.randn(self.n_rows, self.n_mesh * self.nc, dtype=torch.complex64, device=self.device)
        Y = torch.zeros_like(X)
        best, best_t = None, None
        for rows in candidates:
            if rows == 8 and self.nc > 4:
                continue
            self.matvec(z_flat, X, rows, out=Y)  # warm-up
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                self.matvec(z_flat, X, rows, out=Y)
            e1.record()
            torch.cuda.synchronize(self.device)
            t = e0.elapsed_time(e1)
            if best_t is None or t < best_t:
                best, best_t = rows, t
        self.rows_per_warp = best
        return best

    def spai(self, z_flat: torch.Tensor, workspace=None):
        """Near-field sparse approximate inverse of every mesh's Z_i in one launch
        (``mb_spai_build_c64`` over the batch): ``mesh_MOM_3d.SpaiPreconditioner`` with rows
        [sum E_i, SPAI_WIDTH] (mesh i's rows start at ``self.edge_offsets[i]``; local columns)."""
        from .mesh_MOM_3d import SPAI_WIDTH, SpaiPreconditioner

        _lib.check_tensor(z_flat, "z_flat", dtype=torch.complex64, device=self.device)
        if not hasattr(self, "edge_offsets"):
            e = np.asarray(self.n_edges, np.int64)
            eoff = np.concatenate([[0], np.cumsum(e)[:-1]]).astype(np.int64)
            d = np.stack([self._desc_np[:, 0], self._desc_np[:, 1], eoff, e, self._desc_np[:, 3], e + (e & 1)], 1)
            self._spai_desc = torch.tensor(np.ascontiguousarray(d), device=self.device)
            self.edge_offsets = torch.tensor(eoff, device=self.device)
            self.total_edges = int(e.sum())
        ne = self.total_edges
        need = int(_lib.load().mb_spai_workspace_bytes(ne))
        if workspace is None or workspace.numel() < need:
            workspace = torch.empty(need, dtype=torch.uint8, device=self.device)
        cols = torch.empty((ne, SPAI_WIDTH), dtype=torch.int32, device=self.device)
        vals = torch.empty((ne, SPAI_WIDTH), dtype=torch.complex64, device=self.device)
        st = _lib.stream_of(z_flat)
        _lib.call("mb_spai_build_c64", _lib.ptr(self.verts), _lib.ptr(self.faces), _lib.ptr(self.fei),
                  _lib.ptr(self._spai_desc), self.n_mesh, self.total_faces, ne, _lib.ptr(self.near),
                  self.near.shape[0], _lib.ptr(z_flat), _lib.ptr(cols), _lib.ptr(vals), _lib.ptr(workspace),
                  workspace.numel(), st)
        status = ctypes.c_int32(0)
        _lib.call("mb_spai_status", _lib.ptr(workspace), ne, ctypes.byref(status), st)
        if status.value & 4:
            raise ValueError("a mesh of the batch has an edge without faces or with more than two")
        return SpaiPreconditioner(cols, vals, int(status.value))

    def augmentation(self, z_flat: torch.Tensor, U: torch.Tensor):
        """The deflation subspace of every mesh for ``solve(aug=...)``: U [n_rows, n_mesh, K]
        (K in {4, 8, 16}) vectors of x-space per mesh (rows beyond E_i are ignored).  Returns
        (Q, Ut, K): C_i = Z_i U_i by block-diagonal products (8 columns per mesh at a time), an
        orthonormal basis Q_i of its range from the FP64 Gram matrix (C_i^H C_i = V_i S_i^2 V_i^H,
        one batched K x K eigensolve; Q_i = C_i V_i S_i^{-1}) and Ut_i = U_i V_i S_i^{-1} --
        complex64 [n_rows, n_mesh K], so that Z_i Ut_i = Q_i.  Directions whose singular value is
        below 1e-6 of the largest are dropped (zero columns)."""
        n_rows, n_mesh, K = U.shape
        if n_rows != self.n_rows or n_mesh != self.n_mesh or K not in (4, 8, 16):
            raise ValueError("U must be [n_rows, n_mesh, K] with K in {4, 8, 16}")
        rows = torch.arange(n_rows, device=self.device)[:, None]
        valid = rows < torch.as_tensor(self.n_edges, device=self.device)[None, :]  # [n_rows, n_mesh]
        U = torch.where(valid[:, :, None], U.to(torch.complex64), torch.zeros((), dtype=torch.complex64,
                                                                              device=self.device))
        parts = []
        for h in range(0, K, 8):
            w = min(8, K - h)
            Uh = U[:, :, h:h + w].contiguous().view(n_rows, n_mesh * w)
            parts.append(self.matvec(z_flat, Uh, nc=w).view(n_rows, n_mesh, w))
        C = torch.cat(parts, 2).permute(1, 0, 2).to(torch.complex128)  # [n_mesh, n_rows, K]
        # C_i^H C_i = V S^2 V^H (a K x K Hermitian eigenproblem per mesh, batched): Q_i = C_i V S^-1,
        # Ut_i = U_i V S^-1, so Z_i Ut_i = Q_i holds by construction whatever the rounding of Q's
        # orthonormality; directions with S^2 below 1e-12 of the largest get zero columns
        lam, V = torch.linalg.eigh(C.mH @ C)
        keep = lam > 1e-12 * lam[:, -1:].clamp_min(1e-300)
        inv = torch.where(keep, lam.clamp_min(1e-300).rsqrt(), torch.zeros_like(lam)).to(torch.complex128)
        VS = V * inv[:, None, :]
        Q = C @ VS
        Ut = U.permute(1, 0, 2).to(torch.complex128) @ VS
        q = Q.permute(1, 0, 2).reshape(n_rows, n_mesh * K).to(torch.complex64).contiguous()
        ut = Ut.permute(1, 0, 2).reshape(n_rows, n_mesh * K).to(torch.complex64).contiguous()
        return q, ut, K

    def solve(self, z_flat: torch.Tensor, B: torch.Tensor, restart: int = 50, max_iters: int = 2000,
              tol: float = 1e-6, use_graph: bool = True, workspace=None, X0: torch.Tensor | None = None, M=None,
              aug=None):
        """Lockstep GMRES on every (mesh, wave) column -> (X complex128 padded, info dict).

        X0: optional initial guess on the padded layout (rows beyond E_i must be zero).
        M: optional near-field preconditioner from ``spai`` (right preconditioning of every
        mesh's system, ``mb_gmres_blockdiag_pc_c64``).
        aug: optional deflation subspace from ``augmentation`` (``mb_gmres_blockdiag_aug_c64``:
        every cycle starts from the residual-minimising combination of the subspace and the
        Arnoldi steps work in its complement)."""
        if self.nc is None:
            raise RuntimeError("call excitation() first")
        rows = self.rows_per_warp or 2
        goff = self._warp_offsets(rows)
        m = self.n_mesh * self.nc
        bb = B.to(torch.complex128).contiguous()
        X = torch.zeros_like(bb) if X0 is None else X0.to(torch.complex128).clone().contiguous()
        need = int(_lib.load().mb_gmres_blockdiag_workspace_bytes(self.n_rows, m, int(restart)))
        if workspace is None:
            workspace = torch.empty(need, dtype=torch.uint8, device=self.device)
        info = _lib.GmresInfo()
        if M is not None and tuple(M.cols.shape) != (self.total_edges, M.cols.shape[1]):
            raise ValueError("preconditioner does not match the batch")
        if aug is not None:
            q, ut, k = aug
            if tuple(q.shape) != (self.n_rows, self.n_mesh * k) or q.shape != ut.shape:
                raise ValueError("augmentation subspace does not match the batch")
            _lib.call("mb_gmres_blockdiag_aug_c64", _lib.ptr(z_flat), _lib.ptr(self.desc), _lib.ptr(goff),
                      self.n_mesh, int(goff[-1]), rows, self.nc, self.n_rows,
                      _lib.ptr(M.cols) if M is not None else None, _lib.ptr(M.vals) if M is not None else None,
                      _lib.ptr(self.edge_offsets) if M is not None else None, _lib.ptr(q),
                      _lib.ptr(ut), int(k), _lib.ptr(bb), _lib.ptr(X), int(restart), int(max_iters), float(tol),
                      1 if use_graph else 0, _lib.ptr(workspace), workspace.numel(), ctypes.byref(info),
                      _lib.stream_of(bb))
        elif M is not None:
            _lib.call("mb_gmres_blockdiag_pc_c64", _lib.ptr(z_flat), _lib.ptr(self.desc), _lib.ptr(goff), self.n_mesh,
                      int(goff[-1]), rows, self.nc, self.n_rows, _lib.ptr(M.cols), _lib.ptr(M.vals),
                      _lib.ptr(self.edge_offsets), _lib.ptr(bb), _lib.ptr(X), int(restart), int(max_iters),
                      float(tol), 1 if use_graph else 0, _lib.ptr(workspace), workspace.numel(), ctypes.byref(info),
                      _lib.stream_of(bb))
        else:
            _lib.call("mb_gmres_blockdiag_c64", _lib.ptr(z_flat), _lib.ptr(self.desc), _lib.ptr(goff), self.n_mesh,
                      int(goff[-1]), rows, self.nc, self.n_rows, _lib.ptr(bb), _lib.ptr(X), int(restart),
                      int(max_iters), float(tol), 1 if use_graph else 0, _lib.ptr(workspace), workspace.numel(),
                      ctypes.byref(info), _lib.stream_of(bb))
        steps = torch.empty(m, dtype=torch.int32, device=self.device)
        _lib.call("mb_gmres_blockdiag_column_steps", _lib.ptr(workspace), self.n_rows, m, int(restart), _lib.ptr(steps),
                  _lib.stream_of(bb))
        return X, {"iterations": info.iterations, "restarts": info.restarts, "max_rel_residual": info.rel_residual,
                   "converged": info.status == 0, "column_iterations": steps}
