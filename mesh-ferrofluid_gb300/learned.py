"""Learned GMRES initial guess: a message-passing network on the RWG edge graph.

A capability the reference does not have.  One node per RWG edge; neighbours are the other
edges of its one or two triangles.  Node features (per incidence): edge midpoint, length and
direction, the normals of the adjacent triangles, ka, the incidence direction and
polarisation, the incident phase at the midpoint and the excitation coefficient b_e
(normalised per incidence).  Network: a 32 -> 128 embedding, six layers
h' = relu([h, mean_nbr h] W + b) with hidden width 128, and a 128 -> 2 read-out giving the
edge current J_e (normalised).  The initial guess of a column is the residual-minimising
combination of the real and imaginary parts of the predictions for all incidences of its
mesh (``subspace_guess``: a least-squares fit over a 2 nc-vector learned subspace).
Weights and activations are BF16, every product is accumulated in FP32, master weights and
Adam moments are FP32; forward and backward run on this library's kernels (``mb_gnn_*``).
The prediction is only a GMRES initial guess: GMRES still iterates to the requested
residual, so the guess changes the iteration count, never the accuracy of the result.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List

import numpy as np
import torch

from . import _lib
from .utils import compute_face_normals, get_edge_unique

F_IN = 32
HIDDEN = 128
LAYERS = 6
N_FEATURES = 25


@dataclass
class EdgeGraph:
    nbr: torch.Tensor     # [E, 4] int32, -1 where absent
    mid: torch.Tensor     # [E, 3]
    length: torch.Tensor  # [E]
    tdir: torch.Tensor    # [E, 3] unit edge direction
    n1: torch.Tensor      # [E, 3] normal of the first adjacent face
    n2: torch.Tensor      # [E, 3] normal of the second (= n1 on a boundary edge)
    fei: torch.Tensor     # [F, 3] local edge ids (as the assembly uses them)
    n_edges: int


def edge_graph(verts: torch.Tensor, faces: torch.Tensor) -> EdgeGraph:
    """The RWG edge graph of one mesh (device tensors)."""
    verts = verts.to(torch.float32)
    faces = faces.to(torch.int32)
    edges, fei, adj = get_edge_unique(verts, faces)
    ne = int(edges.shape[0])
    fe3 = fei.reshape(-1, 3).long()
    adj = adj.long()
    nbr = torch.full((ne, 4), -1, dtype=torch.int64, device=verts.device)
    eid = torch.arange(ne, device=verts.device)
    for slot in range(2):
        f = adj[:, slot]
        ok = f >= 0
        fs = fe3[f.clamp_min(0)]  # [E, 3]
        others = fs.masked_fill(fs == eid[:, None], -1)
        # keep the two entries that are not the edge itself
        srt = torch.sort(others, dim=1, descending=True).values[:, :2]
        srt = torch.where(ok[:, None], srt, torch.full_like(srt, -1))
        nbr[:, 2 * slot:2 * slot + 2] = srt
    p0, p1 = verts[edges[:, 0].long()], verts[edges[:, 1].long()]
    d = p1 - p0
    length = d.norm(dim=1)
    fn = compute_face_normals(verts, faces)
    n1 = fn[adj[:, 0].clamp_min(0)]
    n2 = torch.where((adj[:, 1] >= 0)[:, None], fn[adj[:, 1].clamp_min(0)], n1)
    return EdgeGraph(nbr.to(torch.int32).contiguous(), 0.5 * (p0 + p1), length, d / length[:, None], n1, n2,
                     fe3.to(torch.int32), ne)


def node_features(g: EdgeGraph, k: float, khat, pol, b: torch.Tensor) -> torch.Tensor:
    """[E, 32] bf16 features of one incidence (khat, pol: 3-vectors; b: [E] complex)."""
    dev = g.mid.device
    khat = torch.as_tensor(khat, dtype=torch.float32, device=dev).reshape(1, 3)
    pol = torch.as_tensor(pol, dtype=torch.float32, device=dev).reshape(1, 3)
    ph = k * (g.mid * khat).sum(1, keepdim=True)
    bs = b.to(torch.complex64)
    bs = bs / bs.abs().pow(2).mean().sqrt().clamp_min(1e-30)
    E = g.n_edges
    cols = [g.mid, g.length[:, None] / g.length.mean(), g.tdir, g.n1, g.n2,
            torch.full((E, 1), k / 8.0, device=dev), khat.expand(E, 3), pol.expand(E, 3),
            torch.cos(ph), torch.sin(ph), bs.real[:, None], bs.imag[:, None],
            (g.tdir * pol).sum(1, keepdim=True)]
    x = torch.cat(cols, 1)
    assert x.shape[1] == N_FEATURES
    out = torch.zeros((E, F_IN), dtype=torch.bfloat16, device=dev)
    out[:, :N_FEATURES] = x.to(torch.bfloat16)
    return out


@dataclass
class BatchGraph:
    """The edge graphs of a batch of meshes back to back (edge ids local to each mesh)."""
    nbr: torch.Tensor       # [S, 4] int32, local ids, -1 where absent
    mid: torch.Tensor       # [S, 3]
    length_n: torch.Tensor  # [S] edge length / the mesh's mean edge length
    tdir: torch.Tensor      # [S, 3]
    n1: torch.Tensor        # [S, 3]
    n2: torch.Tensor        # [S, 3]
    start: torch.Tensor     # [n_mesh + 1] int64, first edge of each mesh
    n_edges: List[int]


def batch_graph(graphs) -> BatchGraph:
    """Concatenate the edge graphs of a batch's meshes (in the batch's mesh order)."""
    graphs = list(graphs)
    dev = graphs[0].mid.device
    ne = [g.n_edges for g in graphs]
    start = torch.tensor(np.concatenate([[0], np.cumsum(ne)]).astype(np.int64), device=dev)
    return BatchGraph(torch.cat([g.nbr for g in graphs]).contiguous(), torch.cat([g.mid for g in graphs]),
                      torch.cat([g.length / g.length.mean() for g in graphs]), torch.cat([g.tdir for g in graphs]),
                      torch.cat([g.n1 for g in graphs]), torch.cat([g.n2 for g in graphs]), start, ne)


def batch_node_features(bg: BatchGraph, ks, khat, pol, B: torch.Tensor, nc: int):
    """The features of ``node_features`` for every (mesh, incidence) column of a batch's
    excitation block B [n_rows, n_mesh * nc] in one pass.  ks [n_mesh]; khat, pol
    [n_mesh, nc, 3].  Nodes run mesh by mesh, incidence by incidence, edge by edge.
    Returns (x0 [N, 32] bf16, nbr [N, 4] int32 node ids, flat [N] int64 positions in B)."""
    dev = bg.mid.device
    n_mesh = len(bg.n_edges)
    E = torch.tensor(bg.n_edges, dtype=torch.int64, device=dev)
    blk = E * nc
    bstart = torch.cat([torch.zeros(1, dtype=torch.int64, device=dev), torch.cumsum(blk, 0)])
    n = int(bstart[-1])
    node = torch.arange(n, device=dev)
    mesh = torch.repeat_interleave(torch.arange(n_mesh, device=dev), blk)
    t = node - bstart[mesh]
    em = E[mesh]
    r = t // em
    e = t - r * em
    g = bg.start[mesh] + e
    col = mesh * nc + r
    flat = e * B.shape[1] + col
    b = B.reshape(-1)[flat].to(torch.complex64)
    sq = torch.zeros(n_mesh * nc, dtype=torch.float32, device=dev).index_add_(0, col, b.abs() ** 2)
    rms = (sq / E.repeat_interleave(nc).to(torch.float32)).sqrt().clamp_min(1e-30)
    bs = b / rms[col]
    kt = torch.as_tensor(np.asarray(ks, np.float32), device=dev)[mesh]
    kh = torch.as_tensor(np.asarray(khat, np.float32), device=dev).reshape(-1, 3)[col]
    po = torch.as_tensor(np.asarray(pol, np.float32), device=dev).reshape(-1, 3)[col]
    mid, tdir = bg.mid[g], bg.tdir[g]
    ph = kt * (mid * kh).sum(1)
    x = torch.cat([mid, bg.length_n[g][:, None], tdir, bg.n1[g], bg.n2[g], (kt / 8.0)[:, None], kh, po,
                   torch.cos(ph)[:, None], torch.sin(ph)[:, None], bs.real[:, None], bs.imag[:, None],
                   (tdir * po).sum(1, keepdim=True)], 1)
    out = torch.zeros((n, F_IN), dtype=torch.bfloat16, device=dev)
    out[:, :N_FEATURES] = x.to(torch.bfloat16)
    nl = bg.nbr[g].long()
    base = bstart[mesh] + r * em
    nbr = torch.where(nl >= 0, base[:, None] + nl, torch.full_like(nl, -1)).to(torch.int32).contiguous()
    return out, nbr, flat


def subspace_guess(bt, Z: torch.Tensor, B: torch.Tensor, pred: torch.Tensor, flat: torch.Tensor, nc: int,
                   reg: float = 1e-8) -> torch.Tensor:
    """Initial guess of every column of a MeshBatch: the combination of the real and imaginary
    parts of the network's predictions for all nc incidences of the same mesh (2 nc vectors)
    that minimises that column's residual |Z x - b| -- a least-squares fit over a small learned
    subspace (one block-diagonal product with 2 nc columns per mesh, then a 2 nc x 2 nc normal
    system per mesh in FP64).  Returns X0 [n_rows, n_mesh * nc] complex128, rows beyond E_i 0."""
    n_rows, m = B.shape
    n_mesh = bt.n_mesh
    P = torch.zeros((n_rows, m), dtype=torch.complex64, device=B.device)
    P.view(-1)[flat] = pred.to(torch.complex64)
    P3 = P.view(n_rows, n_mesh, nc)
    W = torch.cat([P3.real, P3.imag], 2).to(torch.complex64).contiguous()  # [n_rows, n_mesh, 2 nc]
    ZW = bt.matvec(Z, W.view(n_rows, n_mesh * 2 * nc), nc=2 * nc).view(n_rows, n_mesh, 2 * nc)
    A = ZW.permute(1, 0, 2).to(torch.complex128)
    Bm = B.view(n_rows, n_mesh, nc).permute(1, 0, 2).to(torch.complex128)
    G = A.mH @ A
    R = A.mH @ Bm
    lam = reg * G.diagonal(dim1=1, dim2=2).real.sum(-1) / (2 * nc) + 1e-300
    G = G + lam[:, None, None] * torch.eye(2 * nc, dtype=G.dtype, device=G.device)
    alpha = torch.linalg.solve(G, R)  # [n_mesh, 2 nc, nc]
    X0 = W.permute(1, 0, 2).to(torch.complex128) @ alpha
    return X0.permute(1, 0, 2).reshape(n_rows, m).contiguous()


class EdgeGNN:
    """The network's parameters and its forward / backward / Adam steps on the GPU kernels."""

    def __init__(self, device, seed: int = 0):
        gen = torch.Generator(device="cpu").manual_seed(seed)
        shapes = [(F_IN, HIDDEN)] + [(2 * HIDDEN, HIDDEN)] * LAYERS + [(HIDDEN, 2)]
        self.w, self.b, self.w16, self.m, self.v = [], [], [], [], []
        for fan_in, fan_out in shapes:
            w = torch.randn(fan_in, fan_out, generator=gen) * math.sqrt(2.0 / fan_in)
            self.w.append(w.to(device).contiguous())
            self.b.append(torch.zeros(fan_out, device=device))
        self.w[-1] *= 0.1
        self.w16 = [w.to(torch.bfloat16).contiguous() for w in self.w]
        self.m = [torch.zeros_like(t) for t in self.w + self.b]
        self.v = [torch.zeros_like(t) for t in self.w + self.b]
        self.steps = 0
        self.device = device

    # -- kernels -------------------------------------------------------------------------
    def _gemm(self, x, w, bias, relu, out, trans_w=False):
        n, k = x.shape
        m = w.shape[0] if trans_w else w.shape[1]
        _lib.call("mb_gnn_gemm", _lib.ptr(x), int(x.dtype == torch.bfloat16), _lib.ptr(w),
                  int(w.dtype == torch.bfloat16), int(trans_w), _lib.ptr(bias), n, k, m, int(relu), _lib.ptr(out),
                  int(out.dtype == torch.bfloat16), _lib.stream_of(x))
        return out

    def forward(self, x0: torch.Tensor, nbr: torch.Tensor):
        """x0 [N, 32] bf16, nbr [N, 4] int32 -> (out [N, 2] fp32, cache)."""
        n = x0.shape[0]
        dev = x0.device
        hs, cats = [], []
        h = self._gemm(x0, self.w16[0], self.b[0], True,
                       torch.empty((n, HIDDEN), dtype=torch.bfloat16, device=dev))
        hs.append(h)
        for layer in range(1, LAYERS + 1):
            cat = torch.empty((n, 2 * HIDDEN), dtype=torch.bfloat16, device=dev)
            _lib.call("mb_gnn_aggregate", _lib.ptr(h), _lib.ptr(nbr), n, HIDDEN, _lib.ptr(cat), _lib.stream_of(h))
            cats.append(cat)
            h = self._gemm(cat, self.w16[layer], self.b[layer], True,
                           torch.empty((n, HIDDEN), dtype=torch.bfloat16, device=dev))
            hs.append(h)
        out = self._gemm(h, self.w16[-1], self.b[-1], False, torch.empty((n, 2), dtype=torch.float32, device=dev))
        return out, (x0, nbr, hs, cats)

    def backward(self, cache, dout: torch.Tensor):
        """Gradients (list over weights then biases, FP32) of sum(dout * out)."""
        x0, nbr, hs, cats = cache
        n = x0.shape[0]
        s = _lib.stream_of(dout)
        gw = [torch.zeros_like(w) for w in self.w]
        gb = [torch.zeros_like(b) for b in self.b]

        def tn(x, dy, dw):
            _lib.call("mb_gnn_gemm_tn", _lib.ptr(x), int(x.dtype == torch.bfloat16), _lib.ptr(dy), n, x.shape[1],
                      dy.shape[1], _lib.ptr(dw), s)

        def colsum(dy, db):
            _lib.call("mb_gnn_colsum", _lib.ptr(dy), n, dy.shape[1], _lib.ptr(db), s)

        dout = dout.contiguous()
        tn(hs[-1], dout, gw[-1])
        colsum(dout, gb[-1])
        dh = self._gemm(dout, self.w16[-1], None, False, torch.empty((n, HIDDEN), device=dout.device), trans_w=True)
        for layer in range(LAYERS, 0, -1):
            dz = torch.empty_like(dh)
            _lib.call("mb_gnn_relu_bwd", _lib.ptr(hs[layer]), _lib.ptr(dh), dh.numel(), _lib.ptr(dz), s)
            tn(cats[layer - 1], dz, gw[layer])
            colsum(dz, gb[layer])
            dcat = self._gemm(dz, self.w16[layer], None, False, torch.empty((n, 2 * HIDDEN), device=dz.device),
                              trans_w=True)
            dh = torch.zeros((n, HIDDEN), device=dz.device)
            _lib.call("mb_gnn_aggregate_bwd", _lib.ptr(dcat), _lib.ptr(nbr), n, HIDDEN, _lib.ptr(dh), s)
        dz = torch.empty_like(dh)
        _lib.call("mb_gnn_relu_bwd", _lib.ptr(hs[0]), _lib.ptr(dh), dh.numel(), _lib.ptr(dz), s)
        tn(x0, dz, gw[0])
        colsum(dz, gb[0])
        return gw + gb

    def adam(self, grads, lr: float = 1e-3, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8):
        self.steps += 1
        params = self.w + self.b
        for i, (p, g) in enumerate(zip(params, grads)):
            w16 = self.w16[i] if i < len(self.w) else None
            _lib.call("mb_gnn_adam", _lib.ptr(p), _lib.ptr(self.m[i]), _lib.ptr(self.v[i]), _lib.ptr(g), p.numel(),
                      float(lr), float(beta1), float(beta2), float(eps), self.steps, _lib.ptr(w16), _lib.stream_of(p))

    def predict(self, x0: torch.Tensor, nbr: torch.Tensor) -> torch.Tensor:
        out, _ = self.forward(x0, nbr)
        return torch.complex(out[:, 0], out[:, 1])


def fit_scale(matvec, x: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """alpha x with alpha = (Z x)^H b / |Z x|^2 (the best multiple of x in the residual norm)."""
    zx = matvec(x)
    den = (zx.abs() ** 2).sum()
    if den <= 0:
        return torch.zeros_like(x)
    return x * ((zx.conj() * b).sum() / den)


@dataclass
class Samples:
    x0: torch.Tensor      # [N, 32] bf16, all samples back to back
    nbr: torch.Tensor     # [N, 4] int32 local to each sample (offsets added per batch)
    target: torch.Tensor  # [N, 2] fp32, J normalised per sample
    starts: List[int]     # first node of each sample (plus the end)


def build_samples(items) -> Samples:
    """items: iterable of (EdgeGraph, x0 [E, 32], J [E] complex)."""
    xs, nbrs, ts, starts = [], [], [], [0]
    for g, x0, j in items:
        jn = j.to(torch.complex64)
        jn = jn / jn.abs().pow(2).mean().sqrt().clamp_min(1e-30)
        xs.append(x0)
        nbrs.append(g.nbr)
        ts.append(torch.stack([jn.real, jn.imag], 1).float())
        starts.append(starts[-1] + g.n_edges)
    return Samples(torch.cat(xs).contiguous(), torch.cat(nbrs).contiguous(), torch.cat(ts).contiguous(), starts)


def batch_slice(samples: Samples, i0: int, i1: int):
    a, b = samples.starts[i0], samples.starts[i1]
    nbr = samples.nbr[a:b].clone()
    # node ids are local to each sample: shift by the sample's first node inside the batch
    starts = torch.tensor(samples.starts[i0:i1 + 1], device=nbr.device) - a
    lens = starts[1:] - starts[:-1]
    shift = torch.repeat_interleave(starts[:-1], lens)[:, None]
    nbr = torch.where(nbr >= 0, nbr + shift.to(nbr.dtype), nbr).to(torch.int32).contiguous()
    return samples.x0[a:b].contiguous(), nbr, samples.target[a:b].contiguous()


def train(net: EdgeGNN, samples: Samples, epochs: int = 8, batch: int = 32, lr: float = 1e-3, seed: int = 0,
          log=None):
    """Mini-batch Adam on the relative squared error; returns the per-epoch mean losses."""
    rng = np.random.default_rng(seed)
    n_s = len(samples.starts) - 1
    blocks = list(range(0, n_s, batch))
    losses = []
    for ep in range(epochs):
        rng.shuffle(blocks)
        tot, cnt = 0.0, 0
        for i0 in blocks:
            i1 = min(i0 + batch, n_s)
            x0, nbr, t = batch_slice(samples, i0, i1)
            out, cache = net.forward(x0, nbr)
            diff = out - t
            n = out.shape[0]
            loss = float((diff * diff).sum()) / n
            grads = net.backward(cache, (2.0 / n) * diff)
            scale = lr * (0.5 * (1 + math.cos(math.pi * ep / max(1, epochs))))
            net.adam(grads, lr=max(scale, lr * 0.05))
            tot += loss
            cnt += 1
        losses.append(tot / max(cnt, 1))
        if log:
            log(f"epoch {ep}: loss {losses[-1]:.4f}")
    return losses
